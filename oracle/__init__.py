"""ORACLE / TEST INFRASTRUCTURE ONLY: CPU checkers for the ORB front-end path.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package.  The product (orb_slam2_detailed_comments_gb300) never does.
"""
