"""The C++ adapter (orb_slam2_detailed_comments_gb300/adapter/) compiled
against the reference's own headers (include/ORBextractor.h:93-162,
include/ORBmatcher.h, include/Frame.h) and the cv stand-in, linked with
liborbgpu.so.  Without a GPU the test checks the build, the record layout
and that constructing an ORBextractor fails loudly (the library's error as
an exception, no fallback).  With a GPU it also runs two monocular Frames
through the adapter and SearchForInitialization and compares the counts with
the oracle.  Needs the reference tree (skipped where it is not mounted)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(ROOT, "orb_slam2_detailed_comments_gb300", "adapter")


@pytest.fixture(scope="module")
def adapter_bin():
    if subprocess.run(["make", "-s", "-C", ADAPTER, "has-ref"], capture_output=True).returncode != 0:
        pytest.skip("reference headers not mounted")
    from orb_slam2_detailed_comments_gb300 import build
    build.build(table=False)
    r = subprocess.run(["make", "-s", "-C", ADAPTER, "check"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return os.path.join(ADAPTER, "_build", "adapter_check")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_adapter_builds_and_layout(adapter_bin):
    out = subprocess.run([adapter_bin, "layout"], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["keypoint", "28", "28", "point2f", "8"]


def test_adapter_fails_loudly_without_device(adapter_bin):
    if _has_gpu():
        pytest.skip("a device is present")
    r = subprocess.run([adapter_bin, "nodevice"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("threw 3:"), r.stdout


def test_adapter_frames_match_oracle(adapter_bin, tmp_path, oracle):
    if not _has_gpu():
        pytest.skip("no CUDA device")
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    f1, f2, _ = syn.frame_pair(640, 480, seed=0)
    a, b = tmp_path / "a.raw", tmp_path / "b.raw"
    a.write_bytes(f1.tobytes())
    b.write_bytes(f2.tobytes())
    r = subprocess.run([adapter_bin, "run", "640", "480", str(a), str(b)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    _, n1, n2, _, nm = r.stdout.split()
    e1, e2 = oracle.extract(f1, nfeatures=1000), oracle.extract(f2, nfeatures=1000)
    ref_nm, _, _ = oracle.search_for_initialization(e1.keypoints, e1.descriptors, e2.keypoints, e2.descriptors, 640, 480,
                                                    window=100, nnratio=0.9, check_ori=True)
    assert (int(n1), int(n2), int(nm)) == (len(e1.keypoints), len(e2.keypoints), ref_nm)
