"""Helpers of the GPU parity tests (test infrastructure)."""
import os

import numpy as np
import pytest

from oracle import pyoracle


def require_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orb_slam2_detailed_comments_gb300 import build
    build.build()
    return torch


def assert_kps_equal(a, b, what=""):
    a = np.asarray(a)
    b = np.asarray(b)
    assert len(a) == len(b), f"{what}: {len(a)} vs {len(b)} keypoints"
    if a.tobytes() != b.tobytes():
        for f in pyoracle.KP_DTYPE.names:
            d = np.nonzero(a[f] != b[f])[0]
            if len(d):
                raise AssertionError(f"{what}: field {f} differs at {d[:8]}: {a[f][d[:4]]} vs {b[f][d[:4]]}")
