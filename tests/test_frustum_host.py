"""Host side of the batched Frame::isInFrustum: the pose matrices and the
PredictScale level thresholds orbgpu_frustum_frame_init computes (no GPU)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def init():
    from orb_slam2_detailed_comments_gb300 import build
    build.build(table=False)
    from orb_slam2_detailed_comments_gb300 import frustum_frame
    return frustum_frame


def levels_from_thresholds(rec, ratio):
    thr = rec["level_above"][:int(rec["nlevels"]) - 1].astype(np.float32)
    return (ratio[:, None] > thr[None, :]).sum(1).astype(np.int32)


@pytest.mark.parametrize("scale,nlevels", [(1.2, 8), (1.2, 16), (1.5, 5), (2.0, 3), (1.05, 12), (1.2, 1)])
def test_level_thresholds_equal_predict_scale(init, oracle, scale, nlevels):
    """MapPoint::PredictScale (ceil(logf(ratio) / logf(scale)), clamped) equals
    the count of thresholds below the ratio: on every float within 4096 ulps
    of each threshold and of each power of the scale, on a million log-uniform
    ratios, and on 0 and the smallest and largest floats.  (An infinite ratio
    -- a map point on the camera centre with a zero minimum distance -- makes
    the reference convert an infinite float to int, which is undefined: x86
    gives level 0, Arm the last level; the thresholds give the last level.)"""
    rec = init(np.eye(3, 4), 500, 500, 320, 240, 40, 0, 640, 0, 480, scale, nlevels)
    centres = [float(t) for t in rec["level_above"][:nlevels - 1]] + [scale ** k for k in range(-2, nlevels + 2)]
    bits = [np.float32(c).view(np.int32) + np.arange(-4096, 4097, dtype=np.int32) for c in centres if c > 0]
    near = np.concatenate(bits).view(np.float32) if bits else np.zeros(0, np.float32)
    rng = np.random.default_rng(int(scale * 100) + nlevels)
    rand = np.exp(rng.uniform(np.log(1e-4), np.log(1e4), 1_000_000)).astype(np.float32)
    special = np.array([0.0, 1e-45, 1e-38, 1.0, 3.4e38], np.float32)
    ratio = np.concatenate([near, rand, special]).astype(np.float32)
    assert np.array_equal(levels_from_thresholds(rec, ratio), oracle.predict_scale(ratio, scale, nlevels))


def test_pose_matrices(init, oracle):
    """Rcw, tcw and Ow = -Rcw^T tcw (accumulated in double, rounded to float)."""
    rng = np.random.default_rng(3)
    T = rng.normal(size=(3, 4)).astype(np.float32)
    rec = init(T, 500, 500, 320, 240, 40, 0, 640, 0, 480, 1.2, 8)
    assert np.array_equal(rec["Rcw"].reshape(3, 3), T[:, :3]) and np.array_equal(rec["tcw"], T[:, 3])
    R, t = T[:, :3].astype(np.float64), T[:, 3].astype(np.float64)
    Ow = [np.float32(((-R[0, i]) * t[0] + (-R[1, i]) * t[1]) + (-R[2, i]) * t[2]) for i in range(3)]
    assert np.array_equal(rec["Ow"], np.array(Ow, np.float32))


def test_bad_frame_arguments(init):
    from orb_slam2_detailed_comments_gb300 import OrbGpuError
    with pytest.raises(OrbGpuError):
        init(np.eye(3, 4), 500, 500, 320, 240, 40, 0, 640, 0, 480, 1.0, 8)
    with pytest.raises(OrbGpuError):
        init(np.eye(3, 4), 500, 500, 320, 240, 40, 0, 640, 0, 480, 1.2, 17)


@pytest.mark.parametrize("name", ["euroc_752x480", "tum1_640x480", "k1_zero_1241x376", "strong_640x480"])
def test_image_bounds_host(init, golden, name):
    """orbgpu_compute_image_bounds (host) equals the reference's ComputeImageBounds."""
    from orb_slam2_detailed_comments_gb300 import compute_image_bounds
    g = golden("undistort.npz")
    w, h = g[f"{name}_size"]
    b = compute_image_bounds(int(w), int(h), g[f"{name}_K"], g[f"{name}_dist"])
    assert b.tobytes() == g[f"{name}_bounds"].tobytes()
