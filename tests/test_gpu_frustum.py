"""Frame::isInFrustum on the GPU (orbgpu_is_in_frustum) against the oracle
and the golden fixtures, and chained into SearchByProjection on the device."""
import numpy as np
import pytest

from oracle import pyoracle
from tests.gpu_util import require_gpu

pytestmark = pytest.mark.gpu

CASES = ["stereo_1241x376", "mono_640x480", "wide_levels_752x480"]


@pytest.fixture(scope="module")
def torch():
    return require_gpu()


def frame_record(Tcw, camera):
    from orb_slam2_detailed_comments_gb300 import frustum_frame
    fx, fy, cx, cy, bf, w, h, sf, nl, _ = (float(v) for v in camera)
    return frustum_frame(Tcw, fx, fy, cx, cy, bf, 0.0, w, 0.0, h, sf, int(nl))


def run(torch, frames, geoms, initials, lim, pinned=False):
    """One batched call over several frames; returns (records per frame, in-view counts)."""
    from orb_slam2_detailed_comments_gb300 import FRUSTUM_FRAME_DTYPE, is_in_frustum
    offs = np.zeros(len(geoms) + 1, np.int32)
    offs[1:] = np.cumsum([len(g) for g in geoms])
    geom = np.ascontiguousarray(np.concatenate(geoms).astype(np.float32))
    recs = np.ascontiguousarray(np.concatenate(initials))
    fr = np.ascontiguousarray(np.array(frames, FRUSTUM_FRAME_DTYPE)).view(np.uint8)
    if pinned:
        F, O, G = (torch.from_numpy(a).pin_memory() for a in (fr, offs, geom))
        M = torch.from_numpy(recs.view(np.uint8)).pin_memory()
    else:
        F, O, G = (torch.from_numpy(a).cuda() for a in (fr, offs, geom))
        M = torch.from_numpy(recs.view(np.uint8)).cuda()
    iv = torch.zeros(len(geoms), dtype=torch.int32, device="cuda")
    is_in_frustum(F, O, G, M, lim, iv)
    torch.cuda.synchronize()
    out = M.cpu().numpy().view(pyoracle.MP_DTYPE)
    return [out[offs[i]:offs[i + 1]] for i in range(len(geoms))], iv.cpu().numpy()


@pytest.mark.parametrize("name", CASES)
def test_golden_one_frame(torch, golden, name):
    g = golden("frustum.npz")
    rec = frame_record(g[f"{name}_Tcw"], g[f"{name}_camera"])
    (out,), iv = run(torch, [rec], [g[f"{name}_geometry"]], [g[f"{name}_initial"]], float(g[f"{name}_camera"][9]))
    assert out.tobytes() == g[f"{name}_out"].tobytes()
    assert iv[0] == int(g[f"{name}_nin"])


@pytest.mark.parametrize("pinned", [False, True])
def test_batch_of_frames_vs_oracle(torch, oracle, pinned):
    """48 frames of uneven map point counts (0 to 6000) and cameras in one call."""
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    rng = np.random.default_rng(7)
    cams = [(640, 480, 500.0, 1.2, 8), (1241, 376, 718.856, 1.2, 8), (752, 480, 458.7, 1.5, 12),
            (1280, 720, 900.0, 1.3, 10)]
    frames, geoms, inits, refs = [], [], [], []
    for f in range(48):
        w, h, fx, sf, nl = cams[f % 4]
        m = int(rng.choice([0, 1, 37, 800, 3000, 6000]))
        Tcw, g = syn.frustum_case(m, 300 + f, w, h, fx, sf, nl)
        camera = np.array([fx, fx, w / 2, h / 2, 40.0 if f % 2 else 0.0, w, h, sf, nl, 0.5], np.float32)
        frames.append(frame_record(Tcw, camera))
        init = np.zeros(m, pyoracle.MP_DTYPE)
        init["proj_y"] = rng.normal(size=m)
        init["bad"] = rng.integers(0, 2, m)
        geoms.append(g)
        inits.append(init)
        cam = pyoracle.make_frustum_camera(Tcw, fx, fx, w / 2, h / 2, camera[4], 0.0, w, 0.0, h, sf, nl)
        refs.append(oracle.is_in_frustum(cam, np.ascontiguousarray(g).view(pyoracle.GEOM_DTYPE).reshape(-1), 0.5,
                                         init))
    outs, iv = run(torch, frames, geoms, inits, 0.5, pinned=pinned)
    for f in range(48):
        assert outs[f].tobytes() == refs[f][0].tobytes(), f
        assert iv[f] == refs[f][1], f


def test_chained_into_search_by_projection(torch, oracle):
    """isInFrustum then SearchByProjection(Frame&, vector<MapPoint*>, th) with
    the records staying on the device, against the oracle doing the same."""
    from orb_slam2_detailed_comments_gb300 import FrameView, ORBmatcher, is_in_frustum
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    w, h, fx = 640, 480, 500.0
    img = syn.scene(w, h, 17)
    ex = oracle.extract(img, nfeatures=1500)
    kps, desc = ex.keypoints, ex.descriptors
    rng = np.random.default_rng(5)
    # map points behind keypoints at random depths (identity pose), their
    # descriptors a few bits from the keypoints', and more in the box
    sel = rng.choice(len(kps), 900, replace=False)
    z = rng.uniform(2.0, 30.0, len(sel))
    x = (kps["x"][sel] - w / 2) / fx * z
    y = (kps["y"][sel] - h / 2) / fx * z
    pw = np.stack([x, y, z], 1)
    d = np.linalg.norm(pw, axis=1)
    lvl = kps["octave"][sel].astype(np.float64)
    maxd = d * 1.2 ** (lvl + rng.uniform(-0.4, 0.4, len(sel)))
    g = np.zeros((len(sel), 8), np.float32)
    g[:, :3] = pw
    g[:, 3:6] = pw / d[:, None]
    g[:, 6] = maxd / 1.2 ** 7
    g[:, 7] = maxd
    mpd = desc[sel] ^ (rng.integers(0, 256, (len(sel), 32)) & rng.integers(0, 256, (len(sel), 32))
                       & rng.integers(0, 256, (len(sel), 32)) & rng.integers(0, 256, (len(sel), 32))).astype(np.uint8)
    Tcw = np.eye(3, 4, dtype=np.float32)
    camera = np.array([fx, fx, w / 2, h / 2, 0.0, w, h, 1.2, 8, 0.5], np.float32)
    init = np.zeros(len(sel), pyoracle.MP_DTYPE)
    cam = pyoracle.make_frustum_camera(Tcw, fx, fx, w / 2, h / 2, 0.0, 0.0, w, 0.0, h, 1.2, 8)
    ref_recs, nin = oracle.is_in_frustum(cam, g.view(pyoracle.GEOM_DTYPE).reshape(-1), 0.5, init)
    ref_nm, ref_match = oracle.search_by_projection(kps, desc, w, h, ref_recs, mpd, th=1.0, nnratio=0.8)
    assert nin > 500 and ref_nm > 100
    # the same on the device, records never leaving it
    offs = torch.tensor([0, len(sel)], dtype=torch.int32, device="cuda")
    G = torch.from_numpy(g).cuda()
    M = torch.from_numpy(init.view(np.uint8).copy()).cuda()
    F = torch.from_numpy(np.array([frame_record(Tcw, camera)]).view(np.uint8)).cuda()
    is_in_frustum(F, offs, G, M, 0.5)
    s, _ = pyoracle.scale_tables(8, 1.2)
    KD = torch.from_numpy(kps.view(np.float32).reshape(len(kps), 7).copy()).cuda()
    DD = torch.from_numpy(desc).cuda()
    nm, match = ORBmatcher(0.8, True).SearchByProjection(FrameView(KD, DD, w, h, np.array(s, np.float32)), M,
                                                         torch.from_numpy(mpd).cuda(), 1.0)
    assert nm == ref_nm
    assert np.array_equal(match.cpu().numpy(), ref_match)


UNDISTORT_CASES = ["euroc_752x480", "tum1_640x480", "k1_zero_1241x376", "strong_640x480"]


@pytest.mark.parametrize("name", UNDISTORT_CASES)
@pytest.mark.parametrize("where", ["device", "pinned", "in_place"])
def test_undistort_golden(torch, golden, name, where):
    """Frame::UndistortKeyPoints on the GPU equals the reference's (golden)."""
    from orb_slam2_detailed_comments_gb300 import undistort_keypoints
    g = golden("undistort.npz")
    kps = np.ascontiguousarray(g[f"{name}_keypoints"])
    raw = torch.from_numpy(kps.view(np.float32).reshape(len(kps), 7).copy())
    if where == "pinned":
        out = undistort_keypoints(raw.pin_memory(), g[f"{name}_K"], g[f"{name}_dist"])
    elif where == "in_place":
        dev = raw.cuda()
        out = undistort_keypoints(dev, g[f"{name}_K"], g[f"{name}_dist"], out=dev)
    else:
        out = undistort_keypoints(raw.cuda(), g[f"{name}_K"], g[f"{name}_dist"])
    torch.cuda.synchronize()
    assert out.cpu().numpy().tobytes() == g[f"{name}_undistorted"].tobytes()


def test_undistort_extractor_output_vs_oracle(torch, oracle):
    """Keypoints straight from the GPU extractor, undistorted on the device."""
    from orb_slam2_detailed_comments_gb300 import ORBextractor, undistort_keypoints
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    img = syn.scene(752, 480, 33)
    ex = ORBextractor(1500, 1.2, 8, 20, 7, 752, 480)
    kd, _ = ex(torch.from_numpy(img).cuda(), device_out=True)
    K, d = (458.654, 457.296, 367.215, 248.375), (-0.28340811, 0.07395907, 0.00019359, 1.76187114e-05)
    out = undistort_keypoints(kd, K, d)
    torch.cuda.synchronize()
    host = kd.cpu().numpy().view(pyoracle.KP_DTYPE).reshape(-1)
    ref = oracle.undistort_keypoints(K, d, host)
    assert out.cpu().numpy().tobytes() == ref.tobytes()
