"""GPU matchers through the C ABI against the oracle and the golden fixtures."""
import numpy as np
import pytest

from oracle import pyoracle
from tests.gpu_util import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return require_gpu()


def frame(kps, desc, w, h, uright=None):
    from orb_slam2_detailed_comments_gb300 import FrameView
    s, _ = pyoracle.scale_tables(8, 1.2)
    return FrameView(kps, desc, w, h, np.array(s, np.float32), uright)


def test_init_golden(torch, golden):
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    g = golden("init_640x480.npz")
    m = ORBmatcher(0.9, True)
    F1 = frame(g["keypoints1"], g["descriptors1"], 640, 480)
    F2 = frame(g["keypoints2"], g["descriptors2"], 640, 480)
    prev = np.stack([g["keypoints1"]["x"], g["keypoints1"]["y"]], 1)
    nm, m12, prev2 = m.SearchForInitialization(F1, F2, prev, 100)
    assert nm == int(g["nmatches"])
    assert np.array_equal(m12, g["matches12"])
    assert np.array_equal(prev2, g["prev_matched"])


@pytest.mark.parametrize("seed,ori,window", [(1, True, 100), (2, False, 100), (3, True, 50), (4, True, 200)])
def test_init_vs_oracle(torch, oracle, seed, ori, window):
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    f1, f2, _ = syn.frame_pair(640, 480, seed)
    a = oracle.extract(f1, nfeatures=2000)
    b = oracle.extract(f2, nfeatures=2000)
    r = oracle.search_for_initialization(a.keypoints, a.descriptors, b.keypoints, b.descriptors, 640, 480,
                                         window=window, nnratio=0.9, check_ori=ori)
    m = ORBmatcher(0.9, ori)
    prev = np.stack([a.keypoints["x"], a.keypoints["y"]], 1)
    nm, m12, prev2 = m.SearchForInitialization(frame(a.keypoints, a.descriptors, 640, 480),
                                               frame(b.keypoints, b.descriptors, 640, 480), prev, window)
    assert nm == r[0]
    assert np.array_equal(m12, r[1])
    assert np.array_equal(prev2, r[2])


def test_projection_golden(torch, golden):
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    e = golden("extract_640x480.npz")
    g = golden("projection_640x480.npz")
    m = ORBmatcher(0.8, True)
    F = frame(e["keypoints"], e["descriptors"], 640, 480, g["uright"])
    for th in (1.0, 3.75):
        nm, match = m.SearchByProjection(F, g["mappoints"], g["mp_descriptors"], th, g["claimed"])
        assert nm == int(g[f"nmatches_th{th}"])
        assert np.array_equal(match, g[f"match_th{th}"])


def make_mappoints(kps, desc, M, rng):
    n = len(kps)
    src = rng.integers(0, n, M)
    mpd = desc[src] ^ np.packbits(rng.random((M, 256)) < 0.1, axis=1, bitorder="little")
    mps = np.zeros(M, pyoracle.MP_DTYPE)
    mps["proj_x"] = kps["x"][src] + rng.normal(0, 2, M)
    mps["proj_y"] = kps["y"][src] + rng.normal(0, 2, M)
    mps["proj_xr"] = -1
    mps["view_cos"] = 1.0
    mps["track_scale_level"] = kps["octave"][src]
    mps["track_in_view"] = 1
    return mps, mpd


@pytest.mark.parametrize("w,h,nf,seed", [(1280, 720, 2000, 1), (752, 480, 1500, 2)])
def test_projection_vs_oracle(torch, oracle, w, h, nf, seed):
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    rng = np.random.default_rng(seed)
    a = oracle.extract(syn.scene(w, h, seed), nfeatures=nf)
    mps, mpd = make_mappoints(a.keypoints, a.descriptors, 3000, rng)
    th = 15.0 / 2.5
    r = oracle.search_by_projection(a.keypoints, a.descriptors, w, h, mps, mpd, th=th, nnratio=0.8)
    m = ORBmatcher(0.8, True)
    nm, match = m.SearchByProjection(frame(a.keypoints, a.descriptors, w, h), mps, mpd, th)
    assert nm == r[0]
    assert np.array_equal(match, r[1])


def test_stereo_golden(torch, golden, oracle):
    from orb_slam2_detailed_comments_gb300 import ORBextractor, ORBmatcher, compute_stereo_matches
    g = golden("stereo_640x240.npz")
    exL = ORBextractor(1000, 1.2, 8, 20, 7)
    exR = ORBextractor(1000, 1.2, 8, 20, 7)
    kL, dL = exL(g["left"])
    kR, dR = exR(g["right"])
    assert kL.tobytes() == g["keypoints_left"].tobytes()
    assert kR.tobytes() == g["keypoints_right"].tobytes()
    m = ORBmatcher(0.75, True)
    ur, dp = compute_stereo_matches(m, exL, exR, frame(kL, dL, 640, 240), frame(kR, dR, 640, 240),
                                    float(g["bf"]), float(g["fx"]))
    # bit-exact in practice; the contract is |delta| <= 1e-4 px
    np.testing.assert_allclose(ur, g["uright"], atol=1e-4, rtol=0)
    np.testing.assert_allclose(dp, g["depth"], atol=1e-4, rtol=1e-6)
    assert np.array_equal(ur > 0, g["uright"] > 0)


@pytest.mark.parametrize("seed", [1, 2])
def test_stereo_vs_oracle_1241x376(torch, oracle, seed):
    from orb_slam2_detailed_comments_gb300 import ORBextractor, ORBmatcher, compute_stereo_matches
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    left, right, _ = syn.stereo_pair(1241, 376, seed)
    exL = ORBextractor(2000, 1.2, 8, 20, 7)
    exR = ORBextractor(2000, 1.2, 8, 20, 7)
    kL, dL = exL(left)
    kR, dR = exR(right)
    L = oracle.extract(left, nfeatures=2000)
    R = oracle.extract(right, nfeatures=2000)
    u1, d1 = oracle.compute_stereo_matches(L.keypoints, L.descriptors, R.keypoints, R.descriptors, L.pyramid,
                                           R.pyramid, 1241, 376, 386.1, 718.856)
    m = ORBmatcher(0.75, True)
    u2, d2 = compute_stereo_matches(m, exL, exR, frame(kL, dL, 1241, 376), frame(kR, dR, 1241, 376), 386.1, 718.856)
    np.testing.assert_allclose(u2, u1, atol=1e-4, rtol=0)
    np.testing.assert_allclose(d2, d1, atol=1e-4, rtol=1e-6)
    assert np.array_equal(u1 > 0, u2 > 0) and (u1 > 0).sum() > 200


def test_batched_stereo_vs_oracle(torch, oracle):
    """orbgpu_batch_compute_stereo_matches: four stereo pairs of two sizes in
    one batch extraction (left and right frames interleaved, one pair listed
    right-first to exercise the frame indices), every pair against the
    oracle's Frame::ComputeStereoMatches on the same images, uR / depth within
    1e-4."""
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor, BatchStereo
    specs = [(1241, 376, 3), (640, 480, 4), (1241, 376, 5), (640, 480, 6)]
    imgs, pairs, refs = [], [], []
    for w, h, seed in specs:
        left, right, _ = syn.stereo_pair(w, h, seed)
        if seed == 5:  # right frame first in the batch
            pairs.append((len(imgs) + 1, len(imgs)))
            imgs += [right, left]
        else:
            pairs.append((len(imgs), len(imgs) + 1))
            imgs += [left, right]
        L = oracle.extract(left, nfeatures=2000)
        R = oracle.extract(right, nfeatures=2000)
        refs.append(oracle.compute_stereo_matches(L.keypoints, L.descriptors, R.keypoints, R.descriptors, L.pyramid,
                                                  R.pyramid, w, h, 386.1, 718.856) + (len(L.keypoints),))
    b = BatchExtractor(len(imgs), 1280, 720, 2000)
    k, d, c = b.extract([torch.from_numpy(i).cuda() for i in imgs], [2000] * len(imgs))
    ur, dp = BatchStereo(b).compute(pairs, 386.1, 718.856)
    ur, dp, c = ur.cpu().numpy(), dp.cpu().numpy(), c.cpu().numpy()
    for p, (u1, d1, n) in enumerate(refs):
        assert c[pairs[p][0]] == n
        np.testing.assert_allclose(ur[p, :n], u1, atol=1e-4, rtol=0)
        np.testing.assert_allclose(dp[p, :n], d1, atol=1e-4, rtol=1e-6)
        assert np.array_equal(u1 > 0, ur[p, :n] > 0) and (u1 > 0).sum() > 100


def test_knn_golden_and_oracle(torch, golden, oracle):
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    m = ORBmatcher()
    g = golden("knn_200x3000.npz")
    out = m.knn2(torch.from_numpy(g["query"]).cuda(), torch.from_numpy(g["train"]).cuda())
    for a, name in zip(out, ("idx1", "d1", "idx2", "d2")):
        assert np.array_equal(a.cpu().numpy(), g[name]), name
    q = syn.random_descriptors(1000, 3)
    t = syn.random_descriptors(20000, 4)
    ref = oracle.knn2(q, t)
    out = m.knn2(torch.from_numpy(q).cuda(), torch.from_numpy(t).cuda())
    for a, b in zip(out, ref):
        assert np.array_equal(a.cpu().numpy(), b)


def test_descriptor_distance_kat(torch, golden):
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    g = golden("hamming_kat.npz")
    p = g["patterns"]
    n = len(p)
    a = np.repeat(p, n, axis=0)
    b = np.tile(p, (n, 1))
    d = ORBmatcher.DescriptorDistance(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda())
    assert np.array_equal(d.cpu().numpy().reshape(n, n), g["distance"])


def test_projection_device_inputs(torch, oracle):
    """Device-resident frame, map point records as raw bytes and descriptors."""
    from orb_slam2_detailed_comments_gb300 import ORBextractor, ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    rng = np.random.default_rng(21)
    img = syn.scene(1241, 376, 21)
    ex = ORBextractor(2000, 1.2, 8, 20, 7)
    k, d = ex(torch.from_numpy(img).cuda(), device_out=True)
    kh = k.cpu().numpy().view(pyoracle.KP_DTYPE).reshape(-1)
    dh = d.cpu().numpy()
    mps, mpd = make_mappoints(kh, dh, 2500, rng)
    r = oracle.search_by_projection(kh, dh, 1241, 376, mps, mpd, th=6.0, nnratio=0.8)
    m = ORBmatcher(0.8, True)
    nm, match = m.SearchByProjection(frame(k, d, 1241, 376), torch.from_numpy(mps.view(np.uint8)).cuda(),
                                     torch.from_numpy(mpd).cuda(), 6.0)
    assert nm == r[0]
    assert np.array_equal(match.cpu().numpy(), r[1])


def test_tc_operand_layout(torch):
    """One 128 x 256 x 256 tensor-core MMA group on +-1 FP8 expansions equals
    the integer dot products (the shared-memory operand layout self-test)."""
    import ctypes as C
    from orb_slam2_detailed_comments_gb300._lib import lib
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    q = syn.random_descriptors(128, 1)
    t = syn.random_descriptors(256, 2)
    bq = 1 - 2 * np.unpackbits(q, axis=1, bitorder="little").astype(np.int32)
    bt = 1 - 2 * np.unpackbits(t, axis=1, bitorder="little").astype(np.int32)
    dots = np.zeros((128, 256), np.float32)
    st = np.zeros(1, np.int32)
    rc = lib().orbgpu_debug_tc_probe(q.ctypes.data_as(C.c_void_p), t.ctypes.data_as(C.c_void_p),
                                     dots.ctypes.data_as(C.c_void_p), st.ctypes.data_as(C.c_void_p), 128, 2048)
    assert rc == 0 and st[0] == 0
    assert np.array_equal(dots, (bq @ bt.T).astype(np.float32))


@pytest.mark.parametrize("nq,nt", [(1, 1), (129, 257), (1000, 20000)])
def test_knn_tensor_cores_oracle(torch, oracle, nq, nt):
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    q = syn.random_descriptors(nq, 5)
    t = syn.random_descriptors(nt, 6)
    ref = oracle.knn2(q, t)
    out = ORBmatcher().knn2(torch.from_numpy(q).cuda(), torch.from_numpy(t).cuda(), algo=1)
    for a, b, name in zip(out, ref, ("idx1", "d1", "idx2", "d2")):
        assert np.array_equal(a.cpu().numpy(), b), name


def test_knn_tensor_cores_golden_and_ties(torch, golden):
    """Golden vectors, then clustered descriptors (many equal distances) against
    the popcount kernel at a size with many slices."""
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    m = ORBmatcher()
    g = golden("knn_200x3000.npz")
    out = m.knn2(torch.from_numpy(g["query"]).cuda(), torch.from_numpy(g["train"]).cuda(), algo=1)
    for a, name in zip(out, ("idx1", "d1", "idx2", "d2")):
        assert np.array_equal(a.cpu().numpy(), g[name]), name
    # the same seed gives both sets the same 200 centres: many equal distances
    q = torch.from_numpy(syn.clustered_descriptors(5000, 200, 0.05, 8)).cuda()
    t = torch.from_numpy(syn.clustered_descriptors(60000, 200, 0.05, 8)).cuda()
    a = m.knn2(q, t, algo=0)
    b = m.knn2(q, t, algo=1)
    for x, y in zip(a, b):
        assert torch.equal(x, y)


@pytest.mark.parametrize("kind", ["uniform", "clustered"])
def test_knn_full_size_against_oracle_sample(torch, oracle, kind):
    """The brute-force kNN at its stated size (50,000 queries x 200,000 train
    descriptors; uniform bits, or 2,000 centres with 10 % flips): both kernels
    over the whole problem, equal to each other, and 512 seeded queries against
    the oracle's loop over DescriptorDistance (src/ORBmatcher.cc:2083-2103)
    over the full train set.  Integer results: exact equality."""
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    if kind == "uniform":
        q, t = syn.random_descriptors(50000, 1), syn.random_descriptors(200000, 2)
    else:
        q, t = syn.clustered_descriptors(50000, 2000, 0.1, 3), syn.clustered_descriptors(200000, 2000, 0.1, 4)
    m = ORBmatcher()
    qd, td = torch.from_numpy(q).cuda(), torch.from_numpy(t).cuda()
    pop = [a.cpu().numpy() for a in m.knn2(qd, td, algo=0)]
    tc = [a.cpu().numpy() for a in m.knn2(qd, td, algo=1)]
    for a, b, name in zip(pop, tc, ("idx1", "d1", "idx2", "d2")):
        assert np.array_equal(a, b), f"popcount vs tensor cores: {name}"
    sample = np.sort(np.random.default_rng(2024).choice(len(q), 512, replace=False))
    ref = oracle.knn2(q[sample], t)
    for a, b, name in zip(tc, ref, ("idx1", "d1", "idx2", "d2")):
        assert np.array_equal(a[sample], b), f"tensor cores vs oracle: {name}"


# ----------------------------------------------------------------- SearchByProjection(CurrentFrame, LastFrame)
def frame_pair_views(kps, desc, w, h, c, dev=False, torch=None):
    """(CurrentFrame, LastFrame) views of a motion case (host or device arrays)."""
    from orb_slam2_detailed_comments_gb300 import FrameView
    s, _ = pyoracle.scale_tables(8, 1.2)
    sf = np.array(s, np.float32)
    ur = c["uright"]
    lk, mps, mpd, cl = c["last_kps"], c["last_mps"], c["last_mp_desc"], c["claimed"]
    if dev:
        kps = torch.from_numpy(np.ascontiguousarray(kps).view(np.float32).reshape(-1, 7)).cuda()
        desc = torch.from_numpy(np.ascontiguousarray(desc)).cuda()
        ur = None if ur is None else torch.from_numpy(np.ascontiguousarray(ur)).cuda()
        lk = torch.from_numpy(np.ascontiguousarray(lk).view(np.float32).reshape(-1, 7)).cuda()
        mps = torch.from_numpy(np.ascontiguousarray(mps).view(np.uint8)).cuda()
        mpd = torch.from_numpy(np.ascontiguousarray(mpd)).cuda()
        cl = None if cl is None else torch.from_numpy(np.ascontiguousarray(cl)).cuda()
    CF = FrameView(kps, desc, w, h, sf, ur, Tcw=c["Tcw"], fx=c["fx"], fy=c["fy"], cx=c["cx"], cy=c["cy"],
                   mbf=c["bf"], mb=c["b"], claimed=cl)
    LF = FrameView(lk, mpd, w, h, sf, None, Tcw=c["Tlw"], mappoints=mps, mp_descriptors=mpd)
    return CF, LF


@pytest.mark.parametrize("name", ["stereo_fwd_1241x376", "mono_640x480"])
def test_projection_frame_golden(torch, golden, name):
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    g = golden(f"projframe_{name}.npz")
    w, h = (int(v) for v in g["size"])
    cam = [float(v) for v in g["camera"]]
    c = dict(uright=g["uright"] if len(g["uright"]) else None, last_kps=g["last_keypoints"],
             last_mps=g["last_mappoints"], last_mp_desc=g["last_mp_descriptors"], claimed=g["claimed"],
             Tcw=g["Tcw"], Tlw=g["Tlw"], fx=cam[0], fy=cam[1], cx=cam[2], cy=cam[3], bf=cam[4], b=cam[5])
    for dev in (False, True):
        CF, LF = frame_pair_views(g["keypoints"], g["descriptors"], w, h, c, dev=dev, torch=torch)
        nm, match = ORBmatcher(0.9, True).SearchByProjection(CF, LF, float(g["th"]), bool(g["mono"]))
        match = match.cpu().numpy() if dev else match
        assert nm == int(g["nmatches"])
        assert np.array_equal(match, g["match"])


@pytest.mark.parametrize("stereo,dz,mono,th,ori,dev", [(True, 2.0, False, 15.0, True, True),
                                                      (True, -2.0, False, 15.0, True, False),
                                                      (True, 0.2, False, 15.0, False, True),
                                                      (False, 0.0, True, 7.0, True, True),
                                                      (False, 0.0, True, 7.0, False, False)])
def test_projection_frame_vs_oracle(torch, oracle, stereo, dz, mono, th, ori, dev):
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    img = syn.scene(1280, 720, 81)
    cur = oracle.extract(img, nfeatures=2000)
    c = syn.motion_case(cur.keypoints, cur.descriptors, 1280, 720, seed=int(10 * dz) + 90, stereo=stereo, dz=dz)
    mo = pyoracle.make_motion(c["Tcw"], c["Tlw"], c["fx"], c["fy"], c["cx"], c["cy"], c["bf"], c["b"])
    ref = oracle.search_by_projection_frame(cur.keypoints, cur.descriptors, 1280, 720, c["last_kps"], c["last_mps"],
                                            c["last_mp_desc"], mo, th=th, mono=mono, check_ori=ori,
                                            uright=c["uright"], claimed=c["claimed"])
    CF, LF = frame_pair_views(cur.keypoints, cur.descriptors, 1280, 720, c, dev=dev, torch=torch)
    nm, match = ORBmatcher(0.9, ori).SearchByProjection(CF, LF, th, mono)
    match = match.cpu().numpy() if dev else match
    assert nm == ref[0]
    assert np.array_equal(match, ref[1])


@pytest.mark.parametrize("every", [1, 3])
def test_projection_frame_deep_chain(torch, oracle, every):
    """A 30-deep assignment chain: more than the parallel rounds, so the
    sequential fallback decides; observed_every 3 mixes owners that block
    nothing (they are overwritten, and counted, as in the reference)."""
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    kps, desc, c, w, h = syn.chain_case(30, seed=every, observed_every=every)
    mo = pyoracle.make_motion(c["Tcw"], c["Tlw"], c["fx"], c["fy"], c["cx"], c["cy"], c["bf"], c["b"])
    ref = oracle.search_by_projection_frame(kps, desc, w, h, c["last_kps"], c["last_mps"], c["last_mp_desc"], mo,
                                            th=7.0, mono=True, check_ori=False)
    CF, LF = frame_pair_views(kps, desc, w, h, c)
    nm, match = ORBmatcher(0.9, False).SearchByProjection(CF, LF, 7.0, True)
    assert nm == ref[0]
    assert np.array_equal(match, ref[1])


def test_projection_frame_edges(torch, oracle):
    """No LastFrame keypoints; LastFrame without map points; no current keypoints."""
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    kps, desc, c, w, h = syn.chain_case(8, seed=5)
    m = ORBmatcher(0.9, True)
    empty = dict(c, last_kps=c["last_kps"][:0], last_mps=c["last_mps"][:0], last_mp_desc=c["last_mp_desc"][:0])
    CF, LF = frame_pair_views(kps, desc, w, h, empty)
    nm, match = m.SearchByProjection(CF, LF, 7.0, True)
    assert nm == 0 and np.array_equal(match, np.full(8, -1))
    none = dict(c, last_mps=c["last_mps"].copy())
    none["last_mps"]["flags"] = 0
    CF, LF = frame_pair_views(kps, desc, w, h, none)
    nm, match = m.SearchByProjection(CF, LF, 7.0, True)
    assert nm == 0 and np.array_equal(match, np.full(8, -1))
    CF, LF = frame_pair_views(kps[:0], desc[:0], w, h, dict(c, claimed=c["claimed"][:0]))
    nm, match = m.SearchByProjection(CF, LF, 7.0, True)
    assert nm == 0 and len(match) == 0


def test_knn_ratio_accept(torch, oracle):
    """The accept mask is the reference's float test bestDist < bestDist2 * ratio."""
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    q = syn.clustered_descriptors(3000, 50, 0.1, 12)
    t = syn.clustered_descriptors(20000, 50, 0.1, 12)
    i1, d1, i2, d2 = oracle.knn2(q, t)
    out = ORBmatcher().knn2(torch.from_numpy(q).cuda(), torch.from_numpy(t).cuda(), algo=-1, ratio=0.8)
    for a, b in zip(out[:4], (i1, d1, i2, d2)):
        assert np.array_equal(a.cpu().numpy(), b)
    want = (d1.astype(np.float32) < d2.astype(np.float32) * np.float32(0.8)).astype(np.uint8)
    assert np.array_equal(out[4].cpu().numpy(), want)
    assert 0 < want.sum() < len(want)


@pytest.mark.parametrize("seed,th,orbdist,ori,dev", [(0, 10.0, 100, True, False), (1, 3.0, 50, False, False),
                                                     (2, 10.0, 64, True, True), (3, 5.0, 100, True, True)])
def test_search_by_projection_keyframe_vs_oracle(torch, oracle, seed, th, orbdist, ori, dev):
    """SearchByProjection(Frame&, KeyFrame*, sAlreadyFound, th, ORBdist), host
    and device inputs, against the oracle (-4 resets included)."""
    from orb_slam2_detailed_comments_gb300 import ORBmatcher, frustum_frame
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    img = syn.scene(640, 480, 120 + seed)
    e = oracle.extract(img, nfeatures=1500)
    Tcw, cam, kfk, g, mpd, st, cl = syn.relocalisation_case(e.keypoints, e.descriptors, 640, 480, 120 + seed)
    geom = np.ascontiguousarray(g).view(pyoracle.GEOM_DTYPE).reshape(-1)
    ref_nm, ref = oracle.search_by_projection_kf(e.keypoints, e.descriptors, 640, 480, Tcw, cam, kfk, geom, mpd, st,
                                                 th, orbdist, ori, cl)
    pose = frustum_frame(Tcw, cam[0], cam[1], cam[2], cam[3], 0.0, 0.0, 640, 0.0, 480, 1.2, 8)
    usable = (st == 1).astype(np.uint8)
    m = ORBmatcher(0.9, ori)
    if dev:
        kd = torch.from_numpy(e.keypoints.view(np.float32).reshape(-1, 7).copy()).cuda()
        F = frame(kd, torch.from_numpy(e.descriptors).cuda(), 640, 480)
        nm, match = m.SearchByProjectionKeyFrame(
            F, pose, torch.from_numpy(kfk.view(np.float32).reshape(-1, 7).copy()).cuda(), torch.from_numpy(g).cuda(),
            torch.from_numpy(mpd).cuda(), torch.from_numpy(usable).cuda(), th, orbdist, torch.from_numpy(cl).cuda())
        match = match.cpu().numpy()
    else:
        nm, match = m.SearchByProjectionKeyFrame(frame(e.keypoints, e.descriptors, 640, 480), pose, kfk, g, mpd, usable,
                                                 th, orbdist, cl)
    assert nm == ref_nm
    assert np.array_equal(match, ref)
    assert ref_nm > 300


@pytest.mark.parametrize("seed,th,dev", [(0, 10, False), (1, 5, False), (2, 10, True)])
def test_search_by_projection_sim3_vs_oracle(torch, oracle, seed, th, dev):
    """SearchByProjection(KeyFrame*, Scw, vpPoints, vpMatched, th), host and
    device inputs, against the oracle."""
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    e = oracle.extract(syn.scene(640, 480, 140 + seed), nfeatures=1500)
    Scw, cam, g, pd, ps, cl = syn.sim3_case(e.keypoints, e.descriptors, 640, 480, 140 + seed)
    geom = np.ascontiguousarray(g).view(pyoracle.GEOM_DTYPE).reshape(-1)
    ref_nm, ref = oracle.search_by_projection_sim3(e.keypoints, e.descriptors, 640, 480, Scw, cam, geom, pd, ps, th,
                                                   cl)
    usable = (ps == 1).astype(np.uint8)
    m = ORBmatcher(0.9, True)
    if dev:
        kd = torch.from_numpy(e.keypoints.view(np.float32).reshape(-1, 7).copy()).cuda()
        KF = frame(kd, torch.from_numpy(e.descriptors).cuda(), 640, 480)
        nm, match = m.SearchByProjectionSim3(KF, Scw, *cam, torch.from_numpy(g).cuda(), torch.from_numpy(pd).cuda(),
                                             torch.from_numpy(usable).cuda(), th, torch.from_numpy(cl).cuda())
        match = match.cpu().numpy()
    else:
        nm, match = m.SearchByProjectionSim3(frame(e.keypoints, e.descriptors, 640, 480), Scw, *cam, g, pd, usable, th,
                                             cl)
    assert nm == ref_nm
    assert np.array_equal(match, ref)
    assert ref_nm > 300


@pytest.mark.parametrize("seed,th,dev", [(0, 3.0, False), (1, 5.0, True)])
def test_fuse_candidates_vs_oracle(torch, oracle, seed, th, dev):
    """The search half of Fuse(KeyFrame*, vpMapPoints, th) against the oracle."""
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    e = oracle.extract(syn.scene(640, 480, 150 + seed), nfeatures=1500)
    Tcw, cam5, g, pd, ps, ur = syn.fuse_case(e.keypoints, e.descriptors, 150 + seed)
    geom = np.ascontiguousarray(g).view(pyoracle.GEOM_DTYPE).reshape(-1)
    ref_nf, ref = oracle.fuse_candidates(e.keypoints, e.descriptors, ur, 640, 480, Tcw, cam5, geom, pd, ps, th)
    s, _ = pyoracle.scale_tables(8, 1.2)
    inv_sigma2 = (1.0 / (np.array(s, np.float32) ** 2)).astype(np.float32)
    usable = (ps == 1).astype(np.uint8)
    m = ORBmatcher(0.6, True)
    if dev:
        kd = torch.from_numpy(e.keypoints.view(np.float32).reshape(-1, 7).copy()).cuda()
        KF = frame(kd, torch.from_numpy(e.descriptors).cuda(), 640, 480, torch.from_numpy(ur).cuda())
        target, _ = m.FuseCandidates(KF, Tcw, *cam5, inv_sigma2, torch.from_numpy(g).cuda(),
                                     torch.from_numpy(pd).cuda(), torch.from_numpy(usable).cuda(), th)
        target = target.cpu().numpy()
    else:
        KF = frame(e.keypoints, e.descriptors, 640, 480, ur)
        target, _ = m.FuseCandidates(KF, Tcw, *cam5, inv_sigma2, g, pd, usable, th)
    assert np.array_equal(target, ref)
    assert int((target >= 0).sum()) == ref_nf > 300


@pytest.mark.parametrize("seed,th,dev", [(0, 4.0, False), (1, 8.0, True)])
def test_fuse_sim3_candidates_vs_oracle(torch, oracle, seed, th, dev):
    """The search half of Fuse(KeyFrame*, Scw, vpPoints, th, vpReplacePoint) against the oracle."""
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    e = oracle.extract(syn.scene(640, 480, 160 + seed), nfeatures=1500)
    Scw, cam, g, pd, ps, _ = syn.sim3_case(e.keypoints, e.descriptors, 640, 480, 160 + seed)
    geom = np.ascontiguousarray(g).view(pyoracle.GEOM_DTYPE).reshape(-1)
    ref_nf, ref = oracle.fuse_sim3_candidates(e.keypoints, e.descriptors, 640, 480, Scw, cam, geom, pd, ps, th)
    usable = (ps == 1).astype(np.uint8)
    m = ORBmatcher(0.6, True)
    if dev:
        kd = torch.from_numpy(e.keypoints.view(np.float32).reshape(-1, 7).copy()).cuda()
        KF = frame(kd, torch.from_numpy(e.descriptors).cuda(), 640, 480)
        target, _ = m.FuseSim3Candidates(KF, Scw, *cam, torch.from_numpy(g).cuda(), torch.from_numpy(pd).cuda(),
                                         torch.from_numpy(usable).cuda(), th)
        target = target.cpu().numpy()
    else:
        target, _ = m.FuseSim3Candidates(frame(e.keypoints, e.descriptors, 640, 480), Scw, *cam, g, pd, usable, th)
    assert np.array_equal(target, ref)
    assert int((target >= 0).sum()) == ref_nf > 300


@pytest.mark.parametrize("seed,th", [(0, 7.5), (1, 3.0), (2, 7.5)])
def test_search_by_sim3_vs_oracle(torch, oracle, seed, th):
    """SearchBySim3(pKF1, pKF2, vpMatches12, s12, R12, t12, th) against the
    oracle: two views of a plane (keyframes of different poses and feature
    sets), part of vpMatches12 already set and encoded through usable1 /
    usable2."""
    from orb_slam2_detailed_comments_gb300 import ORBmatcher
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    img1, img2, geo = syn.sim3_pair_images(170 + seed)
    e1 = oracle.extract(img1, nfeatures=1500)
    e2 = oracle.extract(img2, nfeatures=1200)
    T1, T2, s12, R12, t12, cam, g1, d1, st1, g2, d2, st2, pre12 = syn.sim3_pair_case(
        e1.keypoints, e1.descriptors, e2.keypoints, e2.descriptors, geo, 170 + seed)
    G1 = np.ascontiguousarray(g1).view(pyoracle.GEOM_DTYPE).reshape(-1)
    G2 = np.ascontiguousarray(g2).view(pyoracle.GEOM_DTYPE).reshape(-1)
    ref_nf, ref = oracle.search_by_sim3(e1.keypoints, e1.descriptors, e2.keypoints, e2.descriptors, 640, 480, T1, T2,
                                        s12, R12, t12, cam, G1, d1, st1, G2, d2, st2, th, pre12=pre12)
    u1, u2 = syn.sim3_usable(st1, st2, pre12)
    nf, m12 = ORBmatcher(0.75, True).SearchBySim3(frame(e1.keypoints, e1.descriptors, 640, 480),
                                                  frame(e2.keypoints, e2.descriptors, 640, 480), T1, T2, s12, R12,
                                                  t12, *cam, g1, d1, u1, g2, d2, u2, th)
    assert nf == ref_nf
    assert np.array_equal(m12, ref)
    assert ref_nf > 100 and (pre12 >= 0).sum() > 20
