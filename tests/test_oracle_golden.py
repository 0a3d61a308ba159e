"""The CPU restatement (oracle/orb_oracle.cpp) against the golden fixtures,
which were produced by the reference's own sources (tests/golden/make_golden.py)."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle


def test_extractor_tables(oracle, golden):
    for nf in (1000, 2000):
        g = golden(f"tables_{nf}.npz")
        p = pyoracle.Params(nf, 1.2, 8, 20, 7)
        arrs = [np.zeros(8, np.float32) for _ in range(4)] + [np.zeros(8, np.int32), np.zeros(16, np.int32)]
        oracle.fn("extractor_tables")(C.byref(p), *[x.ctypes.data_as(C.c_void_p) for x in arrs])
        for name, a in zip(["scale", "inv_scale", "sigma2", "inv_sigma2", "features_per_level", "umax"], arrs):
            assert np.array_equal(a, g[name]), name
    s, inv = pyoracle.scale_tables(8, 1.2)
    assert np.array_equal(np.array(s, np.float32), golden("tables_1000.npz")["scale"])


def test_extract_640x480(oracle, golden):
    g = golden("extract_640x480.npz")
    r = oracle.extract(g["image"], nfeatures=1000)
    assert len(r.keypoints) == len(g["keypoints"])
    assert r.keypoints.tobytes() == g["keypoints"].tobytes()
    assert np.array_equal(r.descriptors, g["descriptors"])
    assert [l.shape for l in r.pyramid] == [tuple(s) for s in g["level_shapes"]]
    assert [int(l.astype(np.int64).sum()) for l in r.pyramid] == list(g["level_sums"])
    assert np.array_equal(r.pyramid[7], g["level7"])


def test_search_for_initialization(oracle, golden):
    g = golden("init_640x480.npz")
    nm, m12, prev = oracle.search_for_initialization(g["keypoints1"], g["descriptors1"], g["keypoints2"],
                                                     g["descriptors2"], 640, 480, window=100, nnratio=0.9,
                                                     check_ori=True)
    assert nm == int(g["nmatches"])
    assert np.array_equal(m12, g["matches12"])
    assert np.array_equal(prev, g["prev_matched"])


def test_stereo(oracle, golden):
    g = golden("stereo_640x240.npz")
    L = oracle.extract(g["left"], nfeatures=1000)
    R = oracle.extract(g["right"], nfeatures=1000)
    assert L.keypoints.tobytes() == g["keypoints_left"].tobytes()
    assert R.keypoints.tobytes() == g["keypoints_right"].tobytes()
    ur, depth = oracle.compute_stereo_matches(L.keypoints, L.descriptors, R.keypoints, R.descriptors, L.pyramid,
                                              R.pyramid, 640, 240, float(g["bf"]), float(g["fx"]))
    assert np.array_equal(ur, g["uright"])
    assert np.array_equal(depth, g["depth"])
    assert (ur > 0).sum() > 50


def test_search_by_projection(oracle, golden):
    e = golden("extract_640x480.npz")
    g = golden("projection_640x480.npz")
    for th in (1.0, 3.75):
        nm, match = oracle.search_by_projection(e["keypoints"], e["descriptors"], 640, 480, g["mappoints"],
                                                g["mp_descriptors"], th=th, nnratio=0.8, uright=g["uright"],
                                                claimed=g["claimed"])
        assert nm == int(g[f"nmatches_th{th}"])
        assert np.array_equal(match, g[f"match_th{th}"])


def test_knn(oracle, golden):
    g = golden("knn_200x3000.npz")
    i1, d1, i2, d2 = oracle.knn2(g["query"], g["train"])
    for a, name in zip((i1, d1, i2, d2), ("idx1", "d1", "idx2", "d2")):
        assert np.array_equal(a, g[name]), name


def test_hamming_kat(oracle, golden):
    g = golden("hamming_kat.npz")
    pats = g["patterns"]
    for i in range(len(pats)):
        for j in range(len(pats)):
            assert oracle.descriptor_distance(pats[i], pats[j]) == g["distance"][i, j]
    assert g["distance"][0, 1] == 256 and g["distance"][2, 3] == 256 and g["distance"][0, 0] == 0


def test_constant_image_has_no_keypoints(oracle):
    r = oracle.extract(np.full((480, 640), 77, np.uint8))
    assert len(r.keypoints) == 0 and r.descriptors.shape == (0, 32)


@pytest.mark.skipif(not pyoracle.ref_available(), reason="reference sources not built here")
def test_oracle_matches_reference_on_fresh_seeds(oracle):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    R = pyoracle.RefOracle()
    for seed, (w, h, nf) in enumerate([(752, 480, 1500), (1241, 376, 2000)]):
        img = syn.scene(w, h, 100 + seed)
        a = R.extract(img, nfeatures=nf)
        b = oracle.extract(img, nfeatures=nf)
        assert a.keypoints.tobytes() == b.keypoints.tobytes()
        assert np.array_equal(a.descriptors, b.descriptors)


def _projframe_args(g):
    w, h = (int(v) for v in g["size"])
    mo = pyoracle.make_motion(g["Tcw"], g["Tlw"], *[float(v) for v in g["camera"]])
    ur = g["uright"] if len(g["uright"]) else None
    return w, h, mo, ur


@pytest.mark.parametrize("name", ["stereo_fwd_1241x376", "mono_640x480"])
def test_search_by_projection_frame(oracle, golden, name):
    g = golden(f"projframe_{name}.npz")
    w, h, mo, ur = _projframe_args(g)
    nm, match = oracle.search_by_projection_frame(g["keypoints"], g["descriptors"], w, h, g["last_keypoints"],
                                                  g["last_mappoints"], g["last_mp_descriptors"], mo,
                                                  th=float(g["th"]), mono=bool(g["mono"]), check_ori=True,
                                                  uright=ur, claimed=g["claimed"])
    assert nm == int(g["nmatches"])
    assert np.array_equal(match, g["match"])
    assert (match == -4).any() and (match >= 0).any()


@pytest.mark.skipif(not pyoracle.ref_available(), reason="reference sources not built here")
def test_search_by_projection_frame_reference_cases(oracle):
    """Oracle against the reference build: forward / backward / static stereo,
    monocular, rotation check on and off, and the k-deep assignment chain."""
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    R = pyoracle.RefOracle()
    img = syn.scene(752, 480, 61)
    cur = oracle.extract(img, nfeatures=1500)
    for seed, (stereo, dz, mono, th) in enumerate([(True, 2.0, False, 15.0), (True, -2.0, False, 15.0),
                                                    (True, 0.2, False, 15.0), (False, 0.0, True, 7.0)]):
        c = syn.motion_case(cur.keypoints, cur.descriptors, 752, 480, seed=70 + seed, stereo=stereo, dz=dz)
        mo = pyoracle.make_motion(c["Tcw"], c["Tlw"], c["fx"], c["fy"], c["cx"], c["cy"], c["bf"], c["b"])
        for co in (True, False):
            args = (cur.keypoints, cur.descriptors, 752, 480, c["last_kps"], c["last_mps"], c["last_mp_desc"], mo)
            kw = dict(th=th, mono=mono, check_ori=co, uright=c["uright"], claimed=c["claimed"])
            a = R.search_by_projection_frame(*args, **kw)
            b = oracle.search_by_projection_frame(*args, **kw)
            assert a[0] == b[0] and np.array_equal(a[1], b[1]), (seed, co)
    for every in (1, 3):
        kps, desc, c, w, h = syn.chain_case(30, seed=every, observed_every=every)
        mo = pyoracle.make_motion(c["Tcw"], c["Tlw"], c["fx"], c["fy"], c["cx"], c["cy"], c["bf"], c["b"])
        args = (kps, desc, w, h, c["last_kps"], c["last_mps"], c["last_mp_desc"], mo)
        a = R.search_by_projection_frame(*args, th=7.0, mono=True, check_ori=False)
        b = oracle.search_by_projection_frame(*args, th=7.0, mono=True, check_ori=False)
        assert a[0] == b[0] and np.array_equal(a[1], b[1])
        if every == 1:
            assert np.array_equal(b[1], np.arange(30))


# MapPoint::ComputeDistinctiveDescriptors (src/MapPoint.cc:365-447)
DISTINCTIVE_KAT_ROWS = [5, 7, 0, 10, 0, 4, -1, -1, 40, 256, 17, 46, 8]


@pytest.mark.parametrize("case", ["kat", "short", "long", "ties"])
def test_distinctive_descriptors_golden(oracle, golden, case):
    g = golden("distinctive.npz")
    pool, offsets, rows = g[f"{case}_pool"], g[f"{case}_offsets"], g[f"{case}_rows"]
    best, desc = oracle.distinctive_descriptors(pool, offsets, rows, g[f"{case}_initial"])
    assert np.array_equal(desc, g[f"{case}_descriptors"])
    # the chosen row is one of the map point's valid observations
    for i in range(len(best)):
        lst = rows[offsets[i]:offsets[i + 1]]
        if best[i] >= 0:
            assert best[i] in lst
        else:
            assert best[i] == -1 and not (lst >= 0).any()
    if case == "kat":
        assert best.tolist() == DISTINCTIVE_KAT_ROWS


def test_distinctive_descriptors_malformed_lists(oracle):
    pool = np.zeros((4, 32), np.uint8)
    offsets = np.array([0, 2, 1, 3, 5], np.int32)  # map point 1 has a decreasing offset
    rows = np.array([0, 1, 2, 4, -2], np.int32)    # map point 3 has rows 4 and -2, outside [-1, 4)
    best, _ = oracle.distinctive_descriptors(pool, offsets, rows)
    assert best.tolist() == [0, -2, 1, -2]


@pytest.mark.skipif(not pyoracle.ref_available(), reason="reference sources not built here")
def test_distinctive_descriptors_reference_fresh_seeds(oracle):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    R = pyoracle.RefOracle()
    for seed, kw in ((101, dict(mean_len=8.0)), (102, dict(mean_len=30.0, max_len=120)),
                     (103, dict(mean_len=5.0, low_entropy=True, extra_rows=32))):
        pool, offsets, rows = syn.observation_case(800, seed, **kw)
        init = np.random.default_rng(seed).integers(0, 256, (800, 32), dtype=np.uint8)
        _, a = oracle.distinctive_descriptors(pool, offsets, rows, init)
        _, b = R.distinctive_descriptors(pool, offsets, rows, init)
        assert np.array_equal(a, b), seed


# Frame::isInFrustum (src/Frame.cc:491-578) with MapPoint::PredictScale
FRUSTUM_CASES = ["stereo_1241x376", "mono_640x480", "wide_levels_752x480"]


def frustum_inputs(g, name):
    fx, fy, cx, cy, bf, w, h, sf, nl, lim = (float(v) for v in g[f"{name}_camera"])
    cam = pyoracle.make_frustum_camera(g[f"{name}_Tcw"], fx, fy, cx, cy, bf, 0.0, w, 0.0, h, sf, int(nl))
    geom = np.ascontiguousarray(g[f"{name}_geometry"]).view(pyoracle.GEOM_DTYPE).reshape(-1)
    return cam, geom, lim


@pytest.mark.parametrize("name", FRUSTUM_CASES)
def test_is_in_frustum_golden(oracle, golden, name):
    g = golden("frustum.npz")
    cam, geom, lim = frustum_inputs(g, name)
    out, nin = oracle.is_in_frustum(cam, geom, lim, g[f"{name}_initial"])
    assert nin == int(g[f"{name}_nin"])
    assert out.tobytes() == g[f"{name}_out"].tobytes()
    # map points out of view keep their earlier fields
    off = out["track_in_view"] == 0
    assert np.array_equal(out["proj_x"][off], g[f"{name}_initial"]["proj_x"][off])


@pytest.mark.skipif(not pyoracle.ref_available(), reason="reference sources not built here")
def test_is_in_frustum_reference_fresh_seeds(oracle):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    R = pyoracle.RefOracle()
    for seed, (w, h, fx, sf, nl) in enumerate([(640, 480, 500.0, 1.2, 8), (1241, 376, 718.9, 1.2, 8),
                                               (1280, 720, 900.0, 1.3, 10), (640, 480, 400.0, 2.0, 4)]):
        Tcw, g = syn.frustum_case(3000, 200 + seed, w, h, fx, sf, nl)
        geom = np.ascontiguousarray(g).view(pyoracle.GEOM_DTYPE).reshape(-1)
        cam = pyoracle.make_frustum_camera(Tcw, fx, fx, w / 2, h / 2, 40.0, 0.0, w, 0.0, h, sf, nl)
        a, na = oracle.is_in_frustum(cam, geom, 0.5)
        b, nb = R.is_in_frustum(cam, geom, 0.5)
        assert na == nb and a.tobytes() == b.tobytes(), seed


# Frame::UndistortKeyPoints / ComputeImageBounds (src/Frame.cc:724-819)
UNDISTORT_CASES = ["euroc_752x480", "tum1_640x480", "k1_zero_1241x376", "strong_640x480"]


@pytest.mark.parametrize("name", UNDISTORT_CASES)
def test_undistort_golden(oracle, golden, name):
    g = golden("undistort.npz")
    K, d, (w, h) = g[f"{name}_K"], g[f"{name}_dist"], g[f"{name}_size"]
    out = oracle.undistort_keypoints(K, d, g[f"{name}_keypoints"])
    assert out.tobytes() == g[f"{name}_undistorted"].tobytes()
    assert oracle.compute_image_bounds(w, h, K, d).tobytes() == g[f"{name}_bounds"].tobytes()
    if name.startswith("k1_zero"):
        assert out.tobytes() == g[f"{name}_keypoints"].tobytes()


# DBoW2 TemplatedVocabulary::transform (Frame::ComputeBoW)
BOW_VOCABULARIES = {"k10_L3_l1_tfidf": (1, 4), "k6_L4_l2_idf": (2, 4)}


def bow_vocabulary(g, name, path):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    voc = {key: g[f"{name}_{key}"] for key in ("parents", "is_leaf", "descriptors", "weights")}
    voc.update({key: int(g[f"{name}_{key}"]) for key in ("k", "L", "scoring", "weighting")})
    syn.write_vocabulary_text(voc, path)
    return voc


@pytest.mark.parametrize("name", list(BOW_VOCABULARIES))
def test_bow_transform_golden(oracle, golden, tmp_path, name):
    g = golden("bow.npz")
    path = str(tmp_path / "voc.txt")
    voc = bow_vocabulary(g, name, path)
    assert oracle.vocabulary_load(path) == int(voc["is_leaf"].sum())
    for fi in range(3):
        for lu in BOW_VOCABULARIES[name]:
            out = oracle.bow_transform(path, g[f"{name}_f{fi}_desc"], lu)
            for key, val in out.items():
                assert np.array_equal(val, g[f"{name}_f{fi}_lu{lu}_{key}"]), (fi, lu, key)


@pytest.mark.parametrize("sc", [0, 1])
def test_search_by_bow_golden(oracle, golden, sc):
    """ORBmatcher::SearchByBoW(KeyFrame*, Frame&) against the reference's outputs."""
    g = golden("search_by_bow.npz")
    pre = f"s{sc}_"
    fv = {side: tuple(g[pre + side + "_" + k] for k in ("fv_nodes", "fv_offsets", "fv_features"))
          for side in ("kf", "f")}
    for ori, ratio in ((1, 0.75), (0, 0.9)):
        nm, match = oracle.search_by_bow(g[pre + "kf_kps"], g[pre + "kf_desc"], g[pre + "kf_mp"], fv["kf"],
                                         g[pre + "f_kps"], g[pre + "f_desc"], fv["f"], ratio, bool(ori))
        assert nm == int(g[pre + f"nm_{ori}"])
        assert np.array_equal(match, g[pre + f"match_{ori}"])


@pytest.mark.parametrize("sc", [0, 1])
def test_search_by_bow_keyframes_golden(oracle, golden, sc):
    """ORBmatcher::SearchByBoW(KeyFrame*, KeyFrame*) against the reference's outputs."""
    g = golden("search_by_bow.npz")
    pre = f"s{sc}_"
    fv = {side: tuple(g[pre + side + "_" + k] for k in ("fv_nodes", "fv_offsets", "fv_features"))
          for side in ("kf", "f")}
    nm, match = oracle.search_by_bow_kf(g[pre + "kf_kps"], g[pre + "kf_desc"], g[pre + "kf_mp"], fv["kf"],
                                        g[pre + "f_kps"], g[pre + "f_desc"], g[pre + "f_mp"], fv["f"])
    assert nm == int(g[pre + "kf_nm"])
    assert np.array_equal(match, g[pre + "kf_match"])


RELOC_PARAMS = ((10.0, 100, True), (3.0, 50, False))


@pytest.mark.parametrize("sc", [0, 1])
def test_search_by_projection_keyframe_golden(oracle, golden, sc):
    """SearchByProjection(Frame&, KeyFrame*, sAlreadyFound, th, ORBdist) against
    the reference's outputs (a reset by the rotation check reads as -1 there)."""
    g = golden("reloc_search.npz")
    pre = f"s{sc}_"
    geom = np.ascontiguousarray(g[pre + "geometry"]).view(pyoracle.GEOM_DTYPE).reshape(-1)
    for k, (th, od, ori) in enumerate(RELOC_PARAMS):
        nm, match = oracle.search_by_projection_kf(g[pre + "kps"], g[pre + "desc"], 640, 480, g[pre + "Tcw"],
                                                   g[pre + "cam"], g[pre + "kf_kps"], geom, g[pre + "mp_desc"],
                                                   g[pre + "mp_state"], th, od, ori, g[pre + "claimed"])
        assert nm == int(g[pre + f"nm_{k}"])
        assert np.array_equal(np.where(match == -4, -1, match), g[pre + f"match_{k}"])


@pytest.mark.parametrize("sc", [0, 1])
def test_search_for_triangulation_golden(oracle, golden, sc):
    """ORBmatcher::SearchForTriangulation against the reference's outputs."""
    g = golden("triangulation.npz")
    pre = f"s{sc}_"
    fv1 = tuple(g[pre + k + "1"] for k in ("fv_nodes", "fv_offsets", "fv_features"))
    fv2 = tuple(g[pre + k + "2"] for k in ("fv_nodes", "fv_offsets", "fv_features"))
    for k, (st, ori) in enumerate(((False, True), (True, False))):
        nm, match = oracle.search_for_triangulation(
            g[pre + "kps1"], g[pre + "desc1"], g[pre + "mp1"], g[pre + "ur1"], fv1, g[pre + "kps2"], g[pre + "desc2"],
            g[pre + "mp2"], g[pre + "ur2"], fv2, g[pre + "Cw1"], g[pre + "T2"], g[pre + "K2"], g[pre + "F12"],
            g["scale"], g["sigma2"], st, ori)
        assert nm == int(g[pre + f"nm_{k}"])
        assert np.array_equal(match, g[pre + f"match_{k}"])


@pytest.mark.parametrize("sc", [0, 1])
def test_search_by_projection_sim3_golden(oracle, golden, sc):
    """SearchByProjection(KeyFrame*, Scw, vpPoints, vpMatched, th) against the reference."""
    g = golden("sim3_search.npz")
    pre = f"s{sc}_"
    geom = np.ascontiguousarray(g[pre + "points"]).view(pyoracle.GEOM_DTYPE).reshape(-1)
    for th in (10, 5):
        nm, match = oracle.search_by_projection_sim3(g[pre + "kps"], g[pre + "desc"], 640, 480, g[pre + "Scw"],
                                                     g[pre + "cam"], geom, g[pre + "pdesc"], g[pre + "pstate"], th,
                                                     g[pre + "claimed"])
        assert nm == int(g[pre + f"nm_{th}"])
        assert np.array_equal(match, g[pre + f"match_{th}"])


@pytest.mark.parametrize("sc", [0, 1])
def test_fuse_candidates_golden(oracle, golden, sc):
    """ORBmatcher::Fuse(KeyFrame*, vpMapPoints, th): every map point's choice against the reference."""
    g = golden("fuse.npz")
    pre = f"s{sc}_"
    geom = np.ascontiguousarray(g[pre + "points"]).view(pyoracle.GEOM_DTYPE).reshape(-1)
    for th in (3.0, 5.0):
        nf, target = oracle.fuse_candidates(g[pre + "kps"], g[pre + "desc"], g[pre + "ur"], 640, 480, g[pre + "Tcw"],
                                            g[pre + "cam"], geom, g[pre + "pdesc"], g[pre + "pstate"], th)
        assert nf == int(g[pre + f"nf_{int(th)}"])
        assert np.array_equal(target, g[pre + f"target_{int(th)}"])


@pytest.mark.parametrize("sc", [0, 1])
def test_fuse_sim3_candidates_golden(oracle, golden, sc):
    """ORBmatcher::Fuse(KeyFrame*, Scw, vpPoints, th, vpReplacePoint): every point's choice."""
    g = golden("fuse.npz")
    pre = f"sim3_s{sc}_"
    geom = np.ascontiguousarray(g[pre + "points"]).view(pyoracle.GEOM_DTYPE).reshape(-1)
    nf, target = oracle.fuse_sim3_candidates(g[pre + "kps"], g[pre + "desc"], 640, 480, g[pre + "Scw"],
                                             g[pre + "cam"], geom, g[pre + "pdesc"], g[pre + "pstate"], 4.0)
    assert nf == int(g[pre + "nf"])
    assert np.array_equal(target, g[pre + "target"])


def sim3_pair_inputs(g, pre):
    G1 = np.ascontiguousarray(g[pre + "g1"]).view(pyoracle.GEOM_DTYPE).reshape(-1)
    G2 = np.ascontiguousarray(g[pre + "g2"]).view(pyoracle.GEOM_DTYPE).reshape(-1)
    return (g[pre + "kps1"], g[pre + "desc1"], g[pre + "kps2"], g[pre + "desc2"], 640, 480, g[pre + "T1"],
            g[pre + "T2"], float(g[pre + "s12"]), g[pre + "R12"], g[pre + "t12"], g[pre + "cam"], G1, g[pre + "d1"],
            g[pre + "st1"], G2, g[pre + "d2"], g[pre + "st2"])


@pytest.mark.parametrize("sc", [0, 1])
def test_search_by_sim3_golden(oracle, golden, sc):
    """ORBmatcher::SearchBySim3 against the reference (its keyframe windows are
    squares): two keyframes with different poses and feature sets, part of
    vpMatches12 already set (the reference reports those entries; the
    restatement skips them, as usable1 / usable2 encode)."""
    g = golden("search_by_sim3.npz")
    pre = f"s{sc}_"
    pre12 = g[pre + "pre12"]
    assert len(g[pre + "kps1"]) != len(g[pre + "kps2"]) and (pre12 >= 0).sum() > 20
    for th in (7.5, 3.0):
        nf, m12 = oracle.search_by_sim3(*sim3_pair_inputs(g, pre), th, pre12=pre12)
        assert nf == int(g[pre + f"nf_{th}"]) > 100
        assert np.array_equal(np.where(pre12 >= 0, pre12, m12), g[pre + f"match_{th}"])
        assert np.all(m12[pre12 >= 0] == -1)
