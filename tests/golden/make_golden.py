"""Generate the golden fixtures of the ORB front-end path.

The outputs come from the reference's own src/ORBextractor.cc,
src/ORBmatcher.cc, src/Frame.cc and src/MapPoint.cc, compiled unmodified against the cv
stand-in (oracle/Makefile target ``ref``; needs the reference sources, so this
script runs only where they are present).  Inputs are stored with the outputs,
so the fixtures do not depend on the generator's random streams.

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py projframe  # only the named groups
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle  # noqa: E402
from oracle.pyoracle import MP_DTYPE, RefOracle  # noqa: E402
from orb_slam2_detailed_comments_gb300 import synthetic as syn  # noqa: E402


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print(f"{name}: {os.path.getsize(path) // 1024} KiB")


GROUPS = ("extract", "projection", "knn", "kat", "tables", "projframe", "distinctive", "frustum", "undistort", "bow", "sbb", "reloc", "tri", "sim3", "fuse", "bysim3")


def main(groups=GROUPS):
    pyoracle.build(ref=True)
    R = RefOracle()
    if any(g in groups for g in ("extract", "projection")):
        base_fixtures(R, groups)
    if "knn" in groups:
        knn_fixture(R)
    if "kat" in groups:
        kat_fixture(R)
    if "tables" in groups:
        tables_fixture(R)
    if "projframe" in groups:
        projframe_fixture(R)
    if "distinctive" in groups:
        distinctive_fixture(R)
    if "frustum" in groups:
        frustum_fixture(R)
    if "undistort" in groups:
        undistort_fixture(R)
    if "bow" in groups:
        bow_fixture(R)
    if "sbb" in groups:
        search_by_bow_fixture(R)
    if "reloc" in groups:
        reloc_fixture(R)
    if "tri" in groups:
        triangulation_fixture(R)
    if "sim3" in groups:
        sim3_fixture(R)
    if "fuse" in groups:
        fuse_fixture(R)
    if "bysim3" in groups:
        by_sim3_fixture(R)


def base_fixtures(R, groups):
    # (extract, init, stereo and projection share their inputs)
    # 1. extraction, 640x480, nFeatures 1000 (and the pyramid, as level digests)
    f1, f2, H = syn.frame_pair(640, 480, seed=0)
    a = R.extract(f1, nfeatures=1000)
    b = R.extract(f2, nfeatures=1000)
    save("extract_640x480.npz", image=f1, keypoints=a.keypoints, descriptors=a.descriptors,
         level_shapes=np.array([l.shape for l in a.pyramid]),
         level_sums=np.array([int(l.astype(np.int64).sum()) for l in a.pyramid]),
         level7=a.pyramid[7])

    # 2. SearchForInitialization between the warped pair (window 100, ratio 0.9, rotation check)
    nm, m12, prev = R.search_for_initialization(a.keypoints, a.descriptors, b.keypoints, b.descriptors, 640, 480,
                                                window=100, nnratio=0.9, check_ori=True)
    save("init_640x480.npz", image2=f2, keypoints1=a.keypoints, descriptors1=a.descriptors,
         keypoints2=b.keypoints, descriptors2=b.descriptors, nmatches=np.array(nm), matches12=m12,
         prev_matched=prev)

    # 3. ComputeStereoMatches on a rectified 640x240 pair, bf 386.1, fx 718.856
    left, right, _ = syn.stereo_pair(640, 240, seed=3)
    L = R.extract(left, nfeatures=1000)
    Rr = R.extract(right, nfeatures=1000)
    ur, depth = R.compute_stereo_matches(L.keypoints, L.descriptors, Rr.keypoints, Rr.descriptors, L.pyramid,
                                         Rr.pyramid, 640, 240, 386.1, 718.856)
    save("stereo_640x240.npz", left=left, right=right, keypoints_left=L.keypoints, descriptors_left=L.descriptors,
         keypoints_right=Rr.keypoints, descriptors_right=Rr.descriptors, uright=ur, depth=depth,
         bf=np.float32(386.1), fx=np.float32(718.856))

    # 4. SearchByProjection(Frame, map points, th) with 1000 map points
    rng = np.random.default_rng(11)
    n = len(a.keypoints)
    M = 1000
    src = rng.integers(0, n, M)
    mpd = a.descriptors[src] ^ np.packbits(rng.random((M, 256)) < 0.1, axis=1, bitorder="little")
    mps = np.zeros(M, MP_DTYPE)
    mps["proj_x"] = a.keypoints["x"][src] + rng.normal(0, 2, M)
    mps["proj_y"] = a.keypoints["y"][src] + rng.normal(0, 2, M)
    mps["proj_xr"] = np.where(rng.random(M) < 0.3, mps["proj_x"] - rng.uniform(5, 50, M), -1)
    mps["view_cos"] = rng.uniform(0.99, 1.0, M)
    mps["track_scale_level"] = a.keypoints["octave"][src]
    mps["track_in_view"] = rng.random(M) < 0.95
    mps["bad"] = rng.random(M) < 0.02
    claimed = (rng.random(n) < 0.05).astype(np.uint8)
    uright = np.where(rng.random(n) < 0.3, a.keypoints["x"] - rng.uniform(5, 50, n), -1).astype(np.float32)
    out = {}
    for th in (1.0, 3.75):
        nmp, match = R.search_by_projection(a.keypoints, a.descriptors, 640, 480, mps, mpd, th=th, nnratio=0.8,
                                            uright=uright, claimed=claimed)
        out[f"nmatches_th{th}"] = np.array(nmp)
        out[f"match_th{th}"] = match
    save("projection_640x480.npz", mappoints=mps, mp_descriptors=mpd, claimed=claimed, uright=uright, **out)


def knn_fixture(R):
    # 5. brute-force k=2 over DescriptorDistance
    q = syn.clustered_descriptors(200, 20, 0.1, seed=5)
    t = syn.clustered_descriptors(3000, 20, 0.1, seed=6)
    i1, d1, i2, d2 = R.knn2(q, t)
    save("knn_200x3000.npz", query=q, train=t, idx1=i1, d1=d1, idx2=i2, d2=d2)


def kat_fixture(R):
    # 6. DescriptorDistance known answers on crafted bit patterns
    pats = [np.zeros(32, np.uint8), np.full(32, 255, np.uint8), np.tile(np.array([0x55], np.uint8), 32),
            np.tile(np.array([0xAA], np.uint8), 32), np.arange(32, dtype=np.uint8),
            np.array([1 << (i % 8) for i in range(32)], np.uint8)]
    pa = np.stack(pats)
    dist = np.array([[R.descriptor_distance(x, y) for y in pats] for x in pats], np.int32)
    save("hamming_kat.npz", patterns=pa, distance=dist)


def tables_fixture(R):
    # 7. tables of the ORBextractor constructor
    import ctypes as C
    for nf in (1000, 2000):
        p = pyoracle.Params(nf, 1.2, 8, 20, 7)
        arrs = [np.zeros(8, np.float32) for _ in range(4)] + [np.zeros(8, np.int32), np.zeros(16, np.int32)]
        R.fn("extractor_tables")(C.byref(p), *[x.ctypes.data_as(C.c_void_p) for x in arrs])
        save(f"tables_{nf}.npz", scale=arrs[0], inv_scale=arrs[1], sigma2=arrs[2], inv_sigma2=arrs[3],
             features_per_level=arrs[4], umax=arrs[5])


def projframe_fixture(R):
    # 8. SearchByProjection(CurrentFrame, LastFrame, th, bMono): a stereo pair
    # moving forward (th 15) and a monocular pair (th 7), rotation check on
    from oracle.pyoracle import make_motion
    cases = {}
    for name, (w, h, nf, stereo, dz, th) in {"stereo_fwd_1241x376": (1241, 376, 2000, True, 2.0, 15.0),
                                             "mono_640x480": (640, 480, 1000, False, 0.0, 7.0)}.items():
        img = syn.scene(w, h, 40 + len(cases))
        cur = R.extract(img, nfeatures=nf)
        c = syn.motion_case(cur.keypoints, cur.descriptors, w, h, seed=50 + len(cases), stereo=stereo, dz=dz)
        mo = make_motion(c["Tcw"], c["Tlw"], c["fx"], c["fy"], c["cx"], c["cy"], c["bf"], c["b"])
        nm, match = R.search_by_projection_frame(cur.keypoints, cur.descriptors, w, h, c["last_kps"], c["last_mps"],
                                                 c["last_mp_desc"], mo, th=th, mono=not stereo, check_ori=True,
                                                 uright=c["uright"], claimed=c["claimed"])
        ur = c["uright"] if c["uright"] is not None else np.zeros(0, np.float32)
        cases[name] = dict(keypoints=cur.keypoints, descriptors=cur.descriptors, uright=ur, claimed=c["claimed"],
                           last_keypoints=c["last_kps"], last_mappoints=c["last_mps"],
                           last_mp_descriptors=c["last_mp_desc"], Tcw=c["Tcw"], Tlw=c["Tlw"],
                           camera=np.array([c["fx"], c["fy"], c["cx"], c["cy"], c["bf"], c["b"]], np.float32),
                           size=np.array([w, h]), th=np.float32(th), mono=np.array(not stereo),
                           nmatches=np.array(nm), match=match)
    for name, arrays in cases.items():
        save(f"projframe_{name}.npz", **arrays)


def distinctive_kats():
    """Hand-made observation lists for MapPoint::ComputeDistinctiveDescriptors
    (pool, offsets, rows).  Descriptor b(k) has its first k bits set, so
    d(b(i), b(j)) = |i - j|."""
    def b(k):
        bits = np.zeros(256, np.uint8)
        bits[:k] = 1
        return np.packbits(bits, bitorder="little")
    pool = np.stack([b(k) for k in range(0, 257)])  # row k = b(k)
    lists = [
        [5],                      # one observation: chosen
        [7, 3],                   # two: both medians 0, the first wins
        [0, 10, 30],              # rows 0/10/30: medians 10, 10, 20 -> row 0
        [30, 10, 0],              # reversed: medians 20, 10, 10 -> row 10
        [0, 4, 9, 20],            # N 4, median element 1: 4, 4, 5, 11 -> row 0
        [20, 9, 4, 0],            # medians 11, 5, 4, 4 -> row 4
        [-1, -1],                 # every keyframe bad: unchanged
        [],                       # no observation: unchanged
        [-1, 40, -1, 42, 100],    # bad entries skipped: 40, 42, 100 -> medians 2, 2, 58 -> row 40
        [256, 0, 128],            # distances up to 256: medians 128, 128, 128 -> row 256
        [17] * 40,                # 40 equal descriptors (long list): all medians 0 -> the first
        list(range(60, 0, -1)),   # rows 60..1, median element 29: rows 16..46 have the least
                                  # median (15); the first in list order is row 46
        [-1] * 35 + [8, 9],       # long list, only two valid
    ]
    offsets = np.zeros(len(lists) + 1, np.int32)
    offsets[1:] = np.cumsum([len(x) for x in lists])
    rows = np.array([r for x in lists for r in x], np.int32)
    return pool, offsets, rows


def distinctive_fixture(R):
    # 9. MapPoint::ComputeDistinctiveDescriptors: hand-made lists and seeded
    # synthetic maps (short, long and tie-heavy lists)
    arrays = {}
    cases = {"kat": distinctive_kats(),
             "short": syn.observation_case(1500, 11, mean_len=6.0, max_len=64),
             "long": syn.observation_case(300, 12, mean_len=40.0, max_len=200),
             "ties": syn.observation_case(1500, 13, mean_len=5.0, max_len=48, low_entropy=True, extra_rows=64)}
    rng = np.random.default_rng(14)
    for name, (pool, offsets, rows) in cases.items():
        m = len(offsets) - 1
        initial = rng.integers(0, 256, (m, 32), dtype=np.uint8)
        _, desc = R.distinctive_descriptors(pool, offsets, rows, initial)
        arrays.update({f"{name}_pool": pool, f"{name}_offsets": offsets, f"{name}_rows": rows,
                       f"{name}_initial": initial, f"{name}_descriptors": desc})
    save("distinctive.npz", **arrays)


FRUSTUM_CAMERAS = {
    # name: (w, h, fx, fy, cx, cy, bf, scale, nlevels, seed, cos limit)
    "stereo_1241x376": (1241, 376, 718.856, 718.856, 607.1928, 185.2157, 386.1448, 1.2, 8, 61, 0.5),
    "mono_640x480": (640, 480, 535.4, 539.2, 320.1, 247.6, 0.0, 1.2, 8, 62, 0.5),
    "wide_levels_752x480": (752, 480, 458.654, 457.296, 367.215, 248.375, 47.9, 1.5, 12, 63, 0.3),
}


def frustum_fixture(R):
    # 10. Frame::isInFrustum with MapPoint::PredictScale on three cameras
    from oracle.pyoracle import GEOM_DTYPE, MP_DTYPE, make_frustum_camera
    arrays = {}
    for name, (w, h, fx, fy, cx, cy, bf, sf, nl, seed, lim) in FRUSTUM_CAMERAS.items():
        Tcw, g = syn.frustum_case(4000, seed, w, h, fx, sf, nl)
        geom = np.ascontiguousarray(g).view(GEOM_DTYPE).reshape(-1)
        cam = make_frustum_camera(Tcw, fx, fy, cx, cy, bf, 0.0, w, 0.0, h, sf, nl)
        init = np.zeros(len(geom), MP_DTYPE)
        init["proj_x"] = -1.0
        init["track_scale_level"] = 99
        out, nin = R.is_in_frustum(cam, geom, lim, init)
        arrays.update({f"{name}_Tcw": Tcw, f"{name}_camera": np.array([fx, fy, cx, cy, bf, w, h, sf, nl, lim],
                                                                        np.float32),
                       f"{name}_geometry": g, f"{name}_initial": init, f"{name}_out": out, f"{name}_nin": np.array(nin)})
    save("frustum.npz", **arrays)


UNDISTORT_CAMERAS = {
    # name: (fx, fy, cx, cy), (k1 k2 p1 p2 [k3]), width, height
    "euroc_752x480": ((458.654, 457.296, 367.215, 248.375), (-0.28340811, 0.07395907, 0.00019359, 1.76187114e-05),
                      752, 480),
    "tum1_640x480": ((517.306408, 516.469215, 318.643040, 255.313989),
                     (0.262383, -0.953104, -0.005358, 0.002628, 1.163314), 640, 480),
    "k1_zero_1241x376": ((718.856, 718.856, 607.1928, 185.2157), (0.0, 0.1, 0.001, 0.0), 1241, 376),
    "strong_640x480": ((400.0, 400.0, 320.0, 240.0), (-0.4, 0.2, 0.001, -0.002, -0.05), 640, 480),
}


def undistort_fixture(R):
    # 11. Frame::UndistortKeyPoints and Frame::ComputeImageBounds (the
    # reference's own functions, cv::undistortPoints restated in the cv stand-in)
    from oracle.pyoracle import KP_DTYPE
    rng = np.random.default_rng(71)
    arrays = {}
    for name, (K, d, w, h) in UNDISTORT_CAMERAS.items():
        n = 3000
        kps = np.zeros(n, KP_DTYPE)
        kps["x"] = rng.uniform(-4, w + 4, n)
        kps["y"] = rng.uniform(-4, h + 4, n)
        kps["size"] = 31.0
        kps["angle"] = rng.uniform(0, 360, n)
        kps["response"] = rng.uniform(0, 100, n)
        kps["octave"] = rng.integers(0, 8, n)
        arrays.update({f"{name}_K": np.array(K, np.float32), f"{name}_dist": np.array(d, np.float32),
                       f"{name}_size": np.array([w, h]), f"{name}_keypoints": kps,
                       f"{name}_undistorted": R.undistort_keypoints(K, d, kps),
                       f"{name}_bounds": R.compute_image_bounds(w, h, K, d)})
    save("undistort.npz", **arrays)


BOW_VOCABULARIES = {
    # name: (k, L, scoring, weighting, seed, levelsup values)
    "k10_L3_l1_tfidf": (10, 3, 0, 0, 81, (1, 4)),
    "k6_L4_l2_idf": (6, 4, 1, 2, 82, (2, 4)),
}


def bow_features(voc, n, seed):
    """Descriptors for the vocabulary transform: noisy copies of random words
    (about 1 bit in 16 flipped) and some uniform ones."""
    rng = np.random.default_rng(seed)
    leaves = np.nonzero(voc["is_leaf"])[0]
    base = voc["descriptors"][rng.choice(leaves, n - n // 8)]
    flips = rng.integers(0, 256, base.shape, dtype=np.uint8)
    for _ in range(3):
        flips &= rng.integers(0, 256, base.shape, dtype=np.uint8)
    return np.concatenate([base ^ flips, rng.integers(0, 256, (n // 8, 32), dtype=np.uint8)])


def bow_fixture(R):
    # 12. DBoW2 TemplatedVocabulary::transform (Frame::ComputeBoW) on synthetic
    # vocabularies written in the loadFromTextFile format
    import tempfile
    arrays = {}
    for name, (k, L, sc, wt, seed, lups) in BOW_VOCABULARIES.items():
        voc = syn.vocabulary(k, L, seed, scoring=sc, weighting=wt)
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "voc.txt")
            syn.write_vocabulary_text(voc, path)
            assert R.vocabulary_load(path) == int(voc["is_leaf"].sum())
            arrays.update({f"{name}_{key}": np.asarray(voc[key]) for key in
                           ("k", "L", "scoring", "weighting", "parents", "is_leaf", "descriptors", "weights")})
            for fi, n in enumerate((1500, 40, 900)):
                desc = bow_features(voc, n, seed * 10 + fi)
                arrays[f"{name}_f{fi}_desc"] = desc
                for lu in lups:
                    out = R.bow_transform(path, desc, lu)
                    for key, val in out.items():
                        arrays[f"{name}_f{fi}_lu{lu}_{key}"] = val
    save("bow.npz", **arrays)


def search_by_bow_fixture(R):
    # 13. ORBmatcher::SearchByBoW(KeyFrame*, Frame&) on two scene pairs, the
    # FeatureVectors from the reference's transform (k 10, L 4, levelsup 2)
    import tempfile
    voc = syn.vocabulary(10, 4, 5)
    arrays = {}
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "voc.txt")
        syn.write_vocabulary_text(voc, path)
        R.vocabulary_load(path)
        for sc in range(2):
            f1, f2, _ = syn.frame_pair(640, 480, 70 + sc)
            a, b = R.extract(f1, nfeatures=1500), R.extract(f2, nfeatures=1500)
            fa, fb = R.bow_transform(path, a.descriptors, 2), R.bow_transform(path, b.descriptors, 2)
            mp = np.random.default_rng(sc).choice([0, 1, 1, 1, 2], len(a.keypoints)).astype(np.uint8)
            pre = f"s{sc}_"
            arrays.update({pre + "kf_kps": a.keypoints, pre + "kf_desc": a.descriptors, pre + "kf_mp": mp,
                           pre + "f_kps": b.keypoints, pre + "f_desc": b.descriptors})
            for side, fv in (("kf", fa), ("f", fb)):
                for key in ("fv_nodes", "fv_offsets", "fv_features"):
                    arrays[pre + side + "_" + key] = fv[key]
            for ori, ratio in ((1, 0.75), (0, 0.9)):
                nm, match = R.search_by_bow(a.keypoints, a.descriptors, mp,
                                            (fa["fv_nodes"], fa["fv_offsets"], fa["fv_features"]), b.keypoints,
                                            b.descriptors, (fb["fv_nodes"], fb["fv_offsets"], fb["fv_features"]),
                                            ratio, bool(ori))
                arrays[pre + f"nm_{ori}"] = np.array(nm)
                arrays[pre + f"match_{ori}"] = match
            # SearchByBoW(KeyFrame*, KeyFrame*): the second view as a keyframe
            mp2 = np.random.default_rng(10 + sc).choice([0, 1, 1, 1, 2], len(b.keypoints)).astype(np.uint8)
            arrays[pre + "f_mp"] = mp2
            nm, match = R.search_by_bow_kf(a.keypoints, a.descriptors, mp,
                                           (fa["fv_nodes"], fa["fv_offsets"], fa["fv_features"]), b.keypoints,
                                           b.descriptors, mp2, (fb["fv_nodes"], fb["fv_offsets"], fb["fv_features"]))
            arrays[pre + "kf_nm"] = np.array(nm)
            arrays[pre + "kf_match"] = match
    save("search_by_bow.npz", **arrays)


def reloc_fixture(R):
    # 14. ORBmatcher::SearchByProjection(Frame&, KeyFrame*, sAlreadyFound, th,
    # ORBdist) (relocalisation) on two scenes
    from oracle.pyoracle import GEOM_DTYPE
    arrays = {}
    for sc in range(2):
        img = syn.scene(640, 480, 90 + sc)
        e = R.extract(img, nfeatures=1500)
        Tcw, cam, kfk, g, mpd, st, cl = syn.relocalisation_case(e.keypoints, e.descriptors, 640, 480, 90 + sc)
        geom = np.ascontiguousarray(g).view(GEOM_DTYPE).reshape(-1)
        pre = f"s{sc}_"
        arrays.update({pre + "kps": e.keypoints, pre + "desc": e.descriptors, pre + "Tcw": Tcw, pre + "cam": cam,
                       pre + "kf_kps": kfk, pre + "geometry": g, pre + "mp_desc": mpd, pre + "mp_state": st,
                       pre + "claimed": cl})
        for k, (th, od, ori) in enumerate(((10.0, 100, True), (3.0, 50, False))):
            nm, match = R.search_by_projection_kf(e.keypoints, e.descriptors, 640, 480, Tcw, cam, kfk, geom, mpd, st,
                                                  th, od, ori, cl)
            arrays[pre + f"nm_{k}"] = np.array(nm)
            arrays[pre + f"match_{k}"] = match
    save("reloc_search.npz", **arrays)


def triangulation_fixture(R):
    # 15. ORBmatcher::SearchForTriangulation on two scene pairs (F12 from the
    # pair's homography and a random epipole)
    import tempfile
    voc = syn.vocabulary(10, 4, 5)
    s, _ = pyoracle.scale_tables(8, 1.2)
    scale = np.array(s, np.float32)
    sigma2 = (scale * scale).astype(np.float32)
    arrays = {"scale": scale, "sigma2": sigma2}
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "voc.txt")
        syn.write_vocabulary_text(voc, path)
        R.vocabulary_load(path)
        for sc in range(2):
            f1, f2, H = syn.frame_pair(640, 480, 80 + sc)
            a, b = R.extract(f1, nfeatures=1500), R.extract(f2, nfeatures=1500)
            fa, fb = R.bow_transform(path, a.descriptors, 2), R.bow_transform(path, b.descriptors, 2)
            Cw1, T2, K2, F12, mp1, mp2, ur1, ur2 = syn.triangulation_case(H, len(a.keypoints), len(b.keypoints), sc)
            pre = f"s{sc}_"
            arrays.update({pre + "kps1": a.keypoints, pre + "desc1": a.descriptors, pre + "kps2": b.keypoints,
                           pre + "desc2": b.descriptors, pre + "mp1": mp1, pre + "mp2": mp2, pre + "ur1": ur1,
                           pre + "ur2": ur2, pre + "Cw1": Cw1, pre + "T2": T2, pre + "K2": K2, pre + "F12": F12})
            for side, fv in (("1", fa), ("2", fb)):
                for key in ("fv_nodes", "fv_offsets", "fv_features"):
                    arrays[pre + key + side] = fv[key]
            for k, (st, ori) in enumerate(((False, True), (True, False))):
                nm, match = R.search_for_triangulation(
                    a.keypoints, a.descriptors, mp1, ur1, (fa["fv_nodes"], fa["fv_offsets"], fa["fv_features"]),
                    b.keypoints, b.descriptors, mp2, ur2, (fb["fv_nodes"], fb["fv_offsets"], fb["fv_features"]),
                    Cw1, T2, K2, F12, scale, sigma2, st, ori)
                arrays[pre + f"nm_{k}"] = np.array(nm)
                arrays[pre + f"match_{k}"] = match
    save("triangulation.npz", **arrays)


def sim3_fixture(R):
    # 16. ORBmatcher::SearchByProjection(KeyFrame*, Scw, vpPoints, vpMatched, th)
    from oracle.pyoracle import GEOM_DTYPE
    arrays = {}
    for sc in range(2):
        e = R.extract(syn.scene(640, 480, 95 + sc), nfeatures=1500)
        Scw, cam, g, pd, ps, cl = syn.sim3_case(e.keypoints, e.descriptors, 640, 480, 95 + sc)
        geom = np.ascontiguousarray(g).view(GEOM_DTYPE).reshape(-1)
        pre = f"s{sc}_"
        arrays.update({pre + "kps": e.keypoints, pre + "desc": e.descriptors, pre + "Scw": Scw, pre + "cam": cam,
                       pre + "points": g, pre + "pdesc": pd, pre + "pstate": ps, pre + "claimed": cl})
        for th in (10, 5):
            nm, match = R.search_by_projection_sim3(e.keypoints, e.descriptors, 640, 480, Scw, cam, geom, pd, ps, th,
                                                    cl)
            arrays[pre + f"nm_{th}"] = np.array(nm)
            arrays[pre + f"match_{th}"] = match
    save("sim3_search.npz", **arrays)


def fuse_fixture(R):
    # 17. ORBmatcher::Fuse(KeyFrame*, vpMapPoints, th): each map point's choice
    from oracle.pyoracle import GEOM_DTYPE
    arrays = {}
    for sc in range(2):
        e = R.extract(syn.scene(640, 480, 97 + sc), nfeatures=1500)
        Tcw, cam5, g, pd, ps, ur = syn.fuse_case(e.keypoints, e.descriptors, 97 + sc)
        geom = np.ascontiguousarray(g).view(GEOM_DTYPE).reshape(-1)
        pre = f"s{sc}_"
        arrays.update({pre + "kps": e.keypoints, pre + "desc": e.descriptors, pre + "ur": ur, pre + "Tcw": Tcw,
                       pre + "cam": cam5, pre + "points": g, pre + "pdesc": pd, pre + "pstate": ps})
        for th in (3.0, 5.0):
            nf, target = R.fuse_candidates(e.keypoints, e.descriptors, ur, 640, 480, Tcw, cam5, geom, pd, ps, th)
            arrays[pre + f"nf_{int(th)}"] = np.array(nf)
            arrays[pre + f"target_{int(th)}"] = target
    # Fuse(KeyFrame*, Scw, vpPoints, th, vpReplacePoint)
    for sc in range(2):
        e = R.extract(syn.scene(640, 480, 99 + sc), nfeatures=1500)
        Scw, cam, g, pd, ps, _ = syn.sim3_case(e.keypoints, e.descriptors, 640, 480, 99 + sc)
        geom = np.ascontiguousarray(g).view(GEOM_DTYPE).reshape(-1)
        pre = f"sim3_s{sc}_"
        arrays.update({pre + "kps": e.keypoints, pre + "desc": e.descriptors, pre + "Scw": Scw, pre + "cam": cam,
                       pre + "points": g, pre + "pdesc": pd, pre + "pstate": ps})
        nf, target = R.fuse_sim3_candidates(e.keypoints, e.descriptors, 640, 480, Scw, cam, geom, pd, ps, 4.0)
        arrays[pre + "nf"] = np.array(nf)
        arrays[pre + "target"] = target
    save("fuse.npz", **arrays)


def by_sim3_fixture(R):
    # 18. ORBmatcher::SearchBySim3(pKF1, pKF2, vpMatches12, s12, R12, t12, th):
    # two views of a plane (different poses and feature sets), some
    # vpMatches12 entries already set
    from oracle.pyoracle import GEOM_DTYPE
    arrays = {}
    for sc in range(2):
        img1, img2, geo = syn.sim3_pair_images(110 + sc)
        e1 = R.extract(img1, nfeatures=1500)
        e2 = R.extract(img2, nfeatures=1200)
        T1, T2, s12, R12, t12, cam, g1, d1, st1, g2, d2, st2, pre12 = syn.sim3_pair_case(
            e1.keypoints, e1.descriptors, e2.keypoints, e2.descriptors, geo, 110 + sc)
        G1 = np.ascontiguousarray(g1).view(GEOM_DTYPE).reshape(-1)
        G2 = np.ascontiguousarray(g2).view(GEOM_DTYPE).reshape(-1)
        pre = f"s{sc}_"
        arrays.update({pre + "kps1": e1.keypoints, pre + "desc1": e1.descriptors, pre + "kps2": e2.keypoints,
                       pre + "desc2": e2.descriptors, pre + "T1": T1, pre + "T2": T2, pre + "s12": np.float32(s12),
                       pre + "R12": R12, pre + "t12": t12, pre + "cam": cam, pre + "g1": g1, pre + "d1": d1,
                       pre + "st1": st1, pre + "g2": g2, pre + "d2": d2, pre + "st2": st2, pre + "pre12": pre12})
        for th in (7.5, 3.0):
            nf, m12 = R.search_by_sim3(e1.keypoints, e1.descriptors, e2.keypoints, e2.descriptors, 640, 480, T1, T2,
                                       s12, R12, t12, cam, G1, d1, st1, G2, d2, st2, th, pre12=pre12)
            arrays[pre + f"nf_{th}"] = np.array(nf)
            arrays[pre + f"match_{th}"] = m12
    save("search_by_sim3.npz", **arrays)


if __name__ == "__main__":
    sel = tuple(sys.argv[1:]) or GROUPS
    bad = [g for g in sel if g not in GROUPS]
    if bad:
        raise SystemExit(f"unknown fixture groups {bad}; known: {GROUPS}")
    main(sel)
