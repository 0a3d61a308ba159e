"""DBoW2 vocabulary transform (Frame::ComputeBoW) on the GPU against the
reference's golden outputs and the oracle: words, weights, nodes,
BowVector doubles and FeatureVector lists bit-exact."""
import numpy as np
import pytest

from tests.gpu_util import require_gpu

pytestmark = pytest.mark.gpu

BOW_VOCABULARIES = {"k10_L3_l1_tfidf": (1, 4), "k6_L4_l2_idf": (2, 4)}


@pytest.fixture(scope="module")
def torch():
    return require_gpu()


def frame_outputs(r, offs, f):
    """One frame's results of Vocabulary.transform in the oracle's layout."""
    o0, o1 = int(offs[f]), int(offs[f + 1])
    nb, nv = int(r["bow_counts"][f]), int(r["fv_counts"][f])
    starts = r["fv_starts"][o0:o0 + nv] - o0
    sizes = r["fv_sizes"][o0:o0 + nv]
    kept = int(sizes.sum())
    return {"word": r["word"][o0:o1], "weight": r["weight"][o0:o1], "node": r["node"][o0:o1],
            "bow_words": r["bow_words"][o0:o0 + nb], "bow_values": r["bow_values"][o0:o0 + nb],
            "fv_nodes": r["fv_nodes"][o0:o0 + nv], "fv_offsets": np.append(starts, kept).astype(np.int32),
            "fv_features": r["fv_features"][o0:o0 + kept]}


def run(torch, voc, descs, levelsup, pinned=False):
    offs = np.zeros(len(descs) + 1, np.int32)
    offs[1:] = np.cumsum([len(d) for d in descs])
    D = torch.from_numpy(np.ascontiguousarray(np.concatenate(descs).reshape(-1, 32)))
    D = D.pin_memory() if pinned else D.cuda()
    O = torch.from_numpy(offs).cuda()
    r = voc.transform(D, O, levelsup)
    torch.cuda.synchronize()
    host = {k: v.cpu().numpy() for k, v in r.items()}
    return [frame_outputs(host, offs, f) for f in range(len(descs))], host


def assert_same(a, b, what):
    for key, val in b.items():
        assert np.array_equal(a[key], val), (what, key)


@pytest.mark.parametrize("name", list(BOW_VOCABULARIES))
@pytest.mark.parametrize("loader", ["text", "arrays"])
def test_golden(torch, golden, tmp_path, name, loader):
    from orb_slam2_detailed_comments_gb300 import Vocabulary
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    g = golden("bow.npz")
    voc = {key: g[f"{name}_{key}"] for key in ("parents", "is_leaf", "descriptors", "weights")}
    voc.update({key: int(g[f"{name}_{key}"]) for key in ("k", "L", "scoring", "weighting")})
    if loader == "text":
        path = str(tmp_path / "voc.txt")
        syn.write_vocabulary_text(voc, path)
        V = Vocabulary(path)
    else:
        V = Vocabulary.from_arrays(voc["k"], voc["L"], voc["scoring"], voc["weighting"], voc["parents"],
                                   voc["is_leaf"], voc["descriptors"], voc["weights"])
    assert V.size() == int(voc["is_leaf"].sum())
    descs = [g[f"{name}_f{fi}_desc"] for fi in range(3)]
    for lu in BOW_VOCABULARIES[name]:
        outs, _ = run(torch, V, descs, lu)
        for fi in range(3):
            ref = {key[len(f"{name}_f{fi}_lu{lu}_"):]: g[key] for key in g.files
                   if key.startswith(f"{name}_f{fi}_lu{lu}_")}
            assert_same(outs[fi], ref, (fi, lu))


def oracle_vocabulary(oracle, tmp_path, voc, tag):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    path = str(tmp_path / f"voc_{tag}.txt")
    syn.write_vocabulary_text(voc, path)
    assert oracle.vocabulary_load(path) == int(voc["is_leaf"].sum())
    return path


def features(voc, n, seed):
    rng = np.random.default_rng(seed)
    leaves = np.nonzero(voc["is_leaf"])[0]
    base = voc["descriptors"][rng.choice(leaves, n)]
    flips = rng.integers(0, 256, base.shape, dtype=np.uint8) & rng.integers(0, 256, base.shape, dtype=np.uint8)
    return base ^ flips


def test_batch_vs_oracle_large_tree(torch, oracle, tmp_path):
    """k 10, L 5 (111,111 nodes), 16 frames of 0-2500 features, levelsup 0-5."""
    from orb_slam2_detailed_comments_gb300 import Vocabulary
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    voc = syn.vocabulary(10, 5, 91)
    path = oracle_vocabulary(oracle, tmp_path, voc, "large")
    V = Vocabulary.from_arrays(10, 5, 0, 0, voc["parents"], voc["is_leaf"], voc["descriptors"], voc["weights"])
    rng = np.random.default_rng(3)
    descs = [features(voc, int(n), 100 + i) for i, n in enumerate(rng.choice([0, 1, 700, 1500, 2500], 16))]
    for lu in (4, 0, 5):
        outs, _ = run(torch, V, descs, lu)
        for f, d in enumerate(descs):
            assert_same(outs[f], oracle.bow_transform(path, d, lu), (f, lu))


@pytest.mark.parametrize("scoring", range(6))
@pytest.mark.parametrize("weighting", range(4))
def test_scoring_and_weighting(torch, oracle, tmp_path, scoring, weighting):
    """Every DBoW2 scoring (normalisation) and weighting rule, levelsup 0-L+1."""
    from orb_slam2_detailed_comments_gb300 import Vocabulary
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    voc = syn.vocabulary(5, 4, 60 + 6 * weighting + scoring, stop_frac=0.1, scoring=scoring, weighting=weighting)
    path = oracle_vocabulary(oracle, tmp_path, voc, f"{scoring}{weighting}")
    V = Vocabulary(path)
    descs = [features(voc, 600, 7), features(voc, 3, 8)]
    for lu in range(0, 6):
        outs, _ = run(torch, V, descs, lu)
        for f, d in enumerate(descs):
            assert_same(outs[f], oracle.bow_transform(path, d, lu), (f, lu))


def test_pinned_descriptors_and_oversized_frame(torch, oracle, tmp_path):
    from orb_slam2_detailed_comments_gb300 import Vocabulary
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    voc = syn.vocabulary(8, 3, 5)
    path = oracle_vocabulary(oracle, tmp_path, voc, "p")
    V = Vocabulary(path)
    descs = [features(voc, 1000, 1), features(voc, 9000, 2), features(voc, 5, 3)]
    outs, host = run(torch, V, descs, 2, pinned=True)
    assert host["bow_counts"][1] == -1 and host["fv_counts"][1] == -1  # more than 8192 features
    for f in (0, 2):
        assert_same(outs[f], oracle.bow_transform(path, descs[f], 2), f)


def test_compute_bow_single_frame(torch, oracle, tmp_path):
    from orb_slam2_detailed_comments_gb300 import Vocabulary
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    voc = syn.vocabulary(10, 3, 9)
    path = oracle_vocabulary(oracle, tmp_path, voc, "s")
    bv, fv = Vocabulary(path).ComputeBoW(torch.from_numpy(features(voc, 800, 4)).cuda(), 1)
    ref = oracle.bow_transform(path, features(voc, 800, 4), 1)
    assert list(bv) == ref["bow_words"].tolist() and list(bv.values()) == ref["bow_values"].tolist()
    assert list(fv) == ref["fv_nodes"].tolist()
    assert sum(fv.values(), []) == ref["fv_features"].tolist()


@pytest.mark.parametrize("check_ori,ratio", [(True, 0.75), (False, 0.75), (True, 0.9)])
def test_search_by_bow_vs_oracle(torch, oracle, check_ori, ratio):
    """SearchByBoW for 8 (keyframe, frame) pairs of 4 scenes in one launch:
    BoW from the GPU transform, matches and counts against the oracle."""
    from oracle import pyoracle
    from orb_slam2_detailed_comments_gb300 import Vocabulary, search_by_bow
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    voc = syn.vocabulary(10, 4, 5)
    oracle.vocabulary_from_arrays("sbb", voc)
    V = Vocabulary.from_arrays(10, 4, 0, 0, voc["parents"], voc["is_leaf"], voc["descriptors"], voc["weights"])
    ents = []
    for seed in range(4):
        f1, f2, _ = syn.frame_pair(640, 480, 40 + seed)
        ents += [oracle.extract(f1, nfeatures=1500), oracle.extract(f2, nfeatures=1500)]
    offs = np.zeros(len(ents) + 1, np.int32)
    offs[1:] = np.cumsum([len(e.keypoints) for e in ents])
    kps = np.concatenate([e.keypoints for e in ents])
    desc = np.concatenate([e.descriptors for e in ents])
    mp = np.random.default_rng(2).choice([0, 1, 1, 1, 2], len(kps)).astype(np.uint8)
    K = torch.from_numpy(kps.view(np.float32).reshape(-1, 7).copy()).cuda()
    D = torch.from_numpy(desc).cuda()
    O = torch.from_numpy(offs).cuda()
    bow = V.transform(D, O, 2)
    # keyframe = even entry, frame = odd entry, both directions
    pairs = [(2 * s, 2 * s + 1) for s in range(4)] + [(2 * s + 1, 2 * s) for s in range(4)]
    nm, matches = search_by_bow(K, D, O, bow, torch.from_numpy(mp).cuda(), pairs, ratio, check_ori)
    torch.cuda.synchronize()
    for p, (a, b) in enumerate(pairs):
        ea, eb = ents[a], ents[b]
        fa = oracle.bow_transform("sbb", ea.descriptors, 2)
        fb = oracle.bow_transform("sbb", eb.descriptors, 2)
        ref_nm, ref = oracle.search_by_bow(ea.keypoints, ea.descriptors, mp[offs[a]:offs[a + 1]],
                                           (fa["fv_nodes"], fa["fv_offsets"], fa["fv_features"]),
                                           eb.keypoints, eb.descriptors,
                                           (fb["fv_nodes"], fb["fv_offsets"], fb["fv_features"]), ratio, check_ori)
        assert int(nm[p]) == ref_nm, p
        assert np.array_equal(matches[p].cpu().numpy(), ref), p
        assert ref_nm > 100


@pytest.mark.parametrize("check_ori,ratio", [(True, 0.75), (False, 0.9)])
def test_search_by_bow_keyframes_vs_oracle(torch, oracle, check_ori, ratio):
    """SearchByBoW(KeyFrame*, KeyFrame*) for 8 keyframe pairs in one launch."""
    from orb_slam2_detailed_comments_gb300 import Vocabulary, search_by_bow
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    voc = syn.vocabulary(10, 4, 5)
    oracle.vocabulary_from_arrays("sbbk", voc)
    V = Vocabulary.from_arrays(10, 4, 0, 0, voc["parents"], voc["is_leaf"], voc["descriptors"], voc["weights"])
    ents = []
    for seed in range(4):
        f1, f2, _ = syn.frame_pair(640, 480, 50 + seed)
        ents += [oracle.extract(f1, nfeatures=1500), oracle.extract(f2, nfeatures=1500)]
    offs = np.zeros(len(ents) + 1, np.int32)
    offs[1:] = np.cumsum([len(e.keypoints) for e in ents])
    kps = np.concatenate([e.keypoints for e in ents])
    desc = np.concatenate([e.descriptors for e in ents])
    mp = np.random.default_rng(4).choice([0, 1, 1, 1, 2], len(kps)).astype(np.uint8)
    K = torch.from_numpy(kps.view(np.float32).reshape(-1, 7).copy()).cuda()
    D = torch.from_numpy(desc).cuda()
    O = torch.from_numpy(offs).cuda()
    bow = V.transform(D, O, 2)
    pairs = [(2 * s, 2 * s + 1) for s in range(4)] + [(2 * s + 1, 2 * s) for s in range(4)]
    nm, matches = search_by_bow(K, D, O, bow, torch.from_numpy(mp).cuda(), pairs, ratio, check_ori, keyframes=True)
    torch.cuda.synchronize()
    for p, (a, b) in enumerate(pairs):
        ea, eb = ents[a], ents[b]
        fa = oracle.bow_transform("sbbk", ea.descriptors, 2)
        fb = oracle.bow_transform("sbbk", eb.descriptors, 2)
        ref_nm, ref = oracle.search_by_bow_kf(ea.keypoints, ea.descriptors, mp[offs[a]:offs[a + 1]],
                                              (fa["fv_nodes"], fa["fv_offsets"], fa["fv_features"]), eb.keypoints,
                                              eb.descriptors, mp[offs[b]:offs[b + 1]],
                                              (fb["fv_nodes"], fb["fv_offsets"], fb["fv_features"]), ratio, check_ori)
        assert int(nm[p]) == ref_nm, p
        assert np.array_equal(matches[p].cpu().numpy(), ref), p
        assert ref_nm > 50


@pytest.mark.parametrize("only_stereo,check_ori", [(False, True), (False, False), (True, True)])
def test_search_for_triangulation_vs_oracle(torch, oracle, only_stereo, check_ori):
    """SearchForTriangulation for 6 keyframe pairs (both directions of 3 scenes)."""
    from oracle import pyoracle
    from orb_slam2_detailed_comments_gb300 import Vocabulary, search_for_triangulation
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    voc = syn.vocabulary(10, 4, 5)
    oracle.vocabulary_from_arrays("tri", voc)
    V = Vocabulary.from_arrays(10, 4, 0, 0, voc["parents"], voc["is_leaf"], voc["descriptors"], voc["weights"])
    ents, Hs = [], []
    for seed in range(3):
        f1, f2, H = syn.frame_pair(640, 480, 60 + seed)
        ents += [oracle.extract(f1, nfeatures=1500), oracle.extract(f2, nfeatures=1500)]
        Hs += [H, np.linalg.inv(H)]
    offs = np.zeros(len(ents) + 1, np.int32)
    offs[1:] = np.cumsum([len(e.keypoints) for e in ents])
    kps = np.concatenate([e.keypoints for e in ents])
    desc = np.concatenate([e.descriptors for e in ents])
    pairs = [(2 * s, 2 * s + 1) for s in range(3)] + [(2 * s + 1, 2 * s) for s in range(3)]
    mp = np.zeros(len(kps), np.uint8)
    ur = np.zeros(len(kps), np.float32)
    geos = []
    for p, (a, b) in enumerate(pairs):
        Cw1, T2, K2, F12, mp1, mp2, ur1, ur2 = syn.triangulation_case(Hs[a], int(offs[a + 1] - offs[a]),
                                                                      int(offs[b + 1] - offs[b]), 500 + p)
        if p < 3:  # map points / stereo flags once per entry
            mp[offs[a]:offs[a + 1]], mp[offs[b]:offs[b + 1]] = mp1, mp2
            ur[offs[a]:offs[a + 1]], ur[offs[b]:offs[b + 1]] = ur1, ur2
        geos.append((Cw1, T2, K2, F12))
    s, _ = pyoracle.scale_tables(8, 1.2)
    scale = np.array(s, np.float32)
    sigma2 = scale * scale
    K = torch.from_numpy(kps.view(np.float32).reshape(-1, 7).copy()).cuda()
    D = torch.from_numpy(desc).cuda()
    O = torch.from_numpy(offs).cuda()
    bow = V.transform(D, O, 2)
    nm, matches = search_for_triangulation(K, D, O, bow, torch.from_numpy(mp).cuda(), torch.from_numpy(ur).cuda(),
                                           pairs, geos, scale, sigma2, only_stereo, check_ori)
    torch.cuda.synchronize()
    total = 0
    for p, (a, b) in enumerate(pairs):
        fa = oracle.bow_transform("tri", ents[a].descriptors, 2)
        fb = oracle.bow_transform("tri", ents[b].descriptors, 2)
        Cw1, T2, K2, F12 = geos[p]
        ref_nm, ref = oracle.search_for_triangulation(
            ents[a].keypoints, ents[a].descriptors, mp[offs[a]:offs[a + 1]], ur[offs[a]:offs[a + 1]],
            (fa["fv_nodes"], fa["fv_offsets"], fa["fv_features"]), ents[b].keypoints, ents[b].descriptors,
            mp[offs[b]:offs[b + 1]], ur[offs[b]:offs[b + 1]], (fb["fv_nodes"], fb["fv_offsets"], fb["fv_features"]),
            Cw1, T2, K2, F12, scale, sigma2, only_stereo, check_ori)
        assert int(nm[p]) == ref_nm, p
        assert np.array_equal(matches[p].cpu().numpy(), ref), p
        total += ref_nm
    assert total > 30
