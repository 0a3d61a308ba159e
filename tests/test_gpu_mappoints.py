"""MapPoint::ComputeDistinctiveDescriptors on the GPU (orbgpu_distinctive_descriptors)
against the oracle and the golden fixtures: chosen rows bit-exact."""
import numpy as np
import pytest

from tests.gpu_util import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return require_gpu()


def run(torch, pool, offsets, rows, initial=None, pinned=False, stream=None):
    from orb_slam2_detailed_comments_gb300 import compute_distinctive_descriptors
    if pinned:
        P = torch.from_numpy(np.ascontiguousarray(pool)).pin_memory()
        O = torch.from_numpy(np.ascontiguousarray(offsets)).pin_memory()
        R = torch.from_numpy(np.ascontiguousarray(rows)).pin_memory()
    else:
        P, O, R = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (pool, offsets, rows))
    D = None if initial is None else torch.from_numpy(np.ascontiguousarray(initial)).cuda()
    best = compute_distinctive_descriptors(P, O, R, D, stream=stream)
    torch.cuda.synchronize()
    return best.cpu().numpy(), None if D is None else D.cpu().numpy()


@pytest.mark.parametrize("case", ["kat", "short", "long", "ties"])
def test_golden(torch, oracle, golden, case):
    g = golden("distinctive.npz")
    pool, offsets, rows, init = (g[f"{case}_{k}"] for k in ("pool", "offsets", "rows", "initial"))
    best, desc = run(torch, pool, offsets, rows, init)
    assert np.array_equal(desc, g[f"{case}_descriptors"])
    ob, _ = oracle.distinctive_descriptors(pool, offsets, rows, init)
    assert np.array_equal(best, ob)


@pytest.mark.parametrize("seed,kw", [
    (1, dict(mean_len=6.0)),
    (2, dict(mean_len=12.0, max_len=32)),          # every lane-group width
    (3, dict(mean_len=60.0, max_len=400)),         # long lists (one warp per map point)
    (4, dict(mean_len=4.0, low_entropy=True, extra_rows=16)),  # equal medians: first in list order
    (5, dict(mean_len=40.0, max_len=100, low_entropy=True, bad_frac=0.5)),
    (6, dict(mean_len=3.0, bad_frac=0.9, empty_frac=0.3)),     # mostly bad keyframes and empty lists
])
def test_vs_oracle(torch, oracle, seed, kw):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    m = 2000 if kw.get("mean_len", 6) > 30 else 50000
    pool, offsets, rows = syn.observation_case(m, seed, **kw)
    init = np.random.default_rng(seed).integers(0, 256, (m, 32), dtype=np.uint8)
    best, desc = run(torch, pool, offsets, rows, init)
    ob, od = oracle.distinctive_descriptors(pool, offsets, rows, init)
    assert np.array_equal(best, ob)
    assert np.array_equal(desc, od)


def test_every_length_up_to_70(torch, oracle):
    """One map point per list length 0..70 (each group width and the long-list path, at its edges)."""
    rng = np.random.default_rng(9)
    lens = np.repeat(np.arange(71), 20)
    offsets = np.zeros(len(lens) + 1, np.int32)
    offsets[1:] = np.cumsum(lens)
    pool = rng.integers(0, 256, (500, 32), dtype=np.uint8) & np.uint8(0x11)
    rows = rng.integers(-1, 500, int(offsets[-1])).astype(np.int32)
    best, _ = run(torch, pool, offsets, rows)
    ob, _ = oracle.distinctive_descriptors(pool, offsets, rows)
    assert np.array_equal(best, ob)


def test_pinned_host_inputs_and_side_stream(torch, oracle):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    pool, offsets, rows = syn.observation_case(20000, 21)
    s = torch.cuda.Stream()
    best, _ = run(torch, pool, offsets, rows, pinned=True, stream=s.cuda_stream)
    ob, _ = oracle.distinctive_descriptors(pool, offsets, rows)
    assert np.array_equal(best, ob)


def test_malformed_lists_and_empty_batch(torch):
    from orb_slam2_detailed_comments_gb300 import OrbGpuError, compute_distinctive_descriptors
    pool = np.zeros((4, 32), np.uint8)
    offsets = np.array([0, 2, 1, 3, 5, 9], np.int32)  # 1: decreasing; 4: beyond the 5 rows
    rows = np.array([0, 1, 2, 4, -2], np.int32)       # 3: rows 4 and -2 outside [-1, 4)
    P, O, R = (torch.from_numpy(a).cuda() for a in (pool, offsets, rows))
    best = compute_distinctive_descriptors(P, O, R, validate=False)
    assert best.cpu().tolist() == [0, -2, 1, -2, -2]
    with pytest.raises(OrbGpuError):
        compute_distinctive_descriptors(P, O, R)
    empty = compute_distinctive_descriptors(P, torch.zeros(1, dtype=torch.int32, device="cuda"), R)
    assert empty.numel() == 0


def test_full_size_sampled_against_oracle(torch, oracle):
    """The 1,000,000-map-point workload: every chosen row is one of its map
    point's valid observations, and a seeded sample of 20,000 map points
    matches the oracle."""
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    m = 1_000_000
    pool, offsets, rows = syn.observation_case(m, 2024, mean_len=6.0, max_len=64)
    best, _ = run(torch, pool, offsets, rows)
    lens = np.diff(offsets)
    owner = np.repeat(np.arange(m), lens)
    hit = np.zeros(m, bool)
    np.logical_or.at(hit, owner, rows == best[owner])
    valid_any = np.zeros(m, bool)
    np.logical_or.at(valid_any, owner, rows >= 0)
    assert np.array_equal(best >= 0, valid_any)
    assert hit[best >= 0].all()
    idx = np.sort(np.random.default_rng(5).choice(m, 20000, replace=False))
    sub_off = np.zeros(len(idx) + 1, np.int32)
    sub_off[1:] = np.cumsum(lens[idx])
    sub_rows = np.concatenate([rows[offsets[i]:offsets[i + 1]] for i in idx]).astype(np.int32)
    ob, _ = oracle.distinctive_descriptors(pool, sub_off, sub_rows)
    assert np.array_equal(best[idx], ob)
