"""Serving loop: admission by HBM budget, per-stream device state, and the
same result for a frame whether it is served alone or in a mixed batch."""
import numpy as np
import pytest

from tests.gpu_util import require_gpu

pytestmark = pytest.mark.gpu

STREAMS = [(640, 480, 1000), (1241, 376, 2000), (1280, 720, 1500), (752, 480, 1000), (640, 480, 2000)]


@pytest.fixture(scope="module")
def torch():
    return require_gpu()


def stream(torch, s, w, h, n, seed0=100):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    frames, poses, K, depth = syn.camera_stream(w, h, seed0 + s, n)
    return [torch.from_numpy(f).cuda() for f in frames], poses, K, depth


def test_alone_equals_mixed(torch):
    from orb_slam2_detailed_comments_gb300.serving import ServingEngine
    nfr = 4
    data = {s: stream(torch, s, w, h, nfr) for s, (w, h, _) in enumerate(STREAMS)}
    mixed = ServingEngine(max_batch=8, keep_outputs=True)
    for s, (w, h, nf) in enumerate(STREAMS):
        assert mixed.admit(s, w, h, nf, K=data[s][2], depth=data[s][3])
    got = {}
    for k in range(nfr):
        # a mixed batch: every stream's k-th frame, in a rotating order
        order = [(s + k) % len(STREAMS) for s in range(len(STREAMS))]
        for r in mixed.run_batch([(s, data[s][0][k], 0.0, data[s][1][k]) for s in order]):
            got[(r.sid, k)] = r
    for s, (w, h, nf) in enumerate(STREAMS):
        alone = ServingEngine(max_batch=1, keep_outputs=True)
        assert alone.admit(s, w, h, nf, K=data[s][2], depth=data[s][3])
        for k in range(nfr):
            (r,) = alone.run_batch([(s, data[s][0][k], 0.0, data[s][1][k])])
            m = got[(s, k)]
            assert r.nkeypoints == m.nkeypoints and r.nmatches == m.nmatches, (s, k)
            assert r.keypoints.tobytes() == m.keypoints.tobytes()
            assert np.array_equal(r.descriptors, m.descriptors)
            assert np.array_equal(r.matches, m.matches)
            if k > 0:
                assert r.nmatches > 0.2 * r.nkeypoints  # neighbouring views of the plane match


def test_frame_search_equals_oracle(torch, oracle):
    """The engine's frame-to-frame search of one stream equals the oracle's
    SearchByProjection(CurrentFrame, LastFrame) on the same keypoints, map
    points (the engine's resident rows) and predicted pose."""
    from oracle import pyoracle
    from orb_slam2_detailed_comments_gb300 import FRAME_MAPPOINT_DTYPE
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    from orb_slam2_detailed_comments_gb300.serving import ServingEngine
    w, h, nf = 1280, 720, 2000
    imgs, poses, K, depth = stream(torch, 7, w, h, 3, seed0=500)
    e = ServingEngine(max_batch=2, keep_outputs=True)
    assert e.admit(0, w, h, nf, K=K, depth=depth)
    prev = None
    for k in range(3):
        _, mrows, _ = e.state_rows(0)
        last_mps = mrows.view(FRAME_MAPPOINT_DTYPE).reshape(-1)
        (cur,) = e.run_batch([(0, imgs[k], 0.0, poses[k])])
        if k > 0:
            T = syn.predict_pose(poses[k - 1], poses[k - 2] if k >= 2 else None)
            mo = pyoracle.make_motion(T, poses[k - 1], *K, 0.0, 0.0)
            nm, match = oracle.search_by_projection_frame(cur.keypoints, cur.descriptors, w, h, prev.keypoints,
                                                          last_mps, prev.descriptors, mo, th=15.0, mono=True,
                                                          check_ori=True)
            assert nm == cur.nmatches, k
            assert np.array_equal(match, cur.matches), k
            assert nm > 0.3 * len(cur.keypoints)
        prev = cur


def test_admission_budget(torch):
    from orb_slam2_detailed_comments_gb300.serving import ServingEngine
    e = ServingEngine(max_batch=4)
    need = e.stream_bytes(1280, 720)
    e.budget = 2 * need + 1
    assert e.admit(0, 1280, 720, 2000)
    assert e.admit(1, 1280, 720, 2000)
    assert not e.admit(2, 1280, 720, 2000)
    e.release(0)
    assert e.admit(2, 1280, 720, 2000)
    assert e.rejected == [2]


def test_serve_loop_latency(torch):
    from orb_slam2_detailed_comments_gb300.serving import ServingEngine, latency_stats, pingpong, poisson_arrivals
    e = ServingEngine(max_batch=16)
    data = {}
    for s, (w, h, nf) in enumerate(STREAMS * 2):
        data[s] = stream(torch, s, w, h, 3, seed0=300)
        assert e.admit(s, w, h, nf, K=data[s][2], depth=data[s][3])
    arr = poisson_arrivals(len(data), 30.0, 0.5, seed=1)
    res = e.serve(arr, lambda s, k: (data[s][0][pingpong(k, 3)], data[s][1][pingpong(k, 3)]), 0.5)
    st = latency_stats(res)
    assert st["frames"] == len(arr)
    assert st["p99_ms"] is not None and st["p99_ms"] < 1000.0


def test_batches_overlap_and_results_match_alone(torch):
    """Two workers: batches run concurrently on the device (their event spans
    overlap) and every served frame equals the same stream served alone."""
    from orb_slam2_detailed_comments_gb300.serving import ServingEngine, overlapping_batches, pingpong, poisson_arrivals
    nfr = 3
    data = {s: stream(torch, s, w, h, nfr, seed0=900) for s, (w, h, _) in enumerate(STREAMS * 3)}
    pinned = {s: ([f.cpu().pin_memory() for f in d[0]], d[1]) for s, d in data.items()}
    e = ServingEngine(max_batch=4, keep_outputs=True, inflight=2)
    for s, (w, h, nf) in enumerate(STREAMS * 3):
        assert e.admit(s, w, h, nf, K=data[s][2], depth=data[s][3])
    # offered far above the engine's rate: batches queue and overlap
    arr = poisson_arrivals(len(data), 400.0, 0.05, seed=3)
    seen = {}

    def frames_of(s, k):
        seen.setdefault(s, []).append(pingpong(k, nfr))
        i = pingpong(k, nfr)
        return pinned[s][0][i], pinned[s][1][i]
    res = e.serve(arr, frames_of, 0.05)
    assert all(r.error is None for r in res)
    assert len(res) == len(arr)
    assert overlapping_batches(e.batch_spans) > 0, e.batch_spans
    by_sid = {}
    for r in sorted(res, key=lambda r: (r.sid, r.arrival)):
        by_sid.setdefault(r.sid, []).append(r)
    for s, rs in list(by_sid.items())[:5]:
        w, h, nf = (STREAMS * 3)[s]
        alone = ServingEngine(max_batch=1, keep_outputs=True, inflight=1)
        assert alone.admit(s, w, h, nf, K=data[s][2], depth=data[s][3])
        for r, i in zip(rs, seen[s]):
            (a,) = alone.run_batch([(s, data[s][0][i], 0.0, data[s][1][i])])
            assert a.nkeypoints == r.nkeypoints and a.nmatches == r.nmatches, (s, i)
            assert a.keypoints.tobytes() == r.keypoints.tobytes()
            assert np.array_equal(a.descriptors, r.descriptors)
            assert np.array_equal(a.matches, r.matches)


def test_bad_frame_release_and_retry(torch):
    """Host-side failure cases of the serving loop: a frame of the wrong size
    fails alone (the others are served and equal their alone results); a
    stream released while it has pending frames loses them and the others are
    unaffected; a frame with fewer than 20 first-search matches is searched
    again with 2 th (src/Tracking.cc:1347-1353)."""
    from orb_slam2_detailed_comments_gb300.serving import ServingEngine, pingpong
    nfr = 3
    data = {s: stream(torch, s, w, h, nfr, seed0=700) for s, (w, h, _) in enumerate(STREAMS)}
    e = ServingEngine(max_batch=8, keep_outputs=True, inflight=2)
    for s, (w, h, nf) in enumerate(STREAMS):
        assert e.admit(s, w, h, nf, K=data[s][2], depth=data[s][3])
    bad = torch.zeros((17, 23), dtype=torch.uint8)
    arr = [(0.001 * k, s) for k in range(6) for s in range(len(STREAMS))]

    def frames_of(s, k):
        if s == 1 and k == 2:
            return bad, data[s][1][0]
        i = pingpong(k, nfr)
        return data[s][0][i], data[s][1][i]
    res = e.serve(arr, frames_of, 0.01, release_at={4: 0.0025})
    errs = [r for r in res if r.error]
    assert len(errs) == 1 and errs[0].sid == 1
    assert all(r.sid != 4 for r in res if r.arrival - min(x.arrival for x in res) > 0.004)
    served = {s: len([r for r in res if r.sid == s and r.error is None]) for s in range(len(STREAMS))}
    assert served[0] == served[2] == served[3] == 6 and served[1] == 5
    # a stream whose next frame has next to no texture (a flat image with one
    # small patch of the scene): fewer than 20 first-pass matches, so the
    # second search (2 th) decides, as the reference's retry does; a frame
    # with enough matches is not searched again
    r0 = ServingEngine(max_batch=1, keep_outputs=True, inflight=1)
    w, h, nf = STREAMS[0]
    assert r0.admit(0, w, h, nf, K=data[0][2], depth=data[0][3])
    (a,) = r0.run_batch([(0, data[0][0][0], 0.0, data[0][1][0])])
    (b_,) = r0.run_batch([(0, data[0][0][1], 0.0, data[0][1][1])])
    flat = torch.full_like(data[0][0][2], 128)
    flat[200:240, 300:340] = data[0][0][2][200:240, 300:340]
    (r,) = r0.run_batch([(0, flat, 0.0, data[0][1][2])])
    assert a.nkeypoints > 500 and b_.nmatches >= 20 and not b_.retried
    assert r.retried and r.nmatches < 20


def test_allocation_failure_is_reported_and_recoverable(torch, oracle):
    """A device allocation that fails (injected on the host: the library's
    next allocation reports out-of-memory) makes the call that needed it
    return ORBGPU_ERR_OOM; the same handle works on the next call, with the
    oracle's results.  In the serving loop the batch whose allocation failed
    comes back as errors and the following batches are served."""
    from orb_slam2_detailed_comments_gb300._lib import KEYPOINT_DTYPE, OrbGpuError, lib
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor
    from orb_slam2_detailed_comments_gb300.serving import ServingEngine, pingpong
    scenes = [syn.scene(640, 480, 41), syn.scene(640, 480, 42)]
    imgs = [torch.from_numpy(s_).cuda() for s_ in scenes]
    b = BatchExtractor(2, 1280, 720, 2000)
    assert lib().orbgpu_debug_fail_allocations(1) == 0
    try:
        with pytest.raises(OrbGpuError) as err:
            b.extract(imgs, [1000, 1000])
        assert err.value.code == 2  # ORBGPU_ERR_OOM
    finally:
        lib().orbgpu_debug_fail_allocations(0)
    k, d, c = b.extract(imgs, [1000, 1000])
    cap = b.per_frame_capacity
    k = k.cpu().numpy().view(KEYPOINT_DTYPE).reshape(2, cap)
    for f, img in enumerate(scenes):
        ref = oracle.extract(img, nfeatures=1000)
        assert int(c[f]) == len(ref.keypoints)
        assert k[f, :len(ref.keypoints)].tobytes() == ref.keypoints.tobytes()
    # serving: the first batch's arena allocation fails
    data = {s: stream(torch, s, w, h, 3, seed0=800) for s, (w, h, _) in enumerate(STREAMS[:3])}
    e = ServingEngine(max_batch=4, keep_outputs=False, inflight=1)
    for s, (w, h, nf) in enumerate(STREAMS[:3]):
        assert e.admit(s, w, h, nf, K=data[s][2], depth=data[s][3])
    arr = [(0.004 * k_, s) for k_ in range(4) for s in range(3)]
    lib().orbgpu_debug_fail_allocations(1)
    try:
        res = e.serve(arr, lambda s, k_: (data[s][0][pingpong(k_, 3)], data[s][1][pingpong(k_, 3)]), 0.02)
    finally:
        lib().orbgpu_debug_fail_allocations(0)
    bad = [r for r in res if r.error]
    good = [r for r in res if r.error is None]
    assert len(res) == len(arr) and 1 <= len(bad) <= 3 and all("OOM" in r.error for r in bad)
    assert len(good) == len(arr) - len(bad) and all(r.nkeypoints > 0 for r in good)
