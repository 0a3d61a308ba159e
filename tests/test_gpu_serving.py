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


def test_alone_equals_mixed(torch):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    from orb_slam2_detailed_comments_gb300.serving import ServingEngine
    nfr = 4
    frames = {s: [torch.from_numpy(f).cuda() for f in syn.stream_frames(w, h, 100 + s, nfr)]
              for s, (w, h, _) in enumerate(STREAMS)}
    mixed = ServingEngine(max_batch=8, keep_outputs=True)
    for s, (w, h, nf) in enumerate(STREAMS):
        assert mixed.admit(s, w, h, nf)
    got = {}
    for k in range(nfr):
        # a mixed batch: every stream's k-th frame, in a rotating order
        order = [(s + k) % len(STREAMS) for s in range(len(STREAMS))]
        for r in mixed.run_batch([(s, frames[s][k], 0.0) for s in order]):
            got[(r.sid, k)] = r
    for s, (w, h, nf) in enumerate(STREAMS):
        alone = ServingEngine(max_batch=1, keep_outputs=True)
        assert alone.admit(s, w, h, nf)
        for k in range(nfr):
            (r,) = alone.run_batch([(s, frames[s][k], 0.0)])
            m = got[(s, k)]
            assert r.nkeypoints == m.nkeypoints and r.nmatches == m.nmatches, (s, k)
            assert r.keypoints.tobytes() == m.keypoints.tobytes()
            assert np.array_equal(r.descriptors, m.descriptors)
            assert np.array_equal(r.matches, m.matches)
            if k > 0:
                assert r.nmatches > 0.2 * r.nkeypoints  # consecutive frames of a slow drift match


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
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    from orb_slam2_detailed_comments_gb300.serving import ServingEngine, latency_stats, poisson_arrivals
    e = ServingEngine(max_batch=16)
    frames = {}
    for s, (w, h, nf) in enumerate(STREAMS * 2):
        assert e.admit(s, w, h, nf)
        frames[s] = [torch.from_numpy(f).cuda() for f in syn.stream_frames(w, h, 300 + s, 3)]
    arr = poisson_arrivals(len(frames), 30.0, 0.5, seed=1)
    res = e.serve(arr, lambda s, k: frames[s][k % 3], 0.5)
    st = latency_stats(res)
    assert st["frames"] == len(arr)
    assert st["p99_ms"] is not None and st["p99_ms"] < 1000.0
