"""Continuous-batching serving loop over many camera streams.

Frames arrive per stream (Poisson arrivals).  A dispatcher forms batches from
every arrived frame whose stream has no frame in flight (at most one frame
per stream per batch, so each stream's frames stay in order) and hands each
batch to a free worker; ``inflight`` workers (host threads, each with its own
batch pipeline, CUDA stream and buffers) run their batches concurrently, so
requests that arrive while others are on the GPU are admitted into the next
batch and its work overlaps on the device with the batches still running.

A batch is one batched extraction (orbgpu_batch_extract, graph-replayed, the
images read in place from page-locked host memory) and TrackWithMotionModel's
search for every frame against its own stream's previous frame --
SearchByProjection(Frame& CurrentFrame, const Frame& LastFrame, th, bMono)
(src/ORBmatcher.cc:1710-1879) as src/Tracking.cc:1321-1353 calls it: empty
CurrentFrame.mvpMapPoints, monocular th 15, the pose predicted by the
constant-velocity model, and a second search with 2 th for the frames whose
first search found fewer than 20 matches.

Each stream's previous keypoints, map points and descriptors stay resident in
the library's stream state store (orbgpu_stream_state_*: one gather kernel
before the search, one update kernel after it, both on the batch's stream).
Streams are admitted while their resident state fits an HBM budget.  The map
points of a frame are its keypoints placed in the world by the stream's depth
source: the synthetic streams view a textured plane Z = depth, so a keypoint's
map point is its ray's intersection with that plane from the frame's pose
(this stands in for the stereo depth or the triangulated map points of a real
tracker).
"""
from __future__ import annotations

import ctypes as C
import queue
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from ._lib import KEYPOINT_DTYPE, MP_OBSERVED, MP_PRESENT, check, lib, ptr
from .batch import BatchExtractor, BatchFrameProjection, motion_struct
from .synthetic import predict_pose

RETRY_BELOW = 20  # src/Tracking.cc:1347: fewer matches than this -> search again with 2 th


@dataclass
class StreamState:
    sid: int
    width: int
    height: int
    nfeatures: int
    resident_bytes: int
    slot: int = 0
    K: tuple = (1.0, 1.0, 0.0, 0.0)  # fx, fy, cx, cy
    depth: float = 1.0
    prev_pose: object = None         # 3 x 4 float32 (LastFrame.mTcw)
    prevprev_pose: object = None
    prev_n: int = 0                  # LastFrame's keypoints (rows of the stream's slot)
    frames: int = 0


@dataclass
class Result:
    sid: int
    arrival: float
    done: float
    nkeypoints: int
    nmatches: int
    retried: bool = False
    error: str | None = None
    batch: int = -1
    keypoints: object = field(default=None, repr=False)
    descriptors: object = field(default=None, repr=False)
    matches: object = field(default=None, repr=False)


class _Worker:
    """One batch pipeline: extractor, two frame searches (first and retry),
    LastFrame staging, device-time events."""

    def __init__(self, engine, idx):
        t = engine.torch
        self.idx = idx
        self.batch = BatchExtractor(engine.max_batch, engine.max_width, engine.max_height, engine.max_nfeatures)
        self.search1 = BatchFrameProjection(self.batch, check_ori=engine.check_ori)
        self.search2 = BatchFrameProjection(self.batch, check_ori=engine.check_ori)
        cap = self.batch.per_frame_capacity
        rows = engine.max_batch * cap
        self.lkps = t.zeros((rows, 7), dtype=t.float32, device="cuda")
        self.lmps = t.zeros((rows, 4), dtype=t.float32, device="cuda")
        self.ldesc = t.zeros((rows, 32), dtype=t.uint8, device="cuda")
        self.rkps = t.zeros((rows, 7), dtype=t.float32, device="cuda")
        self.rmps = t.zeros((rows, 4), dtype=t.float32, device="cuda")
        self.rdesc = t.zeros((rows, 32), dtype=t.uint8, device="cuda")
        # per-batch small arrays: slots, offsets (first search, retry), rays,
        # depths.  Their host sides are ordinary (pageable) memory copied
        # synchronously: torch's page-locked allocator records events on the
        # streams a block was copied on when the block is freed, and the
        # batch's stream belongs to the library, which destroys it first.
        self.h_small = t.zeros(4 * (engine.max_batch + 1), dtype=t.int32)
        self.d_small = t.zeros(4 * (engine.max_batch + 1), dtype=t.int32, device="cuda")
        self.h_geo = t.zeros(13 * engine.max_batch, dtype=t.float64)
        self.d_geo = t.zeros(13 * engine.max_batch, dtype=t.float64, device="cuda")
        self.h_out = t.zeros(2 * engine.max_batch, dtype=t.int32)
        self.stream = t.cuda.ExternalStream(self.batch.stream)
        self.ev_start = t.cuda.Event(enable_timing=True)
        self.ev_end = t.cuda.Event(enable_timing=True)


class ServingEngine:
    """Admission by HBM budget, per-stream device state, continuous batching
    with 'inflight' batches on the device at once."""

    def __init__(self, max_batch: int = 64, max_width: int = 1280, max_height: int = 720, max_nfeatures: int = 2000,
                 hbm_budget_bytes: int = 40 << 30, th: float = 15.0, mono: bool = True, check_ori: bool = True,
                 keep_outputs: bool = False, max_streams: int = 64, inflight: int = 2):
        import torch
        self.torch = torch
        self.max_batch = max_batch
        self.max_width, self.max_height, self.max_nfeatures = max_width, max_height, max_nfeatures
        self.check_ori = check_ori
        self.budget = hbm_budget_bytes
        self.used = 0
        self.th = th
        self.mono = mono
        self.keep_outputs = keep_outputs
        self.streams: dict[int, StreamState] = {}
        self.rejected: list[int] = []
        self.max_streams = max_streams
        self.free_slots = list(range(max_streams))
        self.workers = [_Worker(self, i) for i in range(max(1, inflight))]
        self.cap = self.workers[0].batch.per_frame_capacity
        self._state = C.c_void_p()
        check(lib().orbgpu_stream_state_create(max_streams, self.cap, C.byref(self._state)),
              "orbgpu_stream_state_create")
        self._flags = MP_PRESENT | MP_OBSERVED
        self._lock = threading.Lock()
        self._batches = 0
        self.batch_spans = []  # (batch id, worker, device ms from the serve start: begin, end)
        self._t0_event = None

    def __del__(self):
        st = getattr(self, "_state", None)
        if st is not None and st.value:
            try:
                lib().orbgpu_stream_state_destroy(st)
            except Exception:
                pass
            self._state = None

    # ---------------------------------------------------------------- admission
    def stream_bytes(self, w: int, h: int) -> int:
        # previous keypoints + map points + descriptors, the page-locked image
        # and its share of a batch arena: per level the unblurred and blurred
        # planes and the candidate bit map (~2.2 bytes per level pixel) and
        # the cell and DistributeOctTree buffers (~3.3), over levels summing
        # to ~3.3 w h pixels: ~18 w h
        return self.cap * (28 + 16 + 32) + w * h + 18 * w * h + 64 * 1024

    def admit(self, sid: int, width: int, height: int, nfeatures: int, K=None, depth: float = 8.0) -> bool:
        need = self.stream_bytes(width, height)
        with self._lock:
            if self.used + need > self.budget or not self.free_slots:
                self.rejected.append(sid)
                return False
            if K is None:
                K = (0.9 * width, 0.9 * width, width / 2.0, height / 2.0)
            slot = self.free_slots.pop(0)
            self.streams[sid] = StreamState(sid, width, height, nfeatures, need, slot, tuple(float(v) for v in K),
                                            float(depth))
            self.used += need
        return True

    def release(self, sid: int) -> None:
        """Removes a stream; frames of it that have not been dispatched yet are
        dropped by the serving loop (a frame already on the device finishes,
        its result is discarded)."""
        with self._lock:
            st = self.streams.pop(sid, None)
            if st:
                self.used -= st.resident_bytes
                self.free_slots.append(st.slot)

    def warm(self, width: int, height: int, nfeatures: int, reps: int = 2) -> None:
        """Runs one frame of a configuration through every worker's extraction
        so its plan exists before requests arrive."""
        t = self.torch
        img = t.zeros((height, width), dtype=t.uint8, device="cuda")
        for w in self.workers:
            for _ in range(reps):
                w.batch.extract([img], [nfeatures])

    def valid(self, sid: int, img) -> str | None:
        """Why a request cannot be served (None if it can)."""
        st = self.streams.get(sid)
        if st is None:
            return "stream not admitted"
        h, w = int(img.shape[0]), int(img.shape[1])
        if w < 1 or h < 1 or w > self.max_width or h > self.max_height or (w, h) != (st.width, st.height):
            return f"frame size {w}x{h} not served for this stream"
        if st.nfeatures < 1 or st.nfeatures > self.max_nfeatures:
            return "nFeatures out of range"
        return None

    # ---------------------------------------------------------------- one batch
    def _rays(self, pose, K):
        T = np.asarray(pose, np.float64)
        R, tt = T[:, :3], T[:, 3]
        fx, fy, cx, cy = K
        Kinv = np.array([[1.0 / fx, 0.0, -cx / fx], [0.0, 1.0 / fy, -cy / fy], [0.0, 0.0, 1.0]])
        return np.concatenate([(R.T @ Kinv).reshape(-1), -R.T @ tt])

    def run_batch(self, requests, worker: int = 0):
        """requests: list of (sid, image (page-locked host or CUDA tensor),
        arrival time, true pose 3 x 4), at most one per stream, all valid.
        Runs on worker 'worker''s pipeline and returns Results."""
        t = self.torch
        W = self.workers[worker]
        cap = self.cap
        nb = len(requests)
        with self._lock:
            sts = [self.streams[sid] for sid, _, _, _ in requests]
            bid = self._batches
            self._batches += 1
        slots = [st.slot for st in sts]
        lcount = [st.prev_n for st in sts]
        off1 = np.zeros(nb + 1, np.int32)
        off1[1:] = np.cumsum(lcount)
        hs = W.h_small.numpy()
        hs[:nb] = slots
        hs[nb + 1:2 * nb + 2] = off1
        bs = W.stream
        if self._t0_event is not None:
            W.ev_start.record(bs)
        with t.cuda.stream(bs):
            W.d_small.copy_(W.h_small)
        d_slots = W.d_small[:nb]
        d_off1 = W.d_small[nb + 1:2 * nb + 2]
        # extraction, images read in place from page-locked host memory
        kps, desc, counts = W.batch.extract([img for _, img, _, _ in requests], [st.nfeatures for st in sts],
                                            wait=False)
        # LastFrame rows of every frame, then the first search (th)
        check(lib().orbgpu_stream_state_gather(self._state, nb, ptr(d_slots), ptr(d_off1), max(lcount + [0]),
                                               ptr(W.lkps), ptr(W.lmps), ptr(W.ldesc), C.c_void_p(W.batch.stream)),
              "orbgpu_stream_state_gather")
        ident = np.hstack([np.eye(3), np.zeros((3, 1))])
        motions = [motion_struct(ident, ident, *st.K) if st.prev_pose is None else
                   motion_struct(predict_pose(st.prev_pose, st.prevprev_pose), st.prev_pose, *st.K) for st in sts]
        W.batch.wait()  # the extraction's status; the search below synchronises the stream anyway
        match, nm = W.search1.search(W.lkps, W.lmps.view(t.uint8), W.ldesc, lcount, motions, self.th, self.mono)
        nm_h = nm.cpu().numpy()
        # TrackWithMotionModel's retry: frames below RETRY_BELOW search again with 2 th
        retry = [bool(nm_h[f] < RETRY_BELOW) for f in range(nb)]
        if any(retry):
            lc2 = [lcount[f] if retry[f] else 0 for f in range(nb)]
            off2 = np.zeros(nb + 1, np.int32)
            off2[1:] = np.cumsum(lc2)
            hs[2 * nb + 2:3 * nb + 3] = off2
            with t.cuda.stream(bs):
                W.d_small[2 * nb + 2:3 * nb + 3].copy_(W.h_small[2 * nb + 2:3 * nb + 3])
            check(lib().orbgpu_stream_state_gather(self._state, nb, ptr(d_slots), ptr(W.d_small[2 * nb + 2:]),
                                                   max(lc2 + [0]), ptr(W.rkps), ptr(W.rmps), ptr(W.rdesc),
                                                   C.c_void_p(W.batch.stream)),
                  "orbgpu_stream_state_gather (retry)")
            match2, nm2 = W.search2.search(W.rkps, W.rmps.view(t.uint8), W.rdesc, lc2, motions, 2 * self.th,
                                           self.mono)
            check(lib().orbgpu_serving_retry_select(ptr(match), ptr(nm), ptr(match2), ptr(nm2), cap, nb,
                                                    RETRY_BELOW, C.c_void_p(W.batch.stream)),
                  "orbgpu_serving_retry_select")
        # this batch's keypoints, map points and descriptors become the streams' LastFrames
        geo = W.h_geo.numpy()
        for f, st in enumerate(sts):
            geo[12 * f:12 * f + 12] = self._rays(requests[f][3], st.K)
            geo[12 * nb + f] = st.depth
        with t.cuda.stream(bs):
            W.d_geo[:13 * nb].copy_(W.h_geo[:13 * nb])
        check(lib().orbgpu_stream_state_update(self._state, nb, ptr(d_slots), ptr(kps), ptr(desc), ptr(counts), cap,
                                               ptr(W.d_geo), ptr(W.d_geo[12 * nb:]), self._flags,
                                               C.c_void_p(W.batch.stream)),
              "orbgpu_stream_state_update")
        if self._t0_event is not None:
            W.ev_end.record(bs)
        with t.cuda.stream(bs):
            W.h_out[:nb].copy_(counts[:nb])
            W.h_out[nb:2 * nb].copy_(nm[:nb])
        bs.synchronize()
        done = time.perf_counter()
        if self._t0_event is not None:
            self.batch_spans.append((bid, worker, self._t0_event.elapsed_time(W.ev_start),
                                     self._t0_event.elapsed_time(W.ev_end)))
        ho = W.h_out.numpy()
        out = []
        with self._lock:
            for f, (sid, _, arrival, pose) in enumerate(requests):
                st = sts[f]
                n = int(ho[f])
                st.prev_n = n
                st.prevprev_pose = st.prev_pose
                st.prev_pose = np.asarray(pose, np.float32)
                st.frames += 1
                r = Result(sid, arrival, done, n, int(ho[nb + f]) if lcount[f] else 0, retried=retry[f] and lcount[f] > 0,
                           batch=bid)
                if self.keep_outputs:
                    lo = f * cap
                    r.keypoints = kps[lo:lo + n].cpu().numpy().view(KEYPOINT_DTYPE).reshape(-1)
                    r.descriptors = desc[lo:lo + n].cpu().numpy()
                    r.matches = match[lo:lo + n].cpu().numpy()
                out.append(r)
        return out

    def state_rows(self, sid: int):
        """Copies of the stream's resident LastFrame rows (keypoints, map
        points, descriptors), for tests."""
        st = self.streams[sid]
        k, m, d = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(lib().orbgpu_stream_state_slot(self._state, st.slot, C.byref(k), C.byref(m), C.byref(d)),
              "orbgpu_stream_state_slot")
        n = st.prev_n
        kh = np.zeros(max(n, 1) * 28, np.uint8)
        mh = np.zeros(max(n, 1) * 16, np.uint8)
        dh = np.zeros((max(n, 1), 32), np.uint8)
        if n:
            for dst, src in ((kh, k), (mh, m), (dh, d)):
                check(lib().orbgpu_copy_to_host(ptr(dst), src, C.c_size_t(dst.nbytes)), "orbgpu_copy_to_host")
        return kh[:28 * n], mh[:16 * n], dh[:n]

    # ---------------------------------------------------------------- request loop
    def serve(self, arrivals, frames_of, duration_s: float, release_at=None):
        """Replays 'arrivals' (sorted list of (time_s, sid)) in real time;
        frames_of(sid, k) gives stream sid's k-th (image, true pose 3 x 4) --
        page-locked host tensors are read in place by the extraction.
        release_at: optional {sid: time_s} -- the stream is released then and
        its frames not yet dispatched are dropped.  Returns the Results
        (invalid requests come back with .error set; the others are
        served)."""
        t = self.torch
        self._t0_event = t.cuda.Event(enable_timing=True)
        self._t0_event.record()
        self.batch_spans = []
        results = []
        res_lock = threading.Lock()
        work_q: queue.Queue = queue.Queue()
        free_q: queue.Queue = queue.Queue()
        for w in range(len(self.workers)):
            free_q.put(w)
        inflight_sids = set()
        errors = []

        def worker_loop():
            while True:
                item = work_q.get()
                if item is None:
                    return
                w, batch = item
                try:
                    rs = self.run_batch(batch, worker=w)
                except Exception as e:  # reported, the loop goes on
                    errors.append(repr(e))
                    rs = [Result(sid, arr, time.perf_counter(), 0, 0, error=repr(e)) for sid, _, arr, _ in batch]
                with res_lock:
                    for r in rs:
                        if r.sid in self.streams:  # a stream released meanwhile: result discarded
                            results.append(r)
                        inflight_sids.discard(r.sid)
                free_q.put(w)

        threads = [threading.Thread(target=worker_loop, daemon=True) for _ in self.workers]
        for th in threads:
            th.start()
        t0 = time.perf_counter()
        i = 0
        pending = []
        next_frame = {sid: 0 for sid in self.streams}
        release_at = dict(release_at or {})
        while True:
            now = time.perf_counter() - t0
            for sid, tr in list(release_at.items()):
                if tr <= now:
                    self.release(sid)
                    del release_at[sid]
                    pending = [p for p in pending if p[0] != sid]
            while i < len(arrivals) and arrivals[i][0] <= now:
                ta, sid = arrivals[i]
                if sid in self.streams:
                    img, pose = frames_of(sid, next_frame.get(sid, 0))
                    next_frame[sid] = next_frame.get(sid, 0) + 1
                    why = self.valid(sid, img)
                    if why:
                        with res_lock:
                            results.append(Result(sid, t0 + ta, time.perf_counter(), 0, 0, error=why))
                    else:
                        pending.append((sid, img, t0 + ta, pose))
                i += 1
            dispatched = False
            if pending and not free_q.empty():
                # one frame per stream per batch, none of a stream with a frame in flight
                with res_lock:
                    busy = set(inflight_sids)
                seen, batch, rest = set(), [], []
                for r in pending:
                    if r[0] in seen or r[0] in busy or len(batch) >= self.max_batch:
                        rest.append(r)
                    else:
                        seen.add(r[0])
                        batch.append(r)
                if batch:
                    pending = rest
                    w = free_q.get()
                    with res_lock:
                        inflight_sids.update(seen)
                    work_q.put((w, batch))
                    dispatched = True
            if not dispatched:
                if i >= len(arrivals) and not pending and free_q.qsize() == len(self.workers):
                    break
                nxt = arrivals[i][0] - now if i < len(arrivals) else 0.0002
                time.sleep(max(0.0, min(0.0002, nxt)))
        for _ in threads:
            work_q.put(None)
        for th in threads:
            th.join()
        if errors:
            self.errors = errors
        return results


def pingpong(k: int, n: int) -> int:
    """Index of the k-th request of a stream of n prepared frames replayed
    forwards and backwards (consecutive requests are neighbouring poses)."""
    if n <= 1:
        return 0
    p = k % (2 * n - 2)
    return p if p < n else 2 * n - 2 - p


def poisson_arrivals(nstreams: int, rate_hz: float, duration_s: float, seed: int = 0):
    rng = np.random.default_rng(seed)
    ev = []
    for s in range(nstreams):
        t = rng.exponential(1.0 / rate_hz)
        while t < duration_s:
            ev.append((t, s))
            t += rng.exponential(1.0 / rate_hz)
    ev.sort()
    return ev


def latency_stats(results):
    ok = [r for r in results if r.error is None]
    lat = np.array([(r.done - r.arrival) * 1e3 for r in ok])
    if len(lat) == 0:
        return {"p50_ms": None, "p99_ms": None, "frames": 0}
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "frames": int(len(lat))}


def overlapping_batches(spans) -> int:
    """How many pairs of batches ran on different workers with overlapping
    device time spans (begin, end in ms from the serve start)."""
    n = 0
    for a in range(len(spans)):
        for b in range(a + 1, len(spans)):
            _, wa, sa, ea = spans[a]
            _, wb, sb, eb = spans[b]
            if wa != wb and sa < eb and sb < ea:
                n += 1
    return n
