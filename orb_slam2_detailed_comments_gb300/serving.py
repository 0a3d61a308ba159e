"""Continuous-batching serving loop over many camera streams.

Frames arrive per stream (Poisson arrivals); the loop repeatedly takes every
frame that has arrived and is admitted, runs ONE batched extraction over all
of them (orbgpu_batch_extract, graph-replayed) and ONE batched projection
search that matches every frame against its own stream's previous frame
(the previous keypoints act as map points projected with an identity motion
model -- SearchByProjection(Frame&, vector<MapPoint*>, th) semantics,
src/ORBmatcher.cc:72-183).  Requests that arrive while a batch is on the GPU
join the next batch.  Each stream's previous keypoints/descriptors stay
resident on the device; streams are admitted while their resident state fits
an HBM budget.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from ._lib import KEYPOINT_DTYPE
from .batch import BatchExtractor, BatchProjection


@dataclass
class StreamState:
    sid: int
    width: int
    height: int
    nfeatures: int
    resident_bytes: int
    prev_kps: object = None  # (cap, 7) float32 CUDA tensor
    prev_desc: object = None  # (cap, 32) uint8 CUDA tensor
    prev_n: int = 0
    frames: int = 0


@dataclass
class Result:
    sid: int
    arrival: float
    done: float
    nkeypoints: int
    nmatches: int
    keypoints: object = field(default=None, repr=False)
    descriptors: object = field(default=None, repr=False)
    matches: object = field(default=None, repr=False)


class ServingEngine:
    """Admission by HBM budget, per-stream device state, continuous batching."""

    def __init__(self, max_batch: int = 64, max_width: int = 1280, max_height: int = 720, max_nfeatures: int = 2000,
                 hbm_budget_bytes: int = 40 << 30, th: float = 6.0, nnratio: float = 0.8, keep_outputs: bool = False):
        import torch
        self.torch = torch
        self.batch = BatchExtractor(max_batch, max_width, max_height, max_nfeatures)
        self.proj = BatchProjection(self.batch, nnratio)
        self.max_batch = max_batch
        self.cap = self.batch.per_frame_capacity
        self.budget = hbm_budget_bytes
        self.used = 0
        self.th = th
        self.streams: dict[int, StreamState] = {}
        self.keep_outputs = keep_outputs
        self.rejected: list[int] = []

    # ---------------------------------------------------------------- admission
    def stream_bytes(self, w: int, h: int) -> int:
        # previous keypoints + descriptors, staging of one image and its share
        # of the batch arena (pyramid + blurred pyramid, ~2 * 3.1 * w * h)
        return self.cap * (28 + 32) + w * h + int(2 * 3.1 * w * h) + 64 * 1024

    def admit(self, sid: int, width: int, height: int, nfeatures: int) -> bool:
        need = self.stream_bytes(width, height)
        if self.used + need > self.budget:
            self.rejected.append(sid)
            return False
        t = self.torch
        st = StreamState(sid, width, height, nfeatures, need)
        st.prev_kps = t.zeros((self.cap, 7), dtype=t.float32, device="cuda")
        st.prev_desc = t.zeros((self.cap, 32), dtype=t.uint8, device="cuda")
        self.streams[sid] = st
        self.used += need
        return True

    def release(self, sid: int) -> None:
        st = self.streams.pop(sid, None)
        if st:
            self.used -= st.resident_bytes

    # ---------------------------------------------------------------- one batch
    def _mappoints(self, st: StreamState):
        """The previous frame's keypoints as map-point records (device)."""
        t = self.torch
        n = st.prev_n
        rec = t.zeros((n, 8), dtype=t.int32, device="cuda")
        k = st.prev_kps[:n]
        rec[:, 0] = k[:, 0].contiguous().view(t.int32)
        rec[:, 1] = k[:, 1].contiguous().view(t.int32)
        rec[:, 2] = t.full((n,), -1.0, dtype=t.float32, device="cuda").view(t.int32)
        rec[:, 3] = t.ones((n,), dtype=t.float32, device="cuda").view(t.int32)
        rec[:, 4] = k[:, 5].contiguous().view(t.int32)  # octave
        rec[:, 5] = 1  # in view
        return rec, st.prev_desc[:n]

    def run_batch(self, requests):
        """requests: list of (sid, image CUDA tensor, arrival time).  Returns Results."""
        t = self.torch
        imgs = [img for _, img, _ in requests]
        nfs = [self.streams[sid].nfeatures for sid, _, _ in requests]
        kps, desc, counts = self.batch.extract(imgs, nfs)
        # frame-to-previous-frame matching for frames whose stream has a previous frame
        recs, descs, mcount = [], [], []
        for sid, _, _ in requests:
            st = self.streams[sid]
            if st.prev_n > 0:
                r, d = self._mappoints(st)
            else:
                r = t.zeros((0, 8), dtype=t.int32, device="cuda")
                d = t.zeros((0, 32), dtype=t.uint8, device="cuda")
            recs.append(r)
            descs.append(d)
            mcount.append(int(r.shape[0]))
        mp = t.cat(recs).view(t.uint8).contiguous() if sum(mcount) else t.zeros(8 * 4, dtype=t.uint8, device="cuda")
        md = t.cat(descs).contiguous() if sum(mcount) else t.zeros((1, 32), dtype=t.uint8, device="cuda")
        match, nm = self.proj.search(mp, md, mcount, self.th)
        counts_h = counts.cpu().numpy()
        nm_h = nm.cpu().numpy()
        done = time.perf_counter()
        out = []
        for f, (sid, _, arrival) in enumerate(requests):
            st = self.streams[sid]
            n = int(counts_h[f])
            lo = f * self.cap
            st.prev_kps[:n].copy_(kps[lo:lo + n])
            st.prev_desc[:n].copy_(desc[lo:lo + n])
            st.prev_n = n
            st.frames += 1
            r = Result(sid, arrival, done, n, int(nm_h[f]) if mcount[f] else 0)
            if self.keep_outputs:
                r.keypoints = kps[lo:lo + n].cpu().numpy().view(KEYPOINT_DTYPE).reshape(-1)
                r.descriptors = desc[lo:lo + n].cpu().numpy()
                r.matches = match[lo:lo + n].cpu().numpy()
            out.append(r)
        return out

    # ---------------------------------------------------------------- request loop
    def serve(self, arrivals, frames_of, duration_s: float):
        """Replays 'arrivals' (sorted list of (time_s, sid)) in real time for
        duration_s; frames_of(sid, k) gives stream sid's k-th image (CUDA
        tensor).  Returns the list of Results."""
        results = []
        t0 = time.perf_counter()
        i = 0
        pending = []
        next_frame = {sid: 0 for sid in self.streams}
        while True:
            now = time.perf_counter() - t0
            while i < len(arrivals) and arrivals[i][0] <= now:
                ta, sid = arrivals[i]
                if sid in self.streams:
                    pending.append((sid, frames_of(sid, next_frame[sid]), t0 + ta))
                    next_frame[sid] += 1
                i += 1
            if pending:
                # one frame per stream per batch keeps each stream's frames in order
                seen, batch, rest = set(), [], []
                for r in pending:
                    if r[0] in seen or len(batch) >= self.max_batch:
                        rest.append(r)
                    else:
                        seen.add(r[0])
                        batch.append(r)
                pending = rest
                results.extend(self.run_batch(batch))
            elif i >= len(arrivals) or now > duration_s:
                break
            else:
                time.sleep(max(0.0, min(0.0005, arrivals[i][0] - now)))
            if now > duration_s and not pending and i >= len(arrivals):
                break
        return results


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
    lat = np.array([(r.done - r.arrival) * 1e3 for r in results])
    if len(lat) == 0:
        return {"p50_ms": None, "p99_ms": None, "frames": 0}
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "frames": int(len(lat))}
