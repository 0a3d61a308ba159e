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
    """Admission by HBM budget, per-stream device state, continuous batching.

    Every admitted stream owns a row block of two device arrays that hold its
    previous frame's keypoints and descriptors; after each batch one
    index_copy moves the batch's outputs into the streams' blocks, and the
    next batch's map points are gathered from them with one index_select."""

    def __init__(self, max_batch: int = 64, max_width: int = 1280, max_height: int = 720, max_nfeatures: int = 2000,
                 hbm_budget_bytes: int = 40 << 30, th: float = 6.0, nnratio: float = 0.8, keep_outputs: bool = False,
                 max_streams: int = 64):
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
        self.max_streams = max_streams
        self.free_slots = list(range(max_streams))
        self.slot_of: dict[int, int] = {}
        # previous-frame state of every stream slot, as map point records and descriptors
        self.state_rec = torch.zeros((max_streams * self.cap, 8), dtype=torch.int32, device="cuda")
        self.state_desc = torch.zeros((max_streams * self.cap, 32), dtype=torch.uint8, device="cuda")
        self.prev_n = np.zeros(max_streams, np.int64)
        self._col = torch.arange(self.cap, device="cuda", dtype=torch.int64)
        self._bstream = torch.cuda.ExternalStream(self.batch.stream)

    # ---------------------------------------------------------------- admission
    def stream_bytes(self, w: int, h: int) -> int:
        # previous keypoints (as records) + descriptors, staging of one image and
        # its share of the batch arena (pyramid, blurred pyramid and FAST
        # strength planes, ~3 * 3.1 * w * h)
        return self.cap * (32 + 32) + w * h + int(3 * 3.1 * w * h) + 64 * 1024

    def admit(self, sid: int, width: int, height: int, nfeatures: int) -> bool:
        need = self.stream_bytes(width, height)
        if self.used + need > self.budget or not self.free_slots:
            self.rejected.append(sid)
            return False
        st = StreamState(sid, width, height, nfeatures, need)
        self.streams[sid] = st
        slot = self.free_slots.pop(0)
        self.slot_of[sid] = slot
        self.prev_n[slot] = 0
        self.used += need
        return True

    def release(self, sid: int) -> None:
        st = self.streams.pop(sid, None)
        if st:
            self.used -= st.resident_bytes
            slot = self.slot_of.pop(sid)
            self.free_slots.append(slot)

    def warm(self, width: int, height: int, nfeatures: int, reps: int = 2) -> None:
        """Runs one frame of a configuration through the pipeline so its plan
        exists before requests arrive."""
        t = self.torch
        img = t.zeros((height, width), dtype=t.uint8, device="cuda")
        for _ in range(reps):
            self.batch.extract([img], [nfeatures])

    # ---------------------------------------------------------------- one batch
    def run_batch(self, requests):
        """requests: list of (sid, image CUDA tensor, arrival time), at most one
        per stream.  Returns Results."""
        t = self.torch
        cap = self.cap
        imgs = [img for _, img, _ in requests]
        nfs = [self.streams[sid].nfeatures for sid, _, _ in requests]
        slots = np.array([self.slot_of[sid] for sid, _, _ in requests], np.int64)
        kps, desc, counts = self.batch.extract(imgs, nfs)
        # map points of every frame: its stream's previous keypoints (identity motion)
        mcount = [int(self.prev_n[s]) for s in slots]
        rows = np.concatenate([s * cap + np.arange(n, dtype=np.int64) for s, n in zip(slots, mcount)]) \
            if sum(mcount) else np.zeros(0, np.int64)
        if len(rows):
            ridx = t.from_numpy(rows).to("cuda", non_blocking=True)
            mp = t.index_select(self.state_rec, 0, ridx).view(t.uint8).contiguous()
            md = t.index_select(self.state_desc, 0, ridx).contiguous()
        else:
            mp = t.zeros(32, dtype=t.uint8, device="cuda")
            md = t.zeros((1, 32), dtype=t.uint8, device="cuda")
        # the gathers above run on torch's stream, the search on the batch's
        ev = t.cuda.Event()
        ev.record()
        self._bstream.wait_event(ev)
        match, nm = self.proj.search(mp, md, mcount, self.th)
        # this batch's keypoints become the streams' map point records
        nb = len(requests)
        k = kps[: nb * cap]
        rec = t.empty((nb * cap, 8), dtype=t.int32, device="cuda")
        rec[:, 0:2] = k[:, 0:2].contiguous().view(t.int32)
        rec[:, 2] = -1082130432  # -1.0f: no right coordinate
        rec[:, 3] = 1065353216   # 1.0f: viewing cosine
        rec[:, 4] = k[:, 5].contiguous().view(t.int32)  # octave -> predicted level
        rec[:, 5] = 1
        rec[:, 6:8] = 0
        dst = (t.from_numpy(slots).to("cuda", non_blocking=True)[:, None] * cap + self._col[None, :]).reshape(-1)
        self.state_rec.index_copy_(0, dst, rec)
        self.state_desc.index_copy_(0, dst, desc[: nb * cap])
        counts_h = counts.cpu().numpy()
        nm_h = nm.cpu().numpy()
        done = time.perf_counter()
        out = []
        for f, (sid, _, arrival) in enumerate(requests):
            st = self.streams[sid]
            n = int(counts_h[f])
            self.prev_n[slots[f]] = n
            st.frames += 1
            r = Result(sid, arrival, done, n, int(nm_h[f]) if mcount[f] else 0)
            if self.keep_outputs:
                lo = f * cap
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
            elif i >= len(arrivals):
                break
            else:
                time.sleep(max(0.0, min(0.0002, arrivals[i][0] - now)))
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
