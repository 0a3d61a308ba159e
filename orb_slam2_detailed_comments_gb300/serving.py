"""Continuous-batching serving loop over many camera streams.

Frames arrive per stream (Poisson arrivals); the loop repeatedly takes every
frame that has arrived and is admitted (at most one per stream, so each
stream's frames stay in order), runs ONE batched extraction over all of them
(orbgpu_batch_extract, graph-replayed) and ONE batched frame-to-frame search
that matches every frame against its own stream's previous frame --
SearchByProjection(Frame& CurrentFrame, const Frame& LastFrame, th, bMono)
(src/ORBmatcher.cc:1710-1879) as TrackWithMotionModel calls it
(src/Tracking.cc:1335-1346: empty CurrentFrame.mvpMapPoints, monocular th 15,
the pose predicted by the constant-velocity model).  Requests that arrive
while a batch is on the GPU join the next batch.

Each stream's previous keypoints, map points and descriptors stay resident
on the device in rows of three engine-wide arrays (one gather and one
scatter per batch); streams are admitted while their resident state fits an
HBM budget.  The map points of a frame are its keypoints placed in the world
by the stream's depth source: the synthetic streams view a textured plane
Z = depth, so a keypoint's map point is its ray's intersection with that
plane from the frame's pose (this stands in for the stereo depth or the
triangulated map points of a real tracker).
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from ._lib import KEYPOINT_DTYPE, MP_OBSERVED, MP_PRESENT
from .batch import BatchExtractor, BatchFrameProjection, motion_struct
from .synthetic import predict_pose


@dataclass
class StreamState:
    sid: int
    width: int
    height: int
    nfeatures: int
    resident_bytes: int
    K: tuple = (1.0, 1.0, 0.0, 0.0)  # fx, fy, cx, cy
    depth: float = 1.0
    prev_pose: object = None         # 3 x 4 float32 (LastFrame.mTcw)
    prevprev_pose: object = None
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
                 hbm_budget_bytes: int = 40 << 30, th: float = 15.0, mono: bool = True, check_ori: bool = True,
                 keep_outputs: bool = False, max_streams: int = 64):
        import torch
        self.torch = torch
        self.batch = BatchExtractor(max_batch, max_width, max_height, max_nfeatures)
        self.search = BatchFrameProjection(self.batch, check_ori=check_ori)
        self.max_batch = max_batch
        self.cap = self.batch.per_frame_capacity
        self.budget = hbm_budget_bytes
        self.used = 0
        self.th = th
        self.mono = mono
        self.streams: dict[int, StreamState] = {}
        self.keep_outputs = keep_outputs
        self.rejected: list[int] = []
        self.max_streams = max_streams
        self.free_slots = list(range(max_streams))
        self.slot_of: dict[int, int] = {}
        # previous frame of every stream slot: keypoints, map points, descriptors
        n = max_streams * self.cap
        self.state_kps = torch.zeros((n, 7), dtype=torch.float32, device="cuda")
        self.state_mps = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
        self.state_desc = torch.zeros((n, 32), dtype=torch.uint8, device="cuda")
        self.prev_n = np.zeros(max_streams, np.int64)
        self._col = torch.arange(self.cap, device="cuda", dtype=torch.int64)
        self._bstream = torch.cuda.ExternalStream(self.batch.stream)
        self._flags = float(np.array([MP_PRESENT | MP_OBSERVED], np.int32).view(np.float32)[0])

    # ---------------------------------------------------------------- admission
    def stream_bytes(self, w: int, h: int) -> int:
        # previous keypoints + map points + descriptors, staging of one image
        # and its share of the batch arena (pyramid, blurred pyramid and FAST
        # strength planes, ~3 * 3.1 * w * h)
        return self.cap * (28 + 16 + 32) + w * h + int(3 * 3.1 * w * h) + 64 * 1024

    def admit(self, sid: int, width: int, height: int, nfeatures: int, K=None, depth: float = 8.0) -> bool:
        need = self.stream_bytes(width, height)
        if self.used + need > self.budget or not self.free_slots:
            self.rejected.append(sid)
            return False
        if K is None:
            K = (0.9 * width, 0.9 * width, width / 2.0, height / 2.0)
        st = StreamState(sid, width, height, nfeatures, need, tuple(float(v) for v in K), float(depth))
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
        """Runs one frame of a configuration through the extraction so its
        plan exists before requests arrive."""
        t = self.torch
        img = t.zeros((height, width), dtype=t.uint8, device="cuda")
        for _ in range(reps):
            self.batch.extract([img], [nfeatures])

    # ---------------------------------------------------------------- one batch
    def _plane_mappoints(self, kps, poses, Ks, depths):
        """Map point rows (x, y, z, flags) of the batch's keypoints: each
        keypoint's ray from its frame's pose meets the plane Z = depth.  The
        per-frame ray matrix M = R^T K^-1 and camera centre C = -R^T t come
        from the host; the device does elementwise arithmetic in a fixed
        order, so a frame's map points do not depend on its batch."""
        t = self.torch
        F = len(poses)
        M = np.zeros((F, 3, 3))
        C = np.zeros((F, 3))
        for f, (T, (fx, fy, cx, cy)) in enumerate(zip(poses, Ks)):
            R = np.asarray(T, np.float64)[:, :3]
            Kinv = np.array([[1.0 / fx, 0.0, -cx / fx], [0.0, 1.0 / fy, -cy / fy], [0.0, 0.0, 1.0]])
            M[f] = R.T @ Kinv
            C[f] = -R.T @ np.asarray(T, np.float64)[:, 3]
        Md = t.from_numpy(M).cuda()
        Cd = t.from_numpy(C).cuda()
        dz = t.tensor(depths, dtype=t.float64, device="cuda")
        x = kps[:, 0].reshape(F, 1, self.cap).double()
        y = kps[:, 1].reshape(F, 1, self.cap).double()
        dw = Md[:, :, 0:1] * x + Md[:, :, 1:2] * y + Md[:, :, 2:3]      # (F, 3, cap): ray directions
        lam = (dz[:, None] - Cd[:, 2:3]) / dw[:, 2, :]                  # (F, cap)
        P = Cd[:, :, None] + lam[:, None, :] * dw                        # (F, 3, cap)
        out = t.empty((F, self.cap, 4), dtype=t.float32, device="cuda")
        out[:, :, :3] = P.transpose(1, 2).float()
        out[:, :, 3] = self._flags
        return out.reshape(-1, 4)

    def run_batch(self, requests):
        """requests: list of (sid, image CUDA tensor, arrival time, true pose
        3 x 4), at most one per stream.  Returns Results."""
        t = self.torch
        cap = self.cap
        nb = len(requests)
        sts = [self.streams[sid] for sid, _, _, _ in requests]
        slots = np.array([self.slot_of[sid] for sid, _, _, _ in requests], np.int64)
        kps, desc, counts = self.batch.extract([img for _, img, _, _ in requests], [st.nfeatures for st in sts])
        # LastFrame of every frame: its stream's previous frame
        lcount = [int(self.prev_n[s]) for s in slots]
        rows = np.concatenate([s * cap + np.arange(n, dtype=np.int64) for s, n in zip(slots, lcount)]) \
            if sum(lcount) else np.zeros(1, np.int64)
        ridx = t.from_numpy(rows).to("cuda", non_blocking=True)
        lk = t.index_select(self.state_kps, 0, ridx)
        lm = t.index_select(self.state_mps, 0, ridx)
        ld = t.index_select(self.state_desc, 0, ridx)
        ident = np.hstack([np.eye(3), np.zeros((3, 1))])
        motions = [motion_struct(ident, ident, *st.K) if st.prev_pose is None else
                   motion_struct(predict_pose(st.prev_pose, st.prevprev_pose), st.prev_pose, *st.K) for st in sts]
        # the gathers run on torch's stream, the search on the batch's
        ev = t.cuda.Event()
        ev.record()
        self._bstream.wait_event(ev)
        match, nm = self.search.search(lk, lm.view(t.uint8), ld, lcount, motions, self.th, self.mono)
        # this batch's keypoints, map points and descriptors become the streams' LastFrames
        poses = [p for _, _, _, p in requests]
        Ks = [st.K for st in sts]
        depths = [st.depth for st in sts]
        k = kps[: nb * cap]
        dst = (t.from_numpy(slots).to("cuda", non_blocking=True)[:, None] * cap + self._col[None, :]).reshape(-1)
        self.state_kps.index_copy_(0, dst, k)
        self.state_mps.index_copy_(0, dst, self._plane_mappoints(k, poses, Ks, depths))
        self.state_desc.index_copy_(0, dst, desc[: nb * cap])
        counts_h = counts.cpu().numpy()
        nm_h = nm.cpu().numpy()
        done = time.perf_counter()
        out = []
        for f, (sid, _, arrival, pose) in enumerate(requests):
            st = self.streams[sid]
            n = int(counts_h[f])
            self.prev_n[slots[f]] = n
            st.prevprev_pose = st.prev_pose
            st.prev_pose = np.asarray(pose, np.float32)
            st.frames += 1
            r = Result(sid, arrival, done, n, int(nm_h[f]) if lcount[f] else 0)
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
        duration_s; frames_of(sid, k) gives stream sid's k-th (image CUDA
        tensor, true pose 3 x 4).  Returns the list of Results."""
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
                    img, pose = frames_of(sid, next_frame[sid])
                    pending.append((sid, img, t0 + ta, pose))
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
    lat = np.array([(r.done - r.arrival) * 1e3 for r in results])
    if len(lat) == 0:
        return {"p50_ms": None, "p99_ms": None, "frames": 0}
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "frames": int(len(lat))}
