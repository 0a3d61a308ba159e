"""Batched extraction and projection matching over ragged frame lists
(orbgpu_batch_* in include/orbgpu.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import MEM_DEVICE, check, lib, ptr

STAGES = ("gather", "resize_blur", "fast", "distribute", "describe")


class FrameSet:
    """The argument arrays of one list of images (device or page-locked host
    tensors) and their nFeatures, packed once for repeated extractions of
    the same buffers (their contents may change between calls; the tensors
    must not be resized or freed while the set is used: it holds them)."""

    def __init__(self, images, nfeatures):
        self.images = list(images)
        n = len(self.images)
        self.n = n
        self.ptrs = (C.c_void_p * n)(*[t.data_ptr() for t in self.images])
        self.ws = np.array([t.shape[1] for t in self.images], np.int32)
        self.hs = np.array([t.shape[0] for t in self.images], np.int32)
        self.steps = np.array([t.stride(0) for t in self.images], np.uint64)
        self.nf = np.array(nfeatures, np.int32)
        if len(self.nf) != n:
            raise ValueError("one nFeatures per image")


class BatchExtractor:
    """Extraction of many frames of uneven size per call (device images)."""

    def __init__(self, max_frames: int, max_width: int, max_height: int, max_nfeatures: int,
                 scale_factor: float = 1.2, nlevels: int = 8, ini_th: int = 20, min_th: int = 7, stream=None):
        import torch
        self._h = C.c_void_p()
        st = C.c_void_p(0 if stream is None else int(stream))
        check(lib().orbgpu_batch_create(int(max_frames), int(max_width), int(max_height), int(max_nfeatures), st,
                                        C.byref(self._h)), "orbgpu_batch_create")
        lib().orbgpu_batch_stream.restype = C.c_void_p
        self.scale_factor = scale_factor
        self.nlevels = nlevels
        self.ini_th = ini_th
        self.min_th = min_th
        self.max_frames = max_frames
        self.per_frame_capacity = int(max_nfeatures) + 64 * nlevels + 64
        cap = self.per_frame_capacity
        self.kps = torch.empty((max_frames * cap, 7), dtype=torch.float32, device="cuda")
        self.desc = torch.empty((max_frames * cap, 32), dtype=torch.uint8, device="cuda")
        self.counts = torch.zeros(max_frames, dtype=torch.int32, device="cuda")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            try:
                lib().orbgpu_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return int(lib().orbgpu_batch_stream(self._h) or 0)

    @staticmethod
    def frames(images, nfeatures) -> FrameSet:
        """The argument arrays of 'images' packed once (see FrameSet), for
        extract() calls on the same buffers."""
        return FrameSet(images, nfeatures)

    def extract(self, images, nfeatures=None, wait: bool = True):
        """images: list of 2-D uint8 CUDA tensors (or page-locked host
        tensors read in place) with nfeatures a list of ints, or a FrameSet
        (nfeatures then unused).  Returns (keypoints (F*cap, 7) float32
        records, descriptors (F*cap, 32), counts (F,)) -- frame f's rows start
        at f * per_frame_capacity.  wait=False returns once the work is queued
        on the batch's stream (orbgpu_batch_extract_async); wait() then
        reports its status."""
        fs = images if isinstance(images, FrameSet) else FrameSet(images, nfeatures)
        # the argument arrays only: the images' owner decides how long they
        # live (a page-locked tensor held here past this object's stream
        # would be freed after it)
        self._keep = (fs.ptrs, fs.ws, fs.hs, fs.steps, fs.nf)
        n = fs.n
        fn = lib().orbgpu_batch_extract if wait else lib().orbgpu_batch_extract_async
        check(fn(self._h, n, fs.ptrs, ptr(fs.ws), ptr(fs.hs), ptr(fs.steps), ptr(fs.nf), C.c_float(self.scale_factor),
                 self.nlevels, self.ini_th, self.min_th, ptr(self.kps), ptr(self.desc), self.per_frame_capacity,
                 MEM_DEVICE, ptr(self.counts)),
              "orbgpu_batch_extract" if wait else "orbgpu_batch_extract_async")
        return self.kps[: n * self.per_frame_capacity], self.desc[: n * self.per_frame_capacity], self.counts[:n]

    def wait(self):
        """Synchronises the batch's stream and raises if the last asynchronous
        extraction failed its capacity checks."""
        check(lib().orbgpu_batch_wait(self._h), "orbgpu_batch_wait")

    def stage_times(self) -> dict:
        ms = np.zeros(5, np.float32)
        check(lib().orbgpu_batch_stage_times(self._h, ptr(ms), 5), "orbgpu_batch_stage_times")
        return dict(zip(STAGES, ms.tolist()))

    def launches_per_extract(self) -> int:
        return int(lib().orbgpu_batch_launch_count(self._h))


class BatchProjection:
    """SearchByProjection(Frame&, vector<MapPoint*>, th) for every frame of the
    batch's last extraction."""

    def __init__(self, batch: BatchExtractor, nnratio: float = 0.8):
        import torch
        self.batch = batch
        self.nnratio = nnratio
        self.match = torch.empty(batch.max_frames * batch.per_frame_capacity, dtype=torch.int32, device="cuda")
        self.nm = torch.zeros(batch.max_frames, dtype=torch.int32, device="cuda")

    def search(self, mappoints_u8, mp_descriptors, counts_per_frame, th: float):
        """mappoints_u8: all frames' orbgpu_mappoint records (as uint8 CUDA
        tensor), mp_descriptors: (M, 32) CUDA tensor; counts_per_frame: map
        points per frame.  Returns (match (F*cap,), nmatches (F,))."""
        b = self.batch
        off = np.zeros(len(counts_per_frame) + 1, np.int32)
        off[1:] = np.cumsum(counts_per_frame)
        self._keep = off
        check(lib().orbgpu_batch_search_by_projection(b.handle, ptr(b.kps), ptr(b.desc), ptr(b.counts),
                                                      ptr(mappoints_u8), ptr(mp_descriptors), ptr(off),
                                                      C.c_float(th), C.c_float(self.nnratio), ptr(self.match),
                                                      ptr(self.nm)),
              "orbgpu_batch_search_by_projection")
        n = len(counts_per_frame)
        return self.match[: n * b.per_frame_capacity], self.nm[:n]

    def launches_per_search(self) -> int:
        return int(lib().orbgpu_batch_search_launch_count())

    def rounds(self) -> int:
        """Fixed-point rounds of the slowest frame in the last search."""
        return int(lib().orbgpu_batch_search_rounds())


class BatchStereo:
    """Frame::ComputeStereoMatches (src/Frame.cc:831-1082) for (left, right)
    frame pairs of the batch's last extraction, on its resident pyramids
    (orbgpu_batch_compute_stereo_matches)."""

    def __init__(self, batch: BatchExtractor):
        import torch
        self.batch = batch
        cap = batch.per_frame_capacity
        self.uright = torch.empty(batch.max_frames * cap, dtype=torch.float32, device="cuda")
        self.depth = torch.empty(batch.max_frames * cap, dtype=torch.float32, device="cuda")

    def compute(self, pairs, bf, fx):
        """pairs: [(left frame, right frame)] indices of the last extraction;
        bf / fx: per pair or one value.  Returns (uright, depth) as
        (npairs, per_frame_capacity) CUDA tensors (row p holds the left frame's
        keypoints in order; entries past its count are unspecified)."""
        b = self.batch
        n = len(pairs)
        lf = np.array([p[0] for p in pairs], np.int32)
        rf = np.array([p[1] for p in pairs], np.int32)
        bfa = np.broadcast_to(np.asarray(bf, np.float32), (n,)).copy()
        fxa = np.broadcast_to(np.asarray(fx, np.float32), (n,)).copy()
        check(lib().orbgpu_batch_compute_stereo_matches(b.handle, ptr(b.kps), ptr(b.desc), ptr(b.counts), n, ptr(lf),
                                                        ptr(rf), ptr(bfa), ptr(fxa), ptr(self.uright),
                                                        ptr(self.depth)),
              "orbgpu_batch_compute_stereo_matches")
        cap = b.per_frame_capacity
        return self.uright[: n * cap].view(n, cap), self.depth[: n * cap].view(n, cap)


def motion_struct(Tcw, Tlw, fx, fy, cx, cy, bf=0.0, b=0.0):
    """orbgpu_frame_motion from rows 0-2 of CurrentFrame.mTcw / LastFrame.mTcw."""
    from ._lib import MotionStruct
    m = MotionStruct()
    for i, v in enumerate(np.asarray(Tcw, np.float32).reshape(-1)[:12]):
        m.Tcw[i] = float(v)
    for i, v in enumerate(np.asarray(Tlw, np.float32).reshape(-1)[:12]):
        m.Tlw[i] = float(v)
    m.fx, m.fy, m.cx, m.cy, m.bf, m.b = (float(np.float32(v)) for v in (fx, fy, cx, cy, bf, b))
    return m


class BatchFrameProjection:
    """SearchByProjection(Frame& CurrentFrame, const Frame& LastFrame, th, bMono)
    for every frame of the batch's last extraction, each against its own
    LastFrame (orbgpu_batch_search_by_projection_frame)."""

    def __init__(self, batch: BatchExtractor, check_ori: bool = True):
        import torch
        self.batch = batch
        self.check_ori = check_ori
        self.match = torch.empty(batch.max_frames * batch.per_frame_capacity, dtype=torch.int32, device="cuda")
        self.nm = torch.zeros(batch.max_frames, dtype=torch.int32, device="cuda")

    def search(self, last_kps, last_mps_u8, last_desc, last_counts, motions, th: float, mono: bool):
        """last_kps: (R, 7) float32 CUDA tensor of all frames' LastFrame
        keypoints back to back; last_mps_u8: their orbgpu_frame_mappoint
        records (uint8 CUDA tensor, 16 bytes each); last_desc: (R, 32) CUDA
        tensor of the map points' descriptors; last_counts: rows per frame;
        motions: one motion_struct per frame.  Returns (match (F*cap,),
        nmatches (F,))."""
        from ._lib import MotionStruct
        b = self.batch
        n = len(last_counts)
        off = np.zeros(n + 1, np.int32)
        off[1:] = np.cumsum(last_counts)
        mo = (MotionStruct * n)(*motions)
        self._keep = (off, mo)
        check(lib().orbgpu_batch_search_by_projection_frame(
            b.handle, ptr(b.kps), ptr(b.desc), ptr(b.counts), ptr(last_kps), ptr(last_mps_u8), ptr(last_desc),
            ptr(off), mo, C.c_float(th), int(bool(mono)), int(bool(self.check_ori)), ptr(self.match), ptr(self.nm)),
            "orbgpu_batch_search_by_projection_frame")
        return self.match[: n * b.per_frame_capacity], self.nm[:n]
