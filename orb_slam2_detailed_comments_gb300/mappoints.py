"""MapPoint::ComputeDistinctiveDescriptors for many map points at once
(orbgpu_distinctive_descriptors in include/orbgpu.h).

The reference (src/MapPoint.cc:365-447) runs per map point: it reads the
descriptor of every non-bad keyframe in MapPoint::mObservations (a
std::map<KeyFrame*, size_t>, so in that map's order) and keeps the one with
the least median Hamming distance to the others.  Here the observing
keyframes' descriptor matrices form one pool (rows stacked, e.g. the batched
extractor's output left on the device) and each map point's observations are
a list of pool rows; the lists of all map points go to the GPU in CSR form.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import OrbGpuError, check, lib, ptr

BAD_KEYFRAME = -1  # obs_rows entry of an observation whose keyframe is bad
NO_VALID_OBSERVATION = -1  # best_rows value: mDescriptor left unchanged
MALFORMED_LIST = -2  # best_rows value: a row or an offset out of range


def observations_to_csr(observations, keyframe_first_row, keyframe_bad=None):
    """CSR lists of pool rows from per-map-point observation lists.

    observations: one sequence of (keyframe id, feature index) pairs per map
    point, in the order MapPoint::mObservations iterates them.
    keyframe_first_row[k]: the pool row of keyframe k's descriptor 0 (its
    mDescriptors rows are stacked in the pool).  keyframe_bad[k] (optional):
    KeyFrame::isBad(); those observations become BAD_KEYFRAME entries.
    Returns (obs_offsets int32 [m + 1], obs_rows int32 [n_obs]).
    """
    first = np.asarray(keyframe_first_row, np.int64)
    bad = None if keyframe_bad is None else np.asarray(keyframe_bad, bool)
    counts = np.fromiter((len(o) for o in observations), np.int64, count=len(observations))
    offsets = np.zeros(len(observations) + 1, np.int64)
    np.cumsum(counts, out=offsets[1:])
    pairs = np.array([p for o in observations for p in o], np.int64).reshape(-1, 2)
    rows = first[pairs[:, 0]] + pairs[:, 1] if len(pairs) else np.zeros(0, np.int64)
    if bad is not None and len(pairs):
        rows = np.where(bad[pairs[:, 0]], BAD_KEYFRAME, rows)
    if offsets[-1] > np.iinfo(np.int32).max or (len(rows) and rows.max() > np.iinfo(np.int32).max):
        raise ValueError("observation lists exceed 32-bit indexing")
    return offsets.astype(np.int32), rows.astype(np.int32)


def compute_distinctive_descriptors(pool, obs_offsets, obs_rows, descriptors=None, stream=None, validate=True):
    """The distinctive descriptor of every map point of a CSR batch.

    pool: (P, 32) uint8 tensor (CUDA, or page-locked host memory read in
    place); obs_offsets: (m + 1,) int32; obs_rows: (n_obs,) int32, pool rows
    with BAD_KEYFRAME for observations of bad keyframes.  descriptors: an
    optional (m, 32) uint8 tensor, the map points' current mDescriptor, updated
    in place where a descriptor was chosen.  Returns best_rows (m,) int32 on
    the pool's device: the chosen pool row, NO_VALID_OBSERVATION or
    MALFORMED_LIST.  With validate (the default) the call waits for the kernel
    and raises OrbGpuError on a malformed list; without it, it returns at once
    (the result is ready when the stream reaches it).
    """
    import torch
    dev = obs_offsets.device if obs_offsets.is_cuda else torch.device("cuda")
    m = int(obs_offsets.shape[0]) - 1
    if m < 0:
        raise ValueError("obs_offsets needs m + 1 entries")
    for name, t, dt in (("pool", pool, torch.uint8), ("obs_offsets", obs_offsets, torch.int32),
                        ("obs_rows", obs_rows, torch.int32)):
        if t.dtype != dt or not t.is_contiguous():
            raise ValueError(f"{name} must be a contiguous {dt} tensor")
    if pool.dim() != 2 or pool.shape[1] != 32:
        raise ValueError("pool must be (P, 32)")
    if descriptors is not None and (descriptors.dtype != torch.uint8 or tuple(descriptors.shape) != (m, 32)
                                    or not descriptors.is_contiguous()):
        raise ValueError("descriptors must be a contiguous (m, 32) uint8 tensor")
    best = torch.empty(max(m, 1), dtype=torch.int32, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream if stream is None else int(stream)
    check(lib().orbgpu_distinctive_descriptors(ptr(pool), int(pool.shape[0]), ptr(obs_offsets), ptr(obs_rows),
                                               int(obs_rows.shape[0]), m, ptr(best), ptr(descriptors),
                                               C.c_void_p(st)),
          "orbgpu_distinctive_descriptors")
    best = best[:m]
    if validate and m:
        if stream is not None:
            torch.cuda.ExternalStream(st).synchronize()
        bad = int((best == MALFORMED_LIST).sum().item())
        if bad:
            raise OrbGpuError(1, "orbgpu_distinctive_descriptors",
                              f"{bad} malformed observation lists (a row outside [-1, pool rows) or a bad offset)")
    return best
