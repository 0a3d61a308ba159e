"""Frame::isInFrustum for the local map points of many frames at once
(orbgpu_is_in_frustum in include/orbgpu.h).

Tracking::SearchLocalPoints (src/Tracking.cc) runs Frame::isInFrustum
(src/Frame.cc:491-578) on every local map point and hands the ones in view to
ORBmatcher::SearchByProjection.  Here one launch tests the map points of a
batch of frames and writes the records (MAPPOINT_DTYPE) that the projection
searches read, so the local-map search stays on the device.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import FRUSTUM_FRAME_DTYPE, MAPPOINT_GEOMETRY_DTYPE, check, lib, ptr


def frustum_frame(Tcw, fx, fy, cx, cy, bf, min_x, max_x, min_y, max_y, scale_factor=1.2, nlevels=8):
    """One FRUSTUM_FRAME_DTYPE record from rows 0-2 of the frame's mTcw, the
    camera constants (Frame::fx, fy, cx, cy, mbf), the image bounds (mnMinX,
    mnMaxX, mnMinY, mnMaxY) and the extractor's scale factor and levels.  The
    pose matrices and the level thresholds of MapPoint::PredictScale are
    computed by the library on the host."""
    rec = np.zeros(1, FRUSTUM_FRAME_DTYPE)
    T = np.ascontiguousarray(np.asarray(Tcw, np.float32).reshape(-1)[:12])
    f32 = [C.c_float(float(np.float32(v))) for v in (fx, fy, cx, cy, bf, min_x, max_x, min_y, max_y, scale_factor)]
    check(lib().orbgpu_frustum_frame_init(ptr(T), *f32, int(nlevels), ptr(rec)), "orbgpu_frustum_frame_init")
    return rec[0]


def is_in_frustum(frames, mp_offsets, geometry, mappoints, viewing_cos_limit=0.5, in_view=None, stream=None):
    """Frame::isInFrustum(pMP, viewingCosLimit) for every map point of a batch.

    frames: (nframes,) FRUSTUM_FRAME_DTYPE records as a uint8 tensor view or a
    numpy array (copied to the device); mp_offsets: (nframes + 1,) int32 tensor,
    frame f owning map points [mp_offsets[f], mp_offsets[f + 1]); geometry:
    (n, 8) float32 tensor of MAPPOINT_GEOMETRY_DTYPE rows; mappoints: (n, 8)
    float32-sized records (MAPPOINT_DTYPE, e.g. the tensor handed to the batched
    projection search) updated in place as the reference updates the MapPoint
    fields.  in_view: optional (nframes,) int32 tensor, map points in view per
    frame.  Asynchronous on the current stream.
    """
    import torch
    if isinstance(frames, np.ndarray):
        frames = torch.from_numpy(np.ascontiguousarray(frames, FRUSTUM_FRAME_DTYPE).view(np.uint8)).to("cuda")
    nframes = int(mp_offsets.shape[0]) - 1
    if frames.numel() != nframes * FRUSTUM_FRAME_DTYPE.itemsize:
        raise ValueError("frames must hold nframes FRUSTUM_FRAME_DTYPE records")
    for name, t in (("mp_offsets", mp_offsets), ("geometry", geometry), ("mappoints", mappoints)):
        if not t.is_contiguous():
            raise ValueError(f"{name} must be contiguous")
    if geometry.numel() * geometry.element_size() != int(geometry.shape[0]) * MAPPOINT_GEOMETRY_DTYPE.itemsize:
        raise ValueError("geometry must be (n, 8) float32")
    st = torch.cuda.current_stream().cuda_stream if stream is None else int(stream)
    check(lib().orbgpu_is_in_frustum(ptr(frames), nframes, ptr(mp_offsets), ptr(geometry),
                                     C.c_float(viewing_cos_limit), ptr(mappoints), ptr(in_view), C.c_void_p(st)),
          "orbgpu_is_in_frustum")
    return in_view


def undistort_keypoints(keypoints, K4, dist, out=None, stream=None):
    """Frame::UndistortKeyPoints (src/Frame.cc:724-776) for the keypoints of
    one camera: keypoints an (n, 7) float32 tensor of KEYPOINT_DTYPE records
    (device, or page-locked host memory); K4 = fx, fy, cx, cy; dist = k1 k2
    p1 p2 [k3].  Returns out (a new device tensor unless given; may be the
    input) with x, y undistorted.  Asynchronous on the current stream."""
    import torch
    n = int(keypoints.shape[0])
    if keypoints.dtype != torch.float32 or keypoints.dim() != 2 or keypoints.shape[1] != 7 \
            or not keypoints.is_contiguous():
        raise ValueError("keypoints must be a contiguous (n, 7) float32 tensor")
    if out is None:
        out = torch.empty((max(n, 1), 7), dtype=torch.float32, device="cuda")[:n]
    K = np.ascontiguousarray(K4, np.float32)
    d = np.ascontiguousarray(dist, np.float32)
    st = torch.cuda.current_stream().cuda_stream if stream is None else int(stream)
    check(lib().orbgpu_undistort_keypoints(ptr(keypoints), n, ptr(K), ptr(d), len(d), ptr(out), C.c_void_p(st)),
          "orbgpu_undistort_keypoints")
    return out


def compute_image_bounds(cols, rows, K4, dist):
    """Frame::ComputeImageBounds (src/Frame.cc:778-819): (mnMinX, mnMaxX,
    mnMinY, mnMaxY) of a cols x rows image."""
    K = np.ascontiguousarray(K4, np.float32)
    d = np.ascontiguousarray(dist, np.float32)
    b = np.zeros(4, np.float32)
    check(lib().orbgpu_compute_image_bounds(int(cols), int(rows), ptr(K), ptr(d), len(d), ptr(b)),
          "orbgpu_compute_image_bounds")
    return b
