"""ctypes binding of liborbgpu.so (the C ABI declared in include/orbgpu.h)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liborbgpu.so")

KEYPOINT_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("size", "<f4"), ("angle", "<f4"), ("response", "<f4"),
                           ("octave", "<i4"), ("class_id", "<i4")])
MAPPOINT_DTYPE = np.dtype([("proj_x", "<f4"), ("proj_y", "<f4"), ("proj_xr", "<f4"), ("view_cos", "<f4"),
                           ("track_scale_level", "<i4"), ("track_in_view", "<i4"), ("bad", "<i4"), ("pad", "<i4")])

FRAME_MAPPOINT_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("flags", "<i4")])
# orbgpu_mappoint_geometry: the map point fields Frame::isInFrustum reads
MAPPOINT_GEOMETRY_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("nx", "<f4"), ("ny", "<f4"),
                                    ("nz", "<f4"), ("min_distance", "<f4"), ("max_distance", "<f4")])
# orbgpu_frustum_frame (filled by orbgpu_frustum_frame_init)
FRUSTUM_FRAME_DTYPE = np.dtype([("Rcw", "<f4", 9), ("tcw", "<f4", 3), ("Ow", "<f4", 3), ("fx", "<f4"), ("fy", "<f4"),
                                ("cx", "<f4"), ("cy", "<f4"), ("bf", "<f4"), ("min_x", "<f4"), ("max_x", "<f4"),
                                ("min_y", "<f4"), ("max_y", "<f4"), ("nlevels", "<i4"), ("level_above", "<f4", 15)])
MP_PRESENT, MP_OUTLIER, MP_OBSERVED = 1, 2, 4

MEM_HOST = 0
MEM_DEVICE = 1

STATUS = {0: "OK", 1: "BAD_ARG", 2: "OOM", 3: "CUDA", 4: "TIMEOUT", 5: "CAPACITY"}


class OrbGpuError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        super().__init__(f"{where}: {STATUS.get(code, code)} {detail}".strip())


class FrameStruct(C.Structure):
    _fields_ = [("keypoints", C.c_void_p), ("descriptors", C.c_void_p), ("uright", C.c_void_p), ("n", C.c_int),
                ("width", C.c_int), ("height", C.c_int), ("nlevels", C.c_int), ("scale_factors", C.c_float * 16),
                ("mem", C.c_int)]


class MotionStruct(C.Structure):
    """orbgpu_frame_motion: rows 0-2 of CurrentFrame.mTcw and LastFrame.mTcw,
    fx, fy, cx, cy, mbf, mb."""
    _fields_ = [("Tcw", C.c_float * 12), ("Tlw", C.c_float * 12), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float), ("bf", C.c_float), ("b", C.c_float)]


_lib = None


def lib() -> C.CDLL:
    """The loaded library; raises if it was not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OrbGpuError(3, "liborbgpu.so", f"not built: run orb_slam2_detailed_comments_gb300.build ({LIB_PATH})")
        L = C.CDLL(LIB_PATH)
        L.orbgpu_last_error.restype = C.c_char_p
        L.orbgpu_extractor_stream.restype = C.c_void_p
        _lib = L
    return _lib


def check(rc: int, where: str) -> None:
    if rc != 0:
        raise OrbGpuError(rc, where, lib().orbgpu_last_error().decode(errors="replace"))


def ptr(a) -> C.c_void_p:
    """Raw pointer of a numpy array or a torch tensor (host or device)."""
    if a is None:
        return C.c_void_p(0)
    if isinstance(a, np.ndarray):
        return C.c_void_p(a.ctypes.data)
    return C.c_void_p(a.data_ptr())
