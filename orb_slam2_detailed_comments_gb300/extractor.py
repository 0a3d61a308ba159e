"""ORBextractor on the GPU, with the reference's interface
(include/ORBextractor.h:93-162)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import KEYPOINT_DTYPE, MEM_DEVICE, MEM_HOST, check, lib, ptr


def _is_cuda(a) -> bool:
    return hasattr(a, "is_cuda") and bool(a.is_cuda)


class ORBextractor:
    """ORB_SLAM2::ORBextractor(nfeatures, scaleFactor, nlevels, iniThFAST, minThFAST).

    ``extractor(image, mask)`` returns ``(keypoints, descriptors)``:
    keypoints as a structured array with cv::KeyPoint's fields and
    descriptors as an N x 32 uint8 array (numpy for a numpy image; torch CUDA
    tensors for a CUDA tensor image, with ``device_out=True``).
    """

    def __init__(self, nfeatures: int, scaleFactor: float, nlevels: int, iniThFAST: int, minThFAST: int,
                 max_width: int = 0, max_height: int = 0, stream=None):
        self._h = C.c_void_p()
        st = C.c_void_p(0 if stream is None else int(stream))
        check(lib().orbgpu_extractor_create(int(nfeatures), C.c_float(scaleFactor), int(nlevels), int(iniThFAST),
                                            int(minThFAST), int(max_width), int(max_height), st, C.byref(self._h)),
              "orbgpu_extractor_create")
        self.nfeatures = nfeatures
        self.nlevels = nlevels
        self._tables = self._read_tables()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            try:
                lib().orbgpu_extractor_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    @property
    def stream(self) -> int:
        return int(lib().orbgpu_extractor_stream(self._h) or 0)

    def _read_tables(self):
        n = C.c_int(0)
        arrs = [np.zeros(16, np.float32) for _ in range(4)] + [np.zeros(16, np.int32)]
        check(lib().orbgpu_extractor_tables(self._h, C.byref(n), *[ptr(a) for a in arrs]), "orbgpu_extractor_tables")
        return [a[:n.value].copy() for a in arrs]

    # include/ORBextractor.h:119-159
    def GetLevels(self) -> int:
        return self.nlevels

    def GetScaleFactor(self) -> float:
        return float(self._tables[0][1]) if self.nlevels > 1 else 1.0

    def GetScaleFactors(self):
        return self._tables[0].copy()

    def GetInverseScaleFactors(self):
        return self._tables[1].copy()

    def GetScaleSigmaSquares(self):
        return self._tables[2].copy()

    def GetInverseScaleSigmaSquares(self):
        return self._tables[3].copy()

    def features_per_level(self):
        return self._tables[4].copy()

    def capacity(self) -> int:
        # DistributeOctTree may return a few more keypoints than requested
        return int(self.nfeatures) + 64 * self.nlevels + 64

    def __call__(self, image, mask=None, device_out: bool = False):
        """ORBextractor::operator()(image, mask, keypoints, descriptors); mask is ignored."""
        cap = self.capacity()
        n = C.c_int(0)
        if _is_cuda(image):
            import torch
            img = image.contiguous()
            h, w = img.shape
            in_mem, step = MEM_DEVICE, img.stride(0)
        else:
            img = np.ascontiguousarray(image, dtype=np.uint8)
            h, w = img.shape
            in_mem, step = MEM_HOST, img.strides[0]
        if device_out:
            import torch
            dev = image.device if _is_cuda(image) else torch.device("cuda")
            kps = torch.empty((cap, 7), dtype=torch.float32, device=dev)
            desc = torch.empty((cap, 32), dtype=torch.uint8, device=dev)
            out_mem = MEM_DEVICE
        else:
            kps = np.zeros(cap, KEYPOINT_DTYPE)
            desc = np.zeros((cap, 32), np.uint8)
            out_mem = MEM_HOST
        rc = lib().orbgpu_extract(self._h, ptr(img), int(w), int(h), C.c_size_t(step), in_mem, ptr(kps), ptr(desc),
                                  cap, out_mem, C.byref(n))
        check(rc, "orbgpu_extract")
        k = n.value
        return kps[:k], desc[:k]

    @property
    def mvImagePyramid(self):
        """The unblurred levels of the last call, as (device_ptr, width, height, pitch)."""
        out = []
        for l in range(self.nlevels):
            p, w, h, pitch = C.c_void_p(), C.c_int(), C.c_int(), C.c_size_t()
            check(lib().orbgpu_extractor_pyramid_level(self._h, l, C.byref(p), C.byref(w), C.byref(h), C.byref(pitch)),
                  "orbgpu_extractor_pyramid_level")
            out.append((p.value, w.value, h.value, pitch.value))
        return out

    def pyramid_numpy(self, blurred: bool = False):
        """Copies of the pyramid (or blurred) levels of the last call, for tests."""
        res = []
        for l, (p, w, h, pitch) in enumerate(self.mvImagePyramid):
            if blurred:
                q = C.c_void_p()
                check(lib().orbgpu_extractor_blurred_level(self._h, l, C.byref(q)), "blurred_level")
                p = q.value
            buf = np.empty((h, pitch), dtype=np.uint8)
            check(lib().orbgpu_copy_to_host(ptr(buf), C.c_void_p(p), C.c_size_t(h * pitch)), "orbgpu_copy_to_host")
            res.append(buf[:, :w].copy())
        return res
