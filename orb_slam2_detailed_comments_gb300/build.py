"""Build of liborbgpu.so (the CUDA kernels + C ABI) for sm_103a.

    python -m orb_slam2_detailed_comments_gb300.build

Each translation unit is compiled by nvcc in parallel and linked into
``_build/liborbgpu.so`` inside the package.  Float code is compiled with
``-fmad=false`` (device) and ``-ffp-contract=off`` (host) so that no
multiply-add is fused: the reference's float formulas are reproduced bit for
bit.  After linking, the descriptor-angle sin/cos exception table is built
from the host C library (``_build/sincos_exceptions_<machine>_glibc<version>.bin``).
"""
from __future__ import annotations

import concurrent.futures as cf
import ctypes
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "liborbgpu.so")

SOURCES = [
    "orbgpu_extract_kernels.cu",
    "orbgpu_extract.cu",
    "orbgpu_sincos.cu",
    "orbgpu_batch.cu",
    "orbgpu_match.cu",
    "orbgpu_knn.cu",
    "orbgpu_knn_tc.cu",
    "orbgpu_mappoint.cu",
    "orbgpu_geometry.cu",
    "orbgpu_bow.cu",
    "orbgpu_serving.cu",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def flags() -> list[str]:
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O3",
                   "-I" + os.path.join(ROOT, "include"), "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
    srcp = os.path.join(CSRC, src)
    deps = [srcp] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps += [os.path.join(ROOT, "include", h) for h in ("orbgpu.h", "orbgpu_ext.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), *flags(), "-c", srcp, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(table: bool = True, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if table:
        lib = ctypes.CDLL(LIB)
        lib.orbgpu_sincos_table_path.restype = ctypes.c_char_p
        path = lib.orbgpu_sincos_table_path()
        if not os.path.exists(path.decode()):
            lib.orbgpu_build_sincos_table.argtypes = [ctypes.c_char_p, ctypes.c_int]
            rc = lib.orbgpu_build_sincos_table(path, max(1, os.cpu_count() or 1))
            if rc != 0:
                raise RuntimeError(f"sin/cos table build failed: {rc}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
