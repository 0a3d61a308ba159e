"""The C ABI without a GPU: the headers compile as plain C, the library
loads, and it exports every function the headers declare."""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", h) for h in ("orbgpu.h", "orbgpu_ext.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(orbgpu_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def library():
    from orb_slam2_detailed_comments_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        if not (os.path.exists("/usr/local/cuda/bin/nvcc") or shutil.which("nvcc")):
            pytest.skip("library not built and no nvcc")
        build.build()
    return _lib.lib()


def test_headers_compile_as_c():
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    for h in HEADERS:
        r = subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-x", "c", h,
                            "-I" + os.path.join(ROOT, "include")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_every_declared_symbol_is_exported(library):
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(library, n)]
    assert not missing, missing


def test_version_and_error_string_without_gpu(library):
    assert library.orbgpu_version() > 0
    library.orbgpu_last_error.restype = C.c_char_p
    assert isinstance(library.orbgpu_last_error(), bytes)


def test_bad_arguments_are_rejected_before_any_device_work(library):
    """Argument checks run on the host: they answer BAD_ARG with or without a GPU."""
    h = C.c_void_p()
    # nfeatures < 0, scale factor <= 1, nlevels out of range
    assert library.orbgpu_extractor_create(-1, C.c_float(1.2), 8, 20, 7, 0, 0, None, C.byref(h)) == 1
    assert library.orbgpu_extractor_create(1000, C.c_float(1.0), 8, 20, 7, 0, 0, None, C.byref(h)) == 1
    assert library.orbgpu_extractor_create(1000, C.c_float(1.2), 0, 20, 7, 0, 0, None, C.byref(h)) == 1
    assert library.orbgpu_knn2(None, None, 1, None, 1, None, None, None, None, 0) == 1
    assert library.orbgpu_knn2_noalloc(None, -1, None, 0, None, None, None, None, None) == 1
    # vocabulary: branching factor out of range, a parent after its child, no file
    assert library.orbgpu_vocabulary_create(21, 6, 0, 0, 1, None, None, None, None, C.byref(h)) == 1
    par = (C.c_int * 2)(0, 5)
    assert library.orbgpu_vocabulary_create(2, 1, 0, 0, 3, par, C.c_void_p(16), C.c_void_p(16), C.c_void_p(16),
                                            C.byref(h)) == 1
    assert library.orbgpu_vocabulary_load_text(b"/nonexistent/voc.txt", C.byref(h)) == 1
    # negative map point count; a pool pointer that is not 16-byte aligned
    assert library.orbgpu_distinctive_descriptors(None, 0, None, None, 0, -1, None, None, None) == 1
    assert library.orbgpu_distinctive_descriptors(C.c_void_p(8), 1, C.c_void_p(16), C.c_void_p(16), 1, 1,
                                                  C.c_void_p(16), None, None) == 1
    assert library.orbgpu_batch_create(0, 640, 480, 1000, None, C.byref(h)) == 1


def test_launch_policies_set_and_get_without_gpu(library):
    """The small-launch policies take exactly their documented values."""
    import ctypes as C
    v = C.c_longlong(-1)
    for name, values in (("describe_task", (0, 8, 16, 32)), ("fast_chunk", (0, 1, 2, 4)), ("strip_rows_small", (0, 8))):
        assert library.orbgpu_tune_get(name.encode(), C.byref(v)) == 0
        old = v.value
        for x in values:
            assert library.orbgpu_tune_set(name.encode(), C.c_longlong(x)) == 0
            assert library.orbgpu_tune_get(name.encode(), C.byref(v)) == 0 and v.value == x
        for bad in (-1, 3, 64):
            assert library.orbgpu_tune_set(name.encode(), C.c_longlong(bad)) != 0
        assert library.orbgpu_tune_set(name.encode(), C.c_longlong(old)) == 0
