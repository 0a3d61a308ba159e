"""GPU extraction through the C ABI against the oracle and the golden fixtures."""
import numpy as np
import pytest

from oracle import pyoracle
from tests.gpu_util import assert_kps_equal, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    return require_gpu()


def extractor(nf, w=0, h=0):
    from orb_slam2_detailed_comments_gb300 import ORBextractor
    return ORBextractor(nf, 1.2, 8, 20, 7, w, h)


def test_golden_640x480(torch, golden):
    g = golden("extract_640x480.npz")
    ex = extractor(1000)
    kps, desc = ex(g["image"])
    assert_kps_equal(kps, g["keypoints"], "keypoints")
    assert np.array_equal(desc, g["descriptors"])
    levels = ex.pyramid_numpy()
    assert [l.shape for l in levels] == [tuple(s) for s in g["level_shapes"]]
    assert [int(l.astype(np.int64).sum()) for l in levels] == list(g["level_sums"])
    assert np.array_equal(levels[7], g["level7"])


@pytest.mark.parametrize("w,h,nf,seed", [(640, 480, 1000, 1), (752, 480, 1500, 2), (1241, 376, 2000, 3),
                                         (1280, 720, 2000, 4), (320, 240, 500, 5), (1024, 768, 3000, 6)])
def test_vs_oracle(torch, oracle, w, h, nf, seed):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    img = syn.scene(w, h, seed)
    ex = extractor(nf)
    kps, desc = ex(img)
    ref = oracle.extract(img, nfeatures=nf)
    levels = ex.pyramid_numpy()
    for l, (a, b) in enumerate(zip(levels, ref.pyramid)):
        assert a.shape == b.shape and np.array_equal(a, b), f"pyramid level {l}"
    blurred = ex.pyramid_numpy(blurred=True)
    for l, (a, b) in enumerate(zip(blurred, ref.pyramid)):
        bb = np.zeros_like(b)
        oracle.lib.orc_blur_level(b.ctypes.data_as(pyoracle.C.c_void_p), b.shape[1], b.shape[0],
                                  bb.ctypes.data_as(pyoracle.C.c_void_p))
        assert np.array_equal(a, bb), f"blurred level {l}"
    assert_kps_equal(kps, ref.keypoints, f"{w}x{h}")
    assert np.array_equal(desc, ref.descriptors)


def test_repeated_calls_and_sizes(torch, oracle):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    ex = extractor(1000)
    for seed, (w, h) in enumerate([(640, 480), (320, 240), (640, 480), (800, 600)]):
        img = syn.scene(w, h, 50 + seed)
        kps, desc = ex(img)
        ref = oracle.extract(img, nfeatures=1000)
        assert_kps_equal(kps, ref.keypoints)
        assert np.array_equal(desc, ref.descriptors)


def test_device_in_device_out(torch, oracle):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    img = syn.scene(640, 480, 9)
    ex = extractor(1000)
    t = torch.from_numpy(img).cuda()
    kps, desc = ex(t, device_out=True)
    ref = oracle.extract(img, nfeatures=1000)
    k = kps.cpu().numpy().view(pyoracle.KP_DTYPE).reshape(-1)
    assert_kps_equal(k, ref.keypoints)
    assert np.array_equal(desc.cpu().numpy(), ref.descriptors)


def test_edge_cases(torch):
    from orb_slam2_detailed_comments_gb300 import OrbGpuError
    ex = extractor(1000)
    kps, desc = ex(np.full((480, 640), 77, np.uint8))
    assert len(kps) == 0 and desc.shape == (0, 32)
    kps, desc = ex(np.zeros((0, 0), np.uint8))
    assert len(kps) == 0
    # portrait images make DistributeOctTree index an empty vector in the reference
    with pytest.raises(OrbGpuError):
        ex(np.zeros((800, 200), np.uint8))
    # a capacity that is too small is reported, not truncated
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    import ctypes as C
    from orb_slam2_detailed_comments_gb300._lib import KEYPOINT_DTYPE, lib, ptr
    img = syn.scene(640, 480, 3)
    k = np.zeros(10, KEYPOINT_DTYPE)
    d = np.zeros((10, 32), np.uint8)
    n = C.c_int(0)
    rc = lib().orbgpu_extract(ex.handle, ptr(img), 640, 480, C.c_size_t(640), 0, ptr(k), ptr(d), 10, 0, C.byref(n))
    assert rc == 5 and n.value > 10


def test_descriptor_rotation_matches_host_libm(torch, oracle):
    """cos/sin of the descriptor angle equal the host C library's cosf/sinf."""
    import ctypes as C
    from orb_slam2_detailed_comments_gb300._lib import lib, ptr
    rng = np.random.default_rng(0)
    hi = np.float32(360.0) * np.float32(np.pi / 180.0)
    xs = [rng.uniform(0, hi, 1 << 22).astype(np.float32),
          rng.uniform(0, 1e-3, 1 << 20).astype(np.float32),
          np.arange(0, 1 << 20, dtype=np.uint32).view(np.float32)]
    # every input the rotation of a keypoint at an integer-moment angle can take near 0, 90, 180, 270 degrees
    x = np.ascontiguousarray(np.concatenate(xs))
    xd = torch.from_numpy(x).cuda()
    c = torch.empty_like(xd)
    s = torch.empty_like(xd)
    assert lib().orbgpu_descriptor_sincos(ptr(xd), len(x), ptr(c), ptr(s)) == 0
    hc = np.zeros_like(x)
    hs = np.zeros_like(x)
    oracle.lib.orc_sincos_table(x.ctypes.data_as(C.c_void_p), len(x), hc.ctypes.data_as(C.c_void_p),
                                hs.ctypes.data_as(C.c_void_p))
    assert np.array_equal(c.cpu().numpy().view(np.uint32), hc.view(np.uint32))
    assert np.array_equal(s.cpu().numpy().view(np.uint32), hs.view(np.uint32))


def check_fast_levels(torch, oracle, img, nf):
    """Per level, the GPU's per-cell FAST output (in cell order, retry
    threshold applied) equals the oracle's cell loop on the same pyramid
    level, and every candidate's score is its arc strength - 1."""
    import ctypes as C
    from orb_slam2_detailed_comments_gb300._lib import lib, ptr
    ex = extractor(nf)
    ex(img)
    levels = ex.pyramid_numpy()
    fn = oracle.fn("fast_level")
    for lvl, li in enumerate(levels):
        h, w = li.shape
        cap = 200000
        ref = np.zeros(cap, pyoracle.KP_DTYPE)
        nref = fn(np.ascontiguousarray(li).ctypes.data_as(C.c_void_p), w, h, 20, 7, ref.ctypes.data_as(C.c_void_p), cap)
        ref = ref[:nref]
        geom = np.zeros(8, np.int32)
        assert lib().orbgpu_extractor_debug_level(ex.handle, lvl, 3, ptr(geom), C.c_size_t(geom.nbytes)) == 0
        ncols, nrows, _, _, cell_cap = (int(v) for v in geom[:5])
        counts = np.zeros(ncols * nrows, np.int32)
        slots = np.zeros(ncols * nrows * cell_cap, np.uint32)
        assert lib().orbgpu_extractor_debug_level(ex.handle, lvl, 0, ptr(counts), C.c_size_t(counts.nbytes)) == 0
        assert lib().orbgpu_extractor_debug_level(ex.handle, lvl, 1, ptr(slots), C.c_size_t(slots.nbytes)) == 0
        got = np.concatenate([slots[c * cell_cap: c * cell_cap + counts[c]] for c in range(len(counts))])
        gx = (got & 0xFFF).astype(np.int64) - 16
        gy = ((got >> 12) & 0xFFF).astype(np.int64) - 16
        gs = (got >> 24).astype(np.int64)
        assert len(got) == nref, lvl
        assert np.array_equal(gx, ref["x"].astype(np.int64)), lvl
        assert np.array_equal(gy, ref["y"].astype(np.int64)), lvl
        assert np.array_equal(gs, ref["response"].astype(np.int64)), lvl
        # arc strengths of the whole level at the threshold each cell used
        dimg = torch.from_numpy(li).cuda()
        smap = torch.empty((h, w), dtype=torch.uint8, device="cuda")
        assert lib().orbgpu_debug_fast_strength(ptr(dimg), w, w, h, 7, ptr(smap)) == 0
        sm = smap.cpu().numpy().astype(np.int64)
        assert np.array_equal(sm[gy + 16, gx + 16] - 1, gs), lvl


def test_fast_stage_per_level(torch, oracle):
    """The detector stage alone on a textured scene."""
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    check_fast_levels(torch, oracle, syn.scene(1241, 376, 77), 2000)


def dense_textures():
    """Images whose cells hold far more FAST candidates than one listing batch
    (256) and, for the noise, more corners than a cell's corner list holds
    (about 900 candidates and 350 corners per 31 x 32 cell at threshold 7)."""
    rng = np.random.default_rng(5)
    noise = rng.integers(0, 256, (480, 640)).astype(np.uint8)
    yy, xx = np.indices((376, 1241))
    checker = ((((yy + xx) // 2) % 2) * 200 + rng.integers(0, 40, (376, 1241))).astype(np.uint8)
    return [("noise", noise), ("checker", checker)]


@pytest.mark.parametrize("name", ["noise", "checker"])
def test_fast_stage_dense_texture(torch, oracle, name):
    """Cells past the candidate batch and the corner list: the detector stage
    and the whole extraction equal the oracle's."""
    img = dict(dense_textures())[name]
    check_fast_levels(torch, oracle, img, 2000)
    kps, desc = extractor(2000)(img)
    ref = oracle.extract(img, nfeatures=2000)
    assert_kps_equal(kps, ref.keypoints, name)
    assert np.array_equal(desc, ref.descriptors)


def test_batch_dense_texture(torch, oracle):
    """A batch that mixes dense textures with scenes (the cell kernel's chunks
    go to whichever warp is free) equals the oracle frame by frame."""
    from orb_slam2_detailed_comments_gb300._lib import KEYPOINT_DTYPE
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    fr = [(img, 2000) for _, img in dense_textures()] + [(syn.scene(1280, 720, 41), 2000), (syn.scene(640, 480, 42), 1000)]
    b = BatchExtractor(len(fr), 1280, 720, 2000)
    cap = b.per_frame_capacity
    for _ in range(2):
        k, d, c = b.extract([torch.from_numpy(img).cuda() for img, _ in fr], [nf for _, nf in fr])
    k = k.cpu().numpy().view(KEYPOINT_DTYPE).reshape(len(fr), cap)
    d = d.cpu().numpy().reshape(len(fr), cap, 32)
    c = c.cpu().numpy()
    for f, (img, nf) in enumerate(fr):
        ref = oracle.extract(img, nfeatures=nf, want_pyramid=False)
        n = len(ref.keypoints)
        assert c[f] == n, f"frame {f}"
        assert_kps_equal(k[f, :n], ref.keypoints, f"frame {f}")
        assert np.array_equal(d[f, :n], ref.descriptors), f"frame {f}"


# scale factor (2.5: the resize's source span exceeds the 8-byte fast path),
# level count, iniThFAST / minThFAST (swapped, and zero: the one-pass cell
# suppression's threshold rule)
PARAMS = [(2.5, 4, 20, 7), (1.5, 6, 7, 20), (1.2, 8, 20, 0), (1.2, 3, 0, 0)]


@pytest.mark.parametrize("scale,nlevels,ini,mn", PARAMS)
def test_extractor_parameters_vs_oracle(torch, oracle, scale, nlevels, ini, mn):
    from orb_slam2_detailed_comments_gb300 import ORBextractor
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    for w, h, seed in [(640, 480, 21), (1241, 376, 22)]:
        img = syn.scene(w, h, seed)
        ex = ORBextractor(1000, scale, nlevels, ini, mn)
        kps, desc = ex(img)
        ref = oracle.extract(img, nfeatures=1000, scale_factor=scale, nlevels=nlevels, ini_th=ini, min_th=mn)
        levels = ex.pyramid_numpy()
        for l, (a, b) in enumerate(zip(levels, ref.pyramid)):
            assert a.shape == b.shape and np.array_equal(a, b), f"{w}x{h} pyramid level {l}"
        assert_kps_equal(kps, ref.keypoints, f"{w}x{h} scale {scale} th {ini}/{mn}")
        assert np.array_equal(desc, ref.descriptors)


@pytest.mark.parametrize("scale,nlevels,ini,mn", PARAMS)
def test_batch_parameters_vs_oracle(torch, oracle, scale, nlevels, ini, mn):
    from orb_slam2_detailed_comments_gb300._lib import KEYPOINT_DTYPE
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    fr = [(syn.scene(640, 480, 31), 1000), (syn.scene(1241, 376, 32), 1500), (syn.scene(320, 240, 33), 500)]
    b = BatchExtractor(4, 1280, 720, 2000, scale_factor=scale, nlevels=nlevels, ini_th=ini, min_th=mn)
    cap = b.per_frame_capacity
    k, d, c = b.extract([torch.from_numpy(img).cuda() for img, _ in fr], [nf for _, nf in fr])
    k = k.cpu().numpy().view(KEYPOINT_DTYPE).reshape(len(fr), cap)
    d = d.cpu().numpy().reshape(len(fr), cap, 32)
    c = c.cpu().numpy()
    for f, (img, nf) in enumerate(fr):
        ref = oracle.extract(img, nfeatures=nf, scale_factor=scale, nlevels=nlevels, ini_th=ini, min_th=mn,
                             want_pyramid=False)
        assert c[f] == len(ref.keypoints), f"frame {f}"
        assert_kps_equal(k[f, :c[f]], ref.keypoints, f"frame {f}")
        assert np.array_equal(d[f, :c[f]], ref.descriptors)
