"""Batched (ragged, graph-replayed) extraction and projection matching
against the per-frame oracle."""
import numpy as np
import pytest

from oracle import pyoracle
from tests.gpu_util import assert_kps_equal, require_gpu

pytestmark = pytest.mark.gpu

SIZES = [(640, 480), (752, 480), (1241, 376), (1280, 720), (320, 240)]
NF = [1000, 1500, 2000, 500]


@pytest.fixture(scope="module")
def torch():
    return require_gpu()


def frames(seed, n):
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    rng = np.random.default_rng(seed)
    out = []
    for f in range(n):
        w, h = SIZES[rng.integers(0, len(SIZES))]
        out.append((syn.scene(w, h, seed * 100 + f), int(NF[rng.integers(0, len(NF))])))
    return out


def test_batch_extract_vs_oracle(torch, oracle):
    from orb_slam2_detailed_comments_gb300._lib import KEYPOINT_DTYPE
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor
    b = BatchExtractor(16, 1280, 720, 2000)
    cap = b.per_frame_capacity
    for rep, seed in enumerate([1, 1, 2]):  # same list twice (graph replay), then a new list
        fr = frames(seed, 12)
        imgs = [torch.from_numpy(img).cuda() for img, _ in fr]
        if rep == 1:  # same sizes, different pixels: the replayed graph reads the new images
            from orb_slam2_detailed_comments_gb300 import synthetic as syn
            fr = [(syn.scene(img.shape[1], img.shape[0], 999 + i), nf) for i, (img, nf) in enumerate(fr)]
            imgs = [torch.from_numpy(img).cuda() for img, _ in fr]
        k, d, c = b.extract(imgs, [nf for _, nf in fr])
        k = k.cpu().numpy().view(KEYPOINT_DTYPE).reshape(len(fr), cap)
        d = d.cpu().numpy().reshape(len(fr), cap, 32)
        c = c.cpu().numpy()
        for f, (img, nf) in enumerate(fr):
            ref = oracle.extract(img, nfeatures=nf, want_pyramid=False)
            assert c[f] == len(ref.keypoints), f"frame {f}"
            assert_kps_equal(k[f, :c[f]], ref.keypoints, f"frame {f}")
            assert np.array_equal(d[f, :c[f]], ref.descriptors)


def test_frame_set_equals_the_image_list(torch):
    """A FrameSet (the argument arrays packed once) extracts what the image
    list does, also after the buffers' contents change in place."""
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor
    fr = frames(5, 6)
    imgs = [torch.from_numpy(img).cuda() for img, _ in fr]
    nfs = [nf for _, nf in fr]
    b = BatchExtractor(8, 1280, 720, 2000)
    fs = b.frames(imgs, nfs)
    for rep in range(3):
        if rep == 2:  # new pixels in the same buffers
            for i, t in enumerate(imgs):
                t.copy_(torch.from_numpy(syn.scene(t.shape[1], t.shape[0], 700 + i)))
        k1, d1, c1 = (x.clone() for x in b.extract(imgs, nfs))
        k2, d2, c2 = b.extract(fs)
        assert torch.equal(c1, c2)
        for f in range(len(imgs)):
            n, o = int(c1[f]), f * b.per_frame_capacity
            # records compared bit for bit (class_id -1 reads as a float NaN)
            assert torch.equal(k1[o:o + n].view(torch.int32), k2[o:o + n].view(torch.int32))
            assert torch.equal(d1[o:o + n], d2[o:o + n])


def test_batch_projection_vs_oracle(torch, oracle):
    from orb_slam2_detailed_comments_gb300._lib import KEYPOINT_DTYPE, MAPPOINT_DTYPE
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor, BatchProjection
    b = BatchExtractor(8, 1280, 720, 2000)
    cap = b.per_frame_capacity
    fr = frames(5, 6)
    imgs = [torch.from_numpy(img).cuda() for img, _ in fr]
    k, d, c = b.extract(imgs, [nf for _, nf in fr])
    kh = k.cpu().numpy().view(KEYPOINT_DTYPE).reshape(len(fr), cap)
    dh = d.cpu().numpy().reshape(len(fr), cap, 32)
    ch = c.cpu().numpy()
    rng = np.random.default_rng(3)
    mps_all, mpd_all, counts = [], [], []
    for f in range(len(fr)):
        n = int(ch[f])
        M = 3000
        src = rng.integers(0, n, M)
        mpd = dh[f, src] ^ np.packbits(rng.random((M, 256)) < 0.1, axis=1, bitorder="little")
        mps = np.zeros(M, MAPPOINT_DTYPE)
        mps["proj_x"] = kh[f, src]["x"] + rng.normal(0, 2, M)
        mps["proj_y"] = kh[f, src]["y"] + rng.normal(0, 2, M)
        mps["proj_xr"] = -1
        mps["view_cos"] = 1.0
        mps["track_scale_level"] = kh[f, src]["octave"]
        mps["track_in_view"] = 1
        mps_all.append(mps)
        mpd_all.append(mpd)
        counts.append(M)
    from orb_slam2_detailed_comments_gb300._lib import lib
    p = BatchProjection(b, 0.8)
    refs = []
    for f, (img, _) in enumerate(fr):
        n = int(ch[f])
        refs.append(oracle.search_by_projection(kh[f, :n], dh[f, :n], img.shape[1], img.shape[0],
                                                mps_all[f].view(pyoracle.MP_DTYPE), mpd_all[f], th=6.0, nnratio=0.8))
    # both resolutions: frames in shared memory (default) and the global-memory rounds
    for mode, launches in ((0, 5), (1, 17)):
        assert lib().orbgpu_batch_search_mode(mode) == 0
        try:
            match, nm = p.search(torch.from_numpy(np.concatenate(mps_all).view(np.uint8)).cuda(),
                                 torch.from_numpy(np.ascontiguousarray(np.concatenate(mpd_all))).cuda(), counts, 6.0)
            assert p.launches_per_search() == launches
        finally:
            lib().orbgpu_batch_search_mode(0)
        match = match.cpu().numpy().reshape(len(fr), cap)
        nm = nm.cpu().numpy()
        for f in range(len(fr)):
            n = int(ch[f])
            assert nm[f] == refs[f][0], f"mode {mode} frame {f}"
            assert np.array_equal(match[f, :n], refs[f][1]), f"mode {mode} frame {f}"
            assert (match[f, n:] == -3).all()


def test_async_extraction_then_search_matches_the_synchronous_path(torch, oracle):
    """orbgpu_batch_extract_async + the batched search queued behind it on the
    batch's stream give the synchronous path's results; orbgpu_batch_wait
    reports a capacity failure of an asynchronous extraction."""
    import ctypes as C
    from orb_slam2_detailed_comments_gb300._lib import KEYPOINT_DTYPE, lib, ptr
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor
    b = BatchExtractor(8, 1280, 720, 2000)
    cap = b.per_frame_capacity
    fr = frames(9, 5)
    imgs = [torch.from_numpy(img).cuda() for img, _ in fr]
    nfs = [nf for _, nf in fr]
    k, d, c = b.extract(imgs, nfs)
    ref = (k.cpu().numpy().copy(), d.cpu().numpy().copy(), c.cpu().numpy().copy())
    rk = ref[0].view(KEYPOINT_DTYPE).reshape(len(fr), cap)
    rd = ref[1].reshape(len(fr), cap, 32)
    for _ in range(2):  # plain launch, then the captured graph
        k, d, c = b.extract(imgs, nfs, wait=False)
        b.wait()
        assert np.array_equal(c.cpu().numpy(), ref[2])
        kk = k.cpu().numpy().view(KEYPOINT_DTYPE).reshape(len(fr), cap)
        dd = d.cpu().numpy().reshape(len(fr), cap, 32)
        for f in range(len(fr)):
            assert np.array_equal(kk[f, :ref[2][f]], rk[f, :ref[2][f]]), f"frame {f}"
            assert np.array_equal(dd[f, :ref[2][f]], rd[f, :ref[2][f]]), f"frame {f}"
    kh = rk
    for f, (img, nf) in enumerate(fr):
        r = oracle.extract(img, nfeatures=nf, want_pyramid=False)
        assert_kps_equal(kh[f, :ref[2][f]], r.keypoints, f"frame {f}")
    # a per-frame capacity of 10 rows: queued fine, reported by the wait
    n = len(imgs)
    ptrs = (C.c_void_p * n)(*[t.data_ptr() for t in imgs])
    ws = np.array([t.shape[1] for t in imgs], np.int32)
    hs = np.array([t.shape[0] for t in imgs], np.int32)
    st = np.array([t.stride(0) for t in imgs], np.uint64)
    nf = np.array(nfs, np.int32)
    rc = lib().orbgpu_batch_extract_async(b._h, n, ptrs, ptr(ws), ptr(hs), ptr(st), ptr(nf), C.c_float(1.2), 8, 20, 7,
                                          ptr(b.kps), ptr(b.desc), 10, 1, ptr(b.counts))
    assert rc == 0
    assert lib().orbgpu_batch_wait(b._h) == 5
    assert lib().orbgpu_batch_wait(b._h) == 0  # reported once


def test_pinned_host_images_read_in_place(torch):
    """Page-locked host images (and map points) go straight into the batch
    calls: the same keypoints, descriptors and matches as device copies."""
    from orb_slam2_detailed_comments_gb300._lib import KEYPOINT_DTYPE, MAPPOINT_DTYPE
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor, BatchProjection
    b = BatchExtractor(6, 1280, 720, 2000)
    cap = b.per_frame_capacity
    fr = frames(13, 4)
    nfs = [nf for _, nf in fr]
    dev = [torch.from_numpy(img).cuda() for img, _ in fr]
    host = [torch.from_numpy(img).pin_memory() for img, _ in fr]
    k, d, c = b.extract(dev, nfs)
    ref = (k.cpu().numpy().view(KEYPOINT_DTYPE).reshape(len(fr), cap), d.cpu().numpy().reshape(len(fr), cap, 32),
           c.cpu().numpy().copy())
    rng = np.random.default_rng(2)
    mps, mpd, counts = [], [], []
    for f in range(len(fr)):
        n = int(ref[2][f])
        src = rng.integers(0, n, 500)
        m = np.zeros(500, MAPPOINT_DTYPE)
        m["proj_x"] = ref[0][f, src]["x"] + rng.normal(0, 2, 500)
        m["proj_y"] = ref[0][f, src]["y"] + rng.normal(0, 2, 500)
        m["proj_xr"] = -1
        m["view_cos"] = 1.0
        m["track_scale_level"] = ref[0][f, src]["octave"]
        m["track_in_view"] = 1
        mps.append(m)
        mpd.append(ref[1][f, src] ^ np.packbits(rng.random((500, 256)) < 0.1, axis=1, bitorder="little"))
        counts.append(500)
    mps_b = np.concatenate(mps).view(np.uint8)
    mpd_b = np.ascontiguousarray(np.concatenate(mpd))
    p = BatchProjection(b, 0.8)
    m_dev, nm_dev = p.search(torch.from_numpy(mps_b).cuda(), torch.from_numpy(mpd_b).cuda(), counts, 6.0)
    m_dev, nm_dev = m_dev.cpu().numpy().copy(), nm_dev.cpu().numpy().copy()
    k, d, c = b.extract(host, nfs, wait=False)
    m_h, nm_h = p.search(torch.from_numpy(mps_b).pin_memory(), torch.from_numpy(mpd_b).pin_memory(), counts, 6.0)
    b.wait()
    assert np.array_equal(c.cpu().numpy(), ref[2])
    kk = k.cpu().numpy().view(KEYPOINT_DTYPE).reshape(len(fr), cap)
    dd = d.cpu().numpy().reshape(len(fr), cap, 32)
    for f in range(len(fr)):
        n = int(ref[2][f])
        assert np.array_equal(kk[f, :n], ref[0][f, :n]) and np.array_equal(dd[f, :n], ref[1][f, :n]), f"frame {f}"
    assert np.array_equal(nm_h.cpu().numpy(), nm_dev)
    assert np.array_equal(m_h.cpu().numpy(), m_dev)


@pytest.mark.parametrize("where", ["device", "pinned"])
def test_strided_images_at_every_row_alignment(torch, oracle, where):
    """Images as column windows of wider buffers (row steps w + 5 .. w + 13,
    windows starting 1 .. 7 bytes in), so the rows start at every offset
    modulo 16: the gather's shifted vector path, against the oracle on the
    contiguous images."""
    from orb_slam2_detailed_comments_gb300._lib import KEYPOINT_DTYPE
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor
    fr = frames(17, 5)
    views = []
    for f, (img, _) in enumerate(fr):
        h, w = img.shape
        off, pad = 1 + (3 * f) % 7, 5 + 2 * f
        big = torch.zeros((h, w + off + pad), dtype=torch.uint8)
        big[:, off:off + w] = torch.from_numpy(img)
        big = big.cuda() if where == "device" else big.pin_memory()
        views.append(big[:, off:off + w])
    b = BatchExtractor(len(fr), 1280, 720, 2000)
    cap = b.per_frame_capacity
    k, d, c = b.extract(views, [nf for _, nf in fr])
    k = k.cpu().numpy().view(KEYPOINT_DTYPE).reshape(len(fr), cap)
    d = d.cpu().numpy().reshape(len(fr), cap, 32)
    c = c.cpu().numpy()
    for f, (img, nf) in enumerate(fr):
        ref = oracle.extract(img, nfeatures=nf, want_pyramid=False)
        assert c[f] == len(ref.keypoints), f"frame {f}"
        assert_kps_equal(k[f, :c[f]], ref.keypoints, f"frame {f}")
        assert np.array_equal(d[f, :c[f]], ref.descriptors)


@pytest.mark.parametrize("dz,mono,ori", [(0.0, True, True), (2.0, False, True), (-2.0, False, False)])
def test_batch_frame_projection_vs_oracle(torch, oracle, dz, mono, ori):
    """SearchByProjection(CurrentFrame, LastFrame) for every frame of a batch,
    each against its own LastFrame and pose, equals the oracle frame by frame."""
    from orb_slam2_detailed_comments_gb300._lib import KEYPOINT_DTYPE
    from orb_slam2_detailed_comments_gb300 import synthetic as syn
    from orb_slam2_detailed_comments_gb300.batch import BatchExtractor, BatchFrameProjection, motion_struct
    b = BatchExtractor(8, 1280, 720, 2000)
    cap = b.per_frame_capacity
    fr = frames(11, 5)
    k, d, c = b.extract([torch.from_numpy(img).cuda() for img, _ in fr], [nf for _, nf in fr])
    kh = k.cpu().numpy().view(KEYPOINT_DTYPE).reshape(len(fr), cap)
    dh = d.cpu().numpy().reshape(len(fr), cap, 32)
    ch = c.cpu().numpy()
    cases, motions, refs = [], [], []
    for f, (img, _) in enumerate(fr):
        n = int(ch[f])
        h, w = img.shape
        cs = syn.motion_case(kh[f, :n], dh[f, :n], w, h, seed=40 + f, dz=dz, claimed_p=0.0)
        cases.append(cs)
        motions.append(motion_struct(cs["Tcw"], cs["Tlw"], cs["fx"], cs["fy"], cs["cx"], cs["cy"], cs["bf"], cs["b"]))
        mo = pyoracle.make_motion(cs["Tcw"], cs["Tlw"], cs["fx"], cs["fy"], cs["cx"], cs["cy"], cs["bf"], cs["b"])
        refs.append(oracle.search_by_projection_frame(kh[f, :n], dh[f, :n], w, h, cs["last_kps"], cs["last_mps"],
                                                      cs["last_mp_desc"], mo, th=7.0 if mono else 15.0, mono=mono,
                                                      check_ori=ori))
    lk = np.concatenate([cs["last_kps"] for cs in cases])
    lm = np.concatenate([cs["last_mps"] for cs in cases])
    ld = np.concatenate([cs["last_mp_desc"] for cs in cases])
    p = BatchFrameProjection(b, check_ori=ori)
    match, nm = p.search(torch.from_numpy(lk.view(np.float32).reshape(-1, 7)).cuda(),
                         torch.from_numpy(lm.view(np.uint8)).cuda(), torch.from_numpy(np.ascontiguousarray(ld)).cuda(),
                         [len(cs["last_kps"]) for cs in cases], motions, 7.0 if mono else 15.0, mono)
    match = match.cpu().numpy().reshape(len(fr), cap)
    nm = nm.cpu().numpy()
    for f in range(len(fr)):
        n = int(ch[f])
        assert nm[f] == refs[f][0], f"frame {f}"
        assert np.array_equal(match[f, :n], refs[f][1]), f"frame {f}"
        assert (match[f, n:] == -3).all()
