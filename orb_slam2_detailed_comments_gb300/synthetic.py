"""Seeded synthetic inputs for the ORB front-end workloads.

No public dataset is used: every image is generated from a seed with the
shapes, sizes and value distributions of the benchmark workloads --
200 filled rectangles / ellipses with uniform intensities 0-255 over a random
background, plus a 3x3-smoothed Gaussian noise layer (sigma 8), clipped to
uint8.  Second views are homography warps (rotation <= 3 deg, translation <=
10 px, + noise sigma 2); stereo right views shift each pixel by a
piecewise-planar disparity in 5-80 px (+ noise sigma 2).
"""
from __future__ import annotations

import numpy as np


def _smooth3(a: np.ndarray) -> np.ndarray:
    p = np.pad(a, 1, mode="edge")
    h, w = a.shape
    s = np.zeros_like(a)
    for dy in range(3):
        for dx in range(3):
            s += p[dy:dy + h, dx:dx + w]
    return s / 9.0


def scene(w: int, h: int, seed: int, n_shapes: int = 200, noise_sigma: float = 8.0) -> np.ndarray:
    """A w x h uint8 scene of random filled rectangles and ellipses."""
    rng = np.random.default_rng(seed)
    img = np.full((h, w), float(rng.integers(0, 256)), dtype=np.float32)
    yy, xx = np.mgrid[0:h, 0:w]
    max_half = max(8, min(w, h) // 6)
    for _ in range(n_shapes):
        cx, cy = rng.uniform(0, w), rng.uniform(0, h)
        ax, ay = rng.uniform(3, max_half), rng.uniform(3, max_half)
        val = float(rng.integers(0, 256))
        x0, x1 = max(0, int(cx - ax) - 1), min(w, int(cx + ax) + 2)
        y0, y1 = max(0, int(cy - ay) - 1), min(h, int(cy + ay) + 2)
        if x0 >= x1 or y0 >= y1:
            continue
        sx, sy = xx[y0:y1, x0:x1], yy[y0:y1, x0:x1]
        if rng.random() < 0.5:
            m = (np.abs(sx - cx) <= ax) & (np.abs(sy - cy) <= ay)
        else:
            m = ((sx - cx) / ax) ** 2 + ((sy - cy) / ay) ** 2 <= 1.0
        img[y0:y1, x0:x1][m] = val
    noise = _smooth3(rng.normal(0.0, noise_sigma, size=(h, w)).astype(np.float32))
    return np.clip(np.rint(img + noise), 0, 255).astype(np.uint8)


def _bilinear(img: np.ndarray, sx: np.ndarray, sy: np.ndarray) -> np.ndarray:
    h, w = img.shape
    sx = np.clip(sx, 0, w - 1.0001)
    sy = np.clip(sy, 0, h - 1.0001)
    x0, y0 = np.floor(sx).astype(np.int64), np.floor(sy).astype(np.int64)
    fx, fy = sx - x0, sy - y0
    a = img.astype(np.float32)
    return ((a[y0, x0] * (1 - fx) + a[y0, x0 + 1] * fx) * (1 - fy)
            + (a[y0 + 1, x0] * (1 - fx) + a[y0 + 1, x0 + 1] * fx) * fy)


def random_homography(w: int, h: int, rng: np.random.Generator, max_rot_deg: float = 3.0,
                      max_shift: float = 10.0) -> np.ndarray:
    """Rotation about the image centre plus a translation, as a 3x3 matrix."""
    th = np.deg2rad(rng.uniform(-max_rot_deg, max_rot_deg))
    tx, ty = rng.uniform(-max_shift, max_shift, size=2)
    c, s = np.cos(th), np.sin(th)
    cx, cy = w / 2.0, h / 2.0
    return np.array([[c, -s, cx - c * cx + s * cy + tx],
                     [s, c, cy - s * cx - c * cy + ty],
                     [0.0, 0.0, 1.0]])


def warp(img: np.ndarray, H: np.ndarray, seed: int, noise_sigma: float = 2.0) -> np.ndarray:
    """img warped by H (destination pixel p samples source H^-1 p) plus noise."""
    rng = np.random.default_rng(seed)
    h, w = img.shape
    Hi = np.linalg.inv(H)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    den = Hi[2, 0] * xx + Hi[2, 1] * yy + Hi[2, 2]
    sx = (Hi[0, 0] * xx + Hi[0, 1] * yy + Hi[0, 2]) / den
    sy = (Hi[1, 0] * xx + Hi[1, 1] * yy + Hi[1, 2]) / den
    out = _bilinear(img, sx, sy) + rng.normal(0.0, noise_sigma, size=(h, w))
    return np.clip(np.rint(out), 0, 255).astype(np.uint8)


def frame_pair(w: int, h: int, seed: int):
    """(frame1, frame2, H): frame2 is frame1 under a small homography + noise."""
    f1 = scene(w, h, seed)
    rng = np.random.default_rng(seed + 7919)
    H = random_homography(w, h, rng)
    return f1, warp(f1, H, seed + 104729), H


def disparity_map(w: int, h: int, rng: np.random.Generator, dmin: float = 5.0, dmax: float = 80.0) -> np.ndarray:
    """Piecewise-planar disparity: a few vertical bands, each its own plane."""
    d = np.empty((h, w), dtype=np.float64)
    nb = int(rng.integers(3, 7))
    cuts = np.sort(rng.uniform(0, w, size=nb - 1)).astype(int)
    edges = [0, *cuts.tolist(), w]
    yy, xx = np.mgrid[0:h, 0:w]
    for i in range(nb):
        a = rng.uniform(dmin, dmax)
        gx, gy = rng.uniform(-0.03, 0.03), rng.uniform(-0.05, 0.05)
        sl = slice(edges[i], edges[i + 1])
        d[:, sl] = a + gx * (xx[:, sl] - edges[i]) + gy * (yy[:, sl] - h / 2)
    return np.clip(d, dmin, dmax)


def stereo_pair(w: int, h: int, seed: int, noise_sigma: float = 2.0):
    """(left, right, disparity): right(x, y) = left(x + d(x, y), y) + noise."""
    left = scene(w, h, seed)
    rng = np.random.default_rng(seed + 31337)
    d = disparity_map(w, h, rng)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    right = _bilinear(left, xx + d, yy) + rng.normal(0.0, noise_sigma, size=(h, w))
    return left, np.clip(np.rint(right), 0, 255).astype(np.uint8), d


def random_descriptors(n: int, seed: int) -> np.ndarray:
    """n x 32 uint8 descriptors with independent Bernoulli(0.5) bits."""
    return np.random.default_rng(seed).integers(0, 256, size=(n, 32), dtype=np.uint8)


def clustered_descriptors(n: int, n_centres: int, flip_p: float, seed: int) -> np.ndarray:
    """n descriptors, each a random centre XOR Bernoulli(flip_p) bit flips."""
    rng = np.random.default_rng(seed)
    centres = rng.integers(0, 256, size=(n_centres, 32), dtype=np.uint8)
    pick = rng.integers(0, n_centres, size=n)
    bits = rng.random(size=(n, 256)) < flip_p
    flips = np.packbits(bits, axis=1, bitorder="little")
    return centres[pick] ^ flips


def stream_frames(w: int, h: int, seed: int, nframes: int, noise_sigma: float = 2.0):
    """A camera stream: frame k is the stream's scene under a drifting
    homography (random walk of small rotations / translations) + noise."""
    base = scene(w, h, seed)
    rng = np.random.default_rng(seed + 4242)
    H = np.eye(3)
    out = []
    for k in range(nframes):
        out.append(warp(base, H, seed * 7919 + k, noise_sigma))
        H = random_homography(w, h, rng, max_rot_deg=1.0, max_shift=3.0) @ H
    return out


from ._lib import FRAME_MAPPOINT_DTYPE, MP_OBSERVED, MP_OUTLIER, MP_PRESENT  # noqa: E402


def _rot(rx: float, ry: float, rz: float) -> np.ndarray:
    cx_, sx = np.cos(rx), np.sin(rx)
    cy_, sy = np.cos(ry), np.sin(ry)
    cz, sz = np.cos(rz), np.sin(rz)
    Rx = np.array([[1, 0, 0], [0, cx_, -sx], [0, sx, cx_]])
    Ry = np.array([[cy_, 0, sy], [0, 1, 0], [-sy, 0, cy_]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def motion_case(kps: np.ndarray, desc: np.ndarray, w: int, h: int, seed: int, n_last: int | None = None,
                stereo: bool = False, dz: float = 0.0, rot_offset_deg: float = 8.0, flip_p: float = 0.08,
                claimed_p: float = 0.05):
    """A LastFrame for SearchByProjection(CurrentFrame, LastFrame, th, bMono)
    whose map points project near the given current keypoints.

    kps / desc: the current frame (structured 28-byte keypoints, n x 32).
    dz: the current camera's displacement along the last camera's optical
    axis (metres; > baseline = forward, < -baseline = backward).
    Returns a dict with last_kps, last_mps (FRAME_MAPPOINT_DTYPE),
    last_mp_desc, Tcw, Tlw (3 x 4 float32), fx, fy, cx, cy, bf, b, uright
    (current frame, stereo only) and claimed (current frame)."""
    rng = np.random.default_rng(seed)
    n = len(kps)
    if n_last is None:
        n_last = max(1, int(n * 1.1))
    fx = fy = 718.856
    cx, cy = w / 2.0, h / 2.0
    bf = 386.1
    b = bf / fx
    Rcw = _rot(*rng.normal(0, 0.02, 3))
    tcw = rng.normal(0, 0.3, 3)
    twc = -Rcw.T @ tcw
    Rlw = Rcw @ _rot(*rng.normal(0, 0.005, 3))
    Cl = twc - Rlw.T @ np.array([0.0, 0.0, dz])  # last camera centre in the world
    tlw = -Rlw @ Cl
    Tcw = np.hstack([Rcw, tcw[:, None]]).astype(np.float32)
    Tlw = np.hstack([Rlw, tlw[:, None]]).astype(np.float32)
    zj = rng.uniform(3.0, 40.0, size=max(n, 1))
    uright = None
    if stereo:
        uright = np.full(n, -1.0, np.float32)
        has = rng.random(n) < 0.7
        uright[has] = (kps["x"][has] - bf / zj[:n][has] + rng.normal(0, 0.5, has.sum())).astype(np.float32)
    last_kps = np.zeros(n_last, kps.dtype)
    mps = np.zeros(n_last, FRAME_MAPPOINT_DTYPE)
    mpd = rng.integers(0, 256, size=(n_last, 32), dtype=np.uint8)
    for i in range(n_last):
        if n > 0 and rng.random() < 0.85:
            j = int(rng.integers(0, n))
            u = float(kps["x"][j]) + rng.normal(0, 1.0)
            v = float(kps["y"][j]) + rng.normal(0, 1.0)
            z = zj[j] * (1 + rng.normal(0, 0.01))
            octv = int(np.clip(int(kps["octave"][j]) + rng.choice([-1, 0, 0, 0, 1]), 0, 7))
            ang = float(kps["angle"][j]) + rot_offset_deg + rng.normal(0, 3.0)
            if rng.random() < 0.1:
                ang = rng.uniform(0, 360)
            flips = np.packbits(rng.random(256) < flip_p, bitorder="little")
            mpd[i] = desc[j] ^ flips
        else:
            u, v = rng.uniform(-20, w + 20), rng.uniform(-20, h + 20)
            z = rng.uniform(3.0, 40.0) * (-1 if rng.random() < 0.05 else 1)
            octv = int(rng.integers(0, 8))
            ang = rng.uniform(0, 360)
        Xc = np.array([(u - cx) * z / fx, (v - cy) * z / fy, z])
        Xw = Rcw.T @ (Xc - tcw)
        mps[i] = (Xw[0], Xw[1], Xw[2], 0)
        r = rng.random()
        flags = MP_PRESENT if r < 0.9 else 0
        if flags and rng.random() < 0.05:
            flags |= MP_OUTLIER
        if flags and rng.random() < 0.85:
            flags |= MP_OBSERVED
        mps["flags"][i] = flags
        last_kps[i]["octave"] = octv
        last_kps[i]["angle"] = np.float32(ang % 360.0)
        last_kps[i]["class_id"] = -1
    claimed = (rng.random(n) < claimed_p).astype(np.uint8)
    return dict(last_kps=last_kps, last_mps=mps, last_mp_desc=mpd, Tcw=Tcw, Tlw=Tlw, fx=fx, fy=fy, cx=cx, cy=cy,
                bf=bf, b=b, uright=uright, claimed=claimed)


def chain_case(k: int = 30, seed: int = 0, observed_every: int = 1):
    """k current keypoints on one spot whose descriptors sit 0, 1, 2, ... bits
    from a common descriptor D, and k LastFrame map points with descriptor D
    projecting onto that spot (identity poses): in reference order map point i
    takes keypoint i, so a parallel resolution needs k rounds.  Every
    observed_every-th map point has observations (the others block nothing).
    Returns (kps, desc, case dict as motion_case, w, h)."""
    rng = np.random.default_rng(seed)
    w, h = 640, 480
    from ._lib import KEYPOINT_DTYPE
    kps = np.zeros(k, KEYPOINT_DTYPE)
    kps["x"] = 320.0 + rng.uniform(-1, 1, k).astype(np.float32)
    kps["y"] = 240.0 + rng.uniform(-1, 1, k).astype(np.float32)
    kps["size"] = 31.0
    kps["angle"] = rng.uniform(0, 360, k).astype(np.float32)
    kps["octave"] = 0
    kps["class_id"] = -1
    D = rng.integers(0, 256, 32, dtype=np.uint8)
    desc = np.zeros((k, 32), np.uint8)
    for j in range(k):
        bits = np.zeros(256, bool)
        bits[:j] = True
        desc[j] = D ^ np.packbits(bits, bitorder="little")
    fx = fy = 500.0
    cx, cy = 320.0, 240.0
    last_kps = np.zeros(k, KEYPOINT_DTYPE)
    last_kps["octave"] = 0
    last_kps["angle"] = (kps["angle"] + 5.0) % 360.0
    mps = np.zeros(k, FRAME_MAPPOINT_DTYPE)
    z = 10.0
    mps["x"] = (320.0 - cx) * z / fx
    mps["y"] = (240.0 - cy) * z / fy
    mps["z"] = z
    mps["flags"] = MP_PRESENT
    mps["flags"][::observed_every] |= MP_OBSERVED
    T = np.hstack([np.eye(3), np.zeros((3, 1))]).astype(np.float32)
    case = dict(last_kps=last_kps, last_mps=mps, last_mp_desc=np.tile(D, (k, 1)), Tcw=T, Tlw=T, fx=fx, fy=fy, cx=cx,
                cy=cy, bf=0.0, b=0.0, uright=None, claimed=np.zeros(k, np.uint8))
    return kps, desc, case, w, h


def _plane_points(u, v, Tcw, K, depth):
    """World points of the plane Z = depth seen at pixels (u, v) from pose
    Tcw (3 x 4): ray from the camera centre through the pixel."""
    fx, fy, cx, cy = K
    R, t = Tcw[:, :3].astype(np.float64), Tcw[:, 3].astype(np.float64)
    C = -R.T @ t
    d = np.stack([(u - cx) / fx, (v - cy) / fy, np.ones_like(u)], -1) @ R  # rows: R^T d_c
    lam = (depth - C[2]) / d[..., 2]
    return C + lam[..., None] * d


def camera_stream(w: int, h: int, seed: int, nframes: int, depth: float = 8.0, noise_sigma: float = 2.0):
    """A camera moving in front of a textured plane Z = depth (world frame).

    Frame k is the plane seen from pose Tcw_k, rendered by casting each
    pixel's ray onto the plane and sampling the texture bilinearly, plus
    N(0, noise_sigma).  The poses follow a smooth random walk (rotations of a
    few tenths of a degree and translations of about 1 % of the depth per
    frame).  Returns (frames, poses (3 x 4 float32 each), K = (fx, fy, cx,
    cy), depth)."""
    rng = np.random.default_rng(seed)
    fx = fy = 0.9 * w
    cx, cy = w / 2.0, h / 2.0
    K = (fx, fy, cx, cy)
    tw, th_ = int(w * 1.6), int(h * 1.6)
    tex = scene(tw, th_, seed).astype(np.float64)
    s = depth / fx  # world units per texel: the first view maps texels about 1:1 to pixels
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float64)
    R = np.eye(3)
    t = np.zeros(3)
    w_rot = np.zeros(3)
    v_tr = np.zeros(3)
    frames, poses = [], []
    for _ in range(nframes):
        Tcw = np.hstack([R, t[:, None]])
        P = _plane_points(xx, yy, Tcw, K, depth)
        a = P[..., 0] / s + tw / 2.0
        b = P[..., 1] / s + th_ / 2.0
        img = _bilinear(tex, a, b) + rng.normal(0.0, noise_sigma, size=(h, w))
        frames.append(np.clip(np.rint(img), 0, 255).astype(np.uint8))
        poses.append(Tcw.astype(np.float32))
        w_rot = 0.8 * w_rot + rng.normal(0, 0.0015, 3)
        v_tr = 0.8 * v_tr + rng.normal(0, 0.004 * depth, 3)
        R = _rot(*w_rot) @ R
        t = t + v_tr
    return frames, poses, K, depth


def plane_mappoints(kps, Tcw, K, depth):
    """orbgpu_frame_mappoint records (present and observed) of keypoints seen
    from pose Tcw on the plane Z = depth (level-0 coordinates)."""
    P = _plane_points(np.asarray(kps["x"], np.float64), np.asarray(kps["y"], np.float64), np.asarray(Tcw), K, depth)
    out = np.zeros(len(kps), FRAME_MAPPOINT_DTYPE)
    out["x"], out["y"], out["z"] = P[:, 0], P[:, 1], P[:, 2]
    out["flags"] = MP_PRESENT | MP_OBSERVED
    return out


def predict_pose(T_last, T_lastlast):
    """Constant-velocity prediction mVelocity * LastFrame.mTcw with
    mVelocity = Tcw_last * Twc_lastlast (src/Tracking.cc, TrackWithMotionModel)."""
    def h(T):
        M = np.eye(4)
        M[:3, :4] = T
        return M
    if T_lastlast is None:
        return np.asarray(T_last, np.float32)
    V = h(T_last) @ np.linalg.inv(h(T_lastlast))
    return (V @ h(T_last))[:3, :4].astype(np.float32)


def observation_case(m: int, seed: int, mean_len: float = 6.0, max_len: int = 64, bad_frac: float = 0.05,
                     empty_frac: float = 0.02, flip_ands: int = 3, extra_rows: int = 0, low_entropy: bool = False):
    """Map points with observation lists over a keyframe descriptor pool, the
    input of MapPoint::ComputeDistinctiveDescriptors.

    List lengths are geometric with the given mean (capped at max_len; a
    fraction empty_frac of the map points has none).  Every observation of a
    map point is a noisy copy of that map point's base descriptor, each bit
    flipped with probability 2**-flip_ands; the copies sit at random rows of
    the pool (extra_rows unrelated rows added), and a fraction bad_frac of the
    observations is marked -1 (a bad keyframe).  low_entropy keeps only the two
    low bits of every byte, which makes equal distances and equal medians (the
    tie rule) common.  Returns (pool (P, 32) uint8, obs_offsets (m + 1,) int32,
    obs_rows (n,) int32).
    """
    rng = np.random.default_rng(seed)
    lens = np.minimum(rng.geometric(1.0 / max(mean_len, 1.0), m), max_len).astype(np.int64)
    lens[rng.random(m) < empty_frac] = 0
    offsets = np.zeros(m + 1, np.int64)
    np.cumsum(lens, out=offsets[1:])
    n = int(offsets[-1])
    base = rng.integers(0, 256, (m, 32), dtype=np.uint8)
    flips = rng.integers(0, 256, (n, 32), dtype=np.uint8)
    for _ in range(flip_ands - 1):
        flips &= rng.integers(0, 256, (n, 32), dtype=np.uint8)
    obs = base[np.repeat(np.arange(m), lens)] ^ flips
    pool = np.empty((n + extra_rows, 32), np.uint8)
    rows = rng.permutation(n + extra_rows)[:n]
    pool[rows] = obs
    if extra_rows:
        free = np.ones(n + extra_rows, bool)
        free[rows] = False
        pool[free] = rng.integers(0, 256, (extra_rows, 32), dtype=np.uint8)
    if low_entropy:
        pool &= np.uint8(3)
    rows = rows.astype(np.int32)
    rows[rng.random(n) < bad_frac] = -1
    return pool, offsets.astype(np.int32), rows


def _rotation(a: float, b: float, c: float) -> np.ndarray:
    ca, sa, cb, sb, cc, sc = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(c), np.sin(c)
    rx = np.array([[1, 0, 0], [0, ca, -sa], [0, sa, ca]])
    ry = np.array([[cb, 0, sb], [0, 1, 0], [-sb, 0, cb]])
    rz = np.array([[cc, -sc, 0], [sc, cc, 0], [0, 0, 1]])
    return rz @ ry @ rx


def frustum_case(m: int, seed: int, w: int = 640, h: int = 480, fx: float = 500.0, scale_factor: float = 1.2,
                 nlevels: int = 8):
    """Local map points around a camera for Frame::isInFrustum.

    The camera has a random pose; map points lie in a box in front of it (a
    part behind it and beyond the image borders), with normals near the viewing
    ray (some turned away), and distance invariance limits placed so that the
    ratio mfMaxDistance / distance falls on and beside the predicted-level
    boundaries (powers of the scale factor, off by 0 or 1 ulp-sized factors).
    Returns (Tcw rows 0-2 as float32 (3, 4), geometry records with the fields
    x, y, z, nx, ny, nz, min_distance, max_distance as a float32 (m, 8) array).
    """
    rng = np.random.default_rng(seed)
    R = _rotation(*rng.normal(0, 0.3, 3))
    t = rng.normal(0, 1, 3)
    Tcw = np.hstack([R, t[:, None]]).astype(np.float32)
    Rwc = R.T
    Ow = -Rwc @ t
    zmax = 40.0
    pc = np.stack([rng.uniform(-0.7, 0.7, m) * w / fx * zmax / 2, rng.uniform(-0.7, 0.7, m) * h / fx * zmax / 2,
                   rng.uniform(-2.0, zmax, m)], 1)
    pw = (Rwc @ pc.T).T + Ow
    nrm = pw - Ow + rng.normal(0, 2.5, (m, 3)) * np.linalg.norm(pw - Ow, axis=1, keepdims=True) / 8
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    d = np.linalg.norm(pw - Ow, axis=1)
    lev = rng.integers(-2, nlevels + 2, m)
    jitter = rng.choice([1.0, 1 + 1e-7, 1 - 1e-7, 1 + 3e-7, 1.0001, 0.9999], m)
    maxd = (d * scale_factor ** lev * jitter).astype(np.float32)
    mind = (maxd / scale_factor ** (nlevels - 1) * rng.choice([1.0, 0.5, 2.0, 5.0, 1.25], m)).astype(np.float32)
    g = np.stack([pw[:, 0], pw[:, 1], pw[:, 2], nrm[:, 0], nrm[:, 1], nrm[:, 2], mind, maxd], 1).astype(np.float32)
    return Tcw, g


def vocabulary(k: int, L: int, seed: int, stop_frac: float = 0.02, scoring: int = 0, weighting: int = 0):
    """A DBoW2 vocabulary tree standing in for ORBvoc.txt (which is not in the
    reference tree): the full k-ary tree of depth L in breadth-first order.
    Level-1 node descriptors are random; every child is its parent's
    descriptor with each bit flipped with probability 2**-(level + 1), so the
    tree clusters like a k-means hierarchy.  Leaf weights are idf-like,
    log(N / n) for a random document count n (a fraction stop_frac of the
    words get weight 0, DBoW2's stopped words); inner nodes weigh 0.
    Returns a dict with k, L, scoring, weighting and, for nodes 1..N-1 (node
    0 is the root), parents, is_leaf, descriptors (N-1, 32) and weights."""
    rng = np.random.default_rng(seed)
    sizes = [k ** lvl for lvl in range(1, L + 1)]
    firsts = np.cumsum([1] + sizes[:-1])  # id of the first node of each level
    parents, leaves, descs, weights = [], [], [], []
    prev = np.zeros((1, 32), np.uint8)
    for lvl, (n, first) in enumerate(zip(sizes, firsts), start=1):
        par_local = np.arange(n) // k
        parent_ids = (0 if lvl == 1 else firsts[lvl - 2]) + par_local
        if lvl == 1:
            d = rng.integers(0, 256, (n, 32), dtype=np.uint8)
        else:
            flips = rng.integers(0, 256, (n, 32), dtype=np.uint8)
            for _ in range(lvl):
                flips &= rng.integers(0, 256, (n, 32), dtype=np.uint8)
            d = prev[par_local] ^ flips
        leaf = np.full(n, lvl == L)
        w = np.zeros(n)
        if lvl == L:
            w = np.log(n / rng.integers(1, n, n).astype(np.float64))
            w[rng.random(n) < stop_frac] = 0.0
        parents.append(parent_ids)
        leaves.append(leaf)
        descs.append(d)
        weights.append(w)
        prev = d
    return {"k": k, "L": L, "scoring": scoring, "weighting": weighting,
            "parents": np.concatenate(parents).astype(np.int32), "is_leaf": np.concatenate(leaves).astype(np.uint8),
            "descriptors": np.concatenate(descs), "weights": np.concatenate(weights)}


def write_vocabulary_text(voc: dict, path: str) -> None:
    """The vocabulary in the text format TemplatedVocabulary::loadFromTextFile
    reads: "k L scoring weighting", then one line per node after the root,
    "parent is_leaf d0 .. d31 weight" (no trailing newline)."""
    lines = [f"{voc['k']} {voc['L']} {voc['scoring']} {voc['weighting']}"]
    for p, lf, d, w in zip(voc["parents"], voc["is_leaf"], voc["descriptors"], voc["weights"]):
        lines.append(f"{int(p)} {int(lf)} " + " ".join(str(int(b)) for b in d) + f" {float(w)!r}")
    with open(path, "w") as f:
        f.write("\n".join(lines))


def relocalisation_case(kps: np.ndarray, desc: np.ndarray, w: int, h: int, seed: int, m: int = 1500,
                        fx: float = 500.0):
    """A keyframe's map points for SearchByProjection(Frame&, KeyFrame*, ...)
    against a frame with keypoints kps / descriptors desc: each map point is
    the back-projection of a random keypoint at a random depth through a
    random camera pose (so it projects near that keypoint), its descriptor a
    copy of the keypoint's with some bits flipped (a fifth get random
    descriptors), its distance limits placing the predicted level near the
    keypoint's octave; the keyframe keypoint angles are the frame's rotated by
    a common 12 degrees (a tenth random).  Some map points sit behind the
    camera (the search has no depth test), and the states mix usable (1),
    bad (2), already found (3) and none (0).  Returns (Tcw (3, 4) float32,
    cam (fx, fy, cx, cy), kf_kps, geometry (m, 8) float32, mp_desc,
    mp_state, claimed)."""
    rng = np.random.default_rng(seed)
    cx, cy = w / 2.0, h / 2.0
    R = _rotation(*rng.normal(0, 0.2, 3))
    t = rng.normal(0, 0.5, 3)
    Tcw = np.hstack([R, t[:, None]]).astype(np.float32)
    sel = rng.integers(0, len(kps), m)
    z = rng.uniform(1.5, 25.0, m)
    z[rng.random(m) < 0.05] *= -1.0
    pc = np.stack([(kps["x"][sel] + rng.normal(0, 1.0, m) - cx) / fx * z,
                   (kps["y"][sel] + rng.normal(0, 1.0, m) - cy) / fx * z, z], 1)
    pw = (R.T @ (pc - t).T).T
    Ow = -R.T @ t
    d = np.linalg.norm(pw - Ow, axis=1)
    maxd = d * 1.2 ** (kps["octave"][sel] + rng.uniform(-0.45, 0.45, m))
    geom = np.zeros((m, 8), np.float32)
    geom[:, :3] = pw
    geom[:, 6] = maxd / 1.2 ** 7
    geom[:, 7] = maxd
    flips = rng.integers(0, 256, (m, 32), dtype=np.uint8)
    for _ in range(3):
        flips &= rng.integers(0, 256, (m, 32), dtype=np.uint8)
    mp_desc = desc[sel] ^ flips
    rnd = rng.random(m) < 0.2
    mp_desc[rnd] = rng.integers(0, 256, (int(rnd.sum()), 32), dtype=np.uint8)
    kf_kps = kps[sel].copy()
    kf_kps["angle"] = (kf_kps["angle"] + 12.0) % 360.0
    odd = rng.random(m) < 0.1
    kf_kps["angle"][odd] = rng.uniform(0, 360, int(odd.sum()))
    mp_state = rng.choice([1, 1, 1, 1, 1, 1, 2, 3, 0], m).astype(np.uint8)
    claimed = (rng.random(len(kps)) < 0.05).astype(np.uint8)
    return Tcw, np.array([fx, fx, cx, cy], np.float32), kf_kps, geom, mp_desc, mp_state, claimed


def triangulation_case(H: np.ndarray, n1: int, n2: int, seed: int, w: int = 640, h: int = 480):
    """Inputs of SearchForTriangulation for a frame pair related by the
    homography H (x2 = H x1): F12 = [e]x H^-1 for a random epipole e, which
    every true correspondence satisfies (x1^T F12 x2 = 0); pKF1's camera
    centre and pKF2's pose / camera placing the epipole in pKF2 inside the
    image; a third of the features carrying map points; a quarter stereo.
    Returns (Cw1, T2 (3, 4), K2 (fx, fy, cx, cy), F12 (3, 3), mp1, mp2, ur1,
    ur2) as float32 / uint8 arrays."""
    rng = np.random.default_rng(seed)
    e = np.array([rng.uniform(0, w), rng.uniform(0, h), 1.0])
    ex = np.array([[0, -e[2], e[1]], [e[2], 0, -e[0]], [-e[1], e[0], 0]])
    F12 = (ex @ np.linalg.inv(H)).astype(np.float64)
    F12 /= np.abs(F12).max()
    R2 = _rotation(*rng.normal(0, 0.1, 3))
    t2 = rng.normal(0, 0.5, 3)
    T2 = np.hstack([R2, t2[:, None]]).astype(np.float32)
    K2 = np.array([500.0, 500.0, w / 2, h / 2], np.float32)
    # pKF1's centre: a point that pKF2 sees at a random pixel, depth 5-20
    z = rng.uniform(5, 20)
    pc = np.array([(rng.uniform(0, w) - w / 2) / 500.0 * z, (rng.uniform(0, h) - h / 2) / 500.0 * z, z])
    Cw1 = (R2.T @ (pc - t2)).astype(np.float32)
    mp1 = (rng.random(n1) < 0.33).astype(np.uint8)
    mp2 = (rng.random(n2) < 0.33).astype(np.uint8)
    ur1 = np.where(rng.random(n1) < 0.25, rng.uniform(0, w, n1), -1.0).astype(np.float32)
    ur2 = np.where(rng.random(n2) < 0.25, rng.uniform(0, w, n2), -1.0).astype(np.float32)
    return Cw1, T2, K2, F12.astype(np.float32), mp1, mp2, ur1, ur2


def sim3_case(kps: np.ndarray, desc: np.ndarray, w: int, h: int, seed: int, m: int = 1500):
    """Inputs of SearchByProjection(KeyFrame*, Scw, vpPoints, vpMatched, th)
    for a keyframe with keypoints kps / descriptors desc: the map points of
    relocalisation_case seen through Scw = [s R | s t] (s in 0.5 .. 2), their
    normals along the viewing ray with noise (a fifth turned away), states
    usable (1) or bad (2), and a twentieth of the keypoints already matched.
    Returns (Scw (3, 4) float32, cam, points (m, 8) float32, descriptors,
    states, claimed)."""
    rng = np.random.default_rng(seed)
    Tcw, cam, _, geom, mp_desc, _, claimed = relocalisation_case(kps, desc, w, h, seed, m)
    s = rng.uniform(0.5, 2.0)
    Scw = Tcw.astype(np.float64) * s
    R, t = Tcw[:, :3].astype(np.float64), Tcw[:, 3].astype(np.float64)
    Ow = -R.T @ t
    ray = geom[:, :3] - Ow
    nrm = ray / np.linalg.norm(ray, axis=1, keepdims=True) + rng.normal(0, 0.3, (m, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm[rng.random(m) < 0.2] *= -1.0
    geom = geom.copy()
    geom[:, 3:6] = nrm
    states = np.where(rng.random(m) < 0.1, 2, 1).astype(np.uint8)
    return Scw.astype(np.float32), cam, geom, mp_desc, states, claimed


def fuse_case(kps: np.ndarray, desc: np.ndarray, seed: int, w: int = 640, h: int = 480):
    """Inputs of Fuse(KeyFrame*, vpMapPoints, th) for a keyframe with keypoints
    kps / descriptors desc: the sim3_case map points seen through the
    de-scaled pose, bf 40, a third of the keypoints with a right coordinate.
    Returns (Tcw (3, 4), cam (fx, fy, cx, cy, bf), points (m, 8), descriptors,
    states, uright)."""
    Scw, cam, g, pd, ps, _ = sim3_case(kps, desc, w, h, seed)
    Tcw = (Scw / np.sqrt((Scw[0, :3].astype(np.float64) ** 2).sum())).astype(np.float32)
    rng = np.random.default_rng(seed)
    ur = np.where(rng.random(len(kps)) < 0.3, kps["x"] - rng.uniform(1, 40, len(kps)), -1).astype(np.float32)
    return Tcw, np.array([cam[0], cam[1], cam[2], cam[3], 40.0], np.float32), g, pd, ps, ur


def sim3_pair_images(seed: int, w: int = 640, h: int = 480, fx: float = 500.0, z0: float = 5.0):
    """Two views of one fronto-parallel textured plane for SearchBySim3:
    image 1 is a scene, image 2 the same plane seen by a camera rotated about
    its optical axis (up to 3 degrees) and shifted (up to 10 px at depth z0)
    -- image 2 is image 1 under the matching homography plus noise.  Returns
    (image1, image2, geometry) with geometry = (R21, t21, z0): camera-2
    coordinates P2 = R21 P1 + t21 of a camera-1 point P1."""
    img1 = scene(w, h, seed)
    rng = np.random.default_rng(seed + 7919)
    H = random_homography(w, h, rng)
    img2 = warp(img1, H, seed + 104729)
    c, sn = H[0, 0], H[1, 0]
    cx, cy = w / 2.0, h / 2.0
    # p2 - c = R(p1 - c) + (tx, ty): recover the pixel translation
    tx = H[0, 2] - (cx - c * cx + sn * cy)
    ty = H[1, 2] - (cy - sn * cx - c * cy)
    R21 = np.array([[c, -sn, 0.0], [sn, c, 0.0], [0.0, 0.0, 1.0]])
    t21 = np.array([tx * z0 / fx, ty * z0 / fx, 0.0])
    return img1, img2, (R21, t21, z0)


def sim3_pair_case(kps1: np.ndarray, desc1: np.ndarray, kps2: np.ndarray, desc2: np.ndarray, geometry, seed: int,
                   w: int = 640, h: int = 480, fx: float = 500.0, prematched: float = 0.08):
    """Inputs of SearchBySim3(pKF1, pKF2, vpMatches12, s12, R12, t12, th) for
    two keyframes of different poses and feature sets: (kps1, desc1) and
    (kps2, desc2) are the extractions of sim3_pair_images' two views.  Each
    keyframe gets its own random world pose (their world frames disagree, as
    a loop's do); the Sim3 maps camera 2 to camera 1 (s12 1 +- 0.003 around the
    views' true rigid motion).  About 60 % of each keyframe's features carry a
    map point (a tenth of them bad): the back-projection of the feature onto
    the plane, its descriptor with a few bits flipped, distances placing the
    predicted level at the feature's octave.  vpMatches12 already holds
    'prematched' of pKF1's usable map points: pre12[i] = the pKF2 feature
    whose map point it is (the nearest pKF2 keypoint to the feature's
    projection that has a map point), -1 elsewhere.  Returns (T1w, T2w, s12,
    R12, t12, cam (fx, fy, cx, cy), geometry1, desc1, state1, geometry2, desc2,
    state2, pre12) with state 0 no map point, 1 usable, 2 bad."""
    R21, t21, z0 = geometry
    rng = np.random.default_rng(seed)
    cx, cy = w / 2.0, h / 2.0
    s12 = np.float32(1.0 + rng.uniform(-0.003, 0.003))
    R12 = R21.T.astype(np.float32)
    t12 = (-(R21.T @ t21)).astype(np.float32)

    def pose():
        R = _rotation(*rng.normal(0, 0.2, 3))
        t = rng.normal(0, 0.5, 3)
        return R, t, np.hstack([R, t[:, None]]).astype(np.float32)

    def side(kps, desc, R, t, sd):
        r = np.random.default_rng(sd)
        n = len(kps)
        pc = np.stack([(kps["x"] - cx) / fx * z0, (kps["y"] - cy) / fx * z0, np.full(n, z0)], 1)
        pw = (R.T @ (pc - t).T).T
        d = np.linalg.norm(pc, axis=1)
        maxd = d * 1.2 ** (kps["octave"] + r.uniform(-0.3, 0.3, n))
        g = np.zeros((n, 8), np.float32)
        g[:, :3] = pw
        g[:, 6] = maxd / 1.2 ** 7
        g[:, 7] = maxd
        flips = r.integers(0, 256, (n, 32), dtype=np.uint8)
        for _ in range(3):
            flips &= r.integers(0, 256, (n, 32), dtype=np.uint8)
        u = r.random(n)
        state = np.where(u < 0.06, 2, np.where(u < 0.6, 1, 0)).astype(np.uint8)
        return g, desc ^ flips, state

    R1, t1, T1 = pose()
    R2, t2, T2 = pose()
    g1, d1, st1 = side(kps1, desc1, R1, t1, seed * 2 + 1)
    g2, d2, st2 = side(kps2, desc2, R2, t2, seed * 2 + 2)
    # vpMatches12 entries that are already set
    pre12 = np.full(len(kps1), -1, np.int32)
    p1 = np.stack([kps1["x"], kps1["y"]], 1).astype(np.float64)
    P1 = np.concatenate([(p1 - [cx, cy]) / fx * z0, np.full((len(p1), 1), z0)], 1)
    P2 = (R21 @ P1.T).T + t21
    proj = P2[:, :2] / P2[:, 2:3] * fx + [cx, cy]
    p2 = np.stack([kps2["x"], kps2["y"]], 1).astype(np.float64)
    taken = set()
    for i in np.nonzero(st1 == 1)[0]:
        if rng.random() >= prematched:
            continue
        dd = np.hypot(*(p2 - proj[i]).T)
        for j in np.argsort(dd)[:3]:
            if st2[j] != 0 and j not in taken and dd[j] < 3.0:
                pre12[i] = j
                taken.add(int(j))
                break
    return T1, T2, s12, R12, t12, np.array([fx, fx, cx, cy], np.float32), g1, d1, st1, g2, d2, st2, pre12


def sim3_usable(state1, state2, pre12):
    """usable1 / usable2 of orbgpu_search_by_sim3 (and the oracle's states)
    for pre-set vpMatches12: pKF1 feature i is skipped where vpMatches12[i]
    is set, pKF2's map point j where j = vpMatches12[i]->GetIndexInKeyFrame(pKF2)
    for some i (src/ORBmatcher.cc:1478-1490)."""
    u1 = (np.asarray(state1) == 1) & (np.asarray(pre12) < 0)
    u2 = np.asarray(state2) == 1
    u2 = u2.copy()
    u2[np.asarray(pre12)[np.asarray(pre12) >= 0]] = False
    return u1.astype(np.uint8), u2.astype(np.uint8)
