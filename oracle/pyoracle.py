"""ORACLE / TEST INFRASTRUCTURE ONLY: ctypes bindings of the two CPU checkers.

* ``Oracle``    -- liborb_oracle.so, this repository's CPU restatement of the
  reference path (orb_oracle.cpp).  Builds anywhere.
* ``RefOracle`` -- oracle/_ref/libref_orb.so, the reference's own sources
  compiled against the cv stand-in (only where those sources are present).
Both expose the same methods so tests can run one against the other.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liborb_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_orb.so")

KP_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("size", "<f4"), ("angle", "<f4"), ("response", "<f4"),
                     ("octave", "<i4"), ("class_id", "<i4")])
MP_DTYPE = np.dtype([("proj_x", "<f4"), ("proj_y", "<f4"), ("proj_xr", "<f4"), ("view_cos", "<f4"),
                     ("track_scale_level", "<i4"), ("track_in_view", "<i4"), ("bad", "<i4"), ("pad", "<i4")])


FMP_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("flags", "<i4")])
GEOM_DTYPE = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("nx", "<f4"), ("ny", "<f4"), ("nz", "<f4"),
                       ("min_distance", "<f4"), ("max_distance", "<f4")])
MP_PRESENT, MP_OUTLIER, MP_OBSERVED = 1, 2, 4


class Motion(C.Structure):
    """Rows 0-2 of both frames' Tcw (row-major 3 x 4) and fx, fy, cx, cy, mbf, mb."""
    _fields_ = [("Tcw", C.c_float * 12), ("Tlw", C.c_float * 12), ("fx", C.c_float), ("fy", C.c_float),
                ("cx", C.c_float), ("cy", C.c_float), ("bf", C.c_float), ("b", C.c_float)]


def make_motion(Tcw, Tlw, fx, fy, cx, cy, bf=0.0, b=0.0) -> Motion:
    m = Motion()
    for i, v in enumerate(np.asarray(Tcw, np.float32).reshape(-1)[:12]):
        m.Tcw[i] = float(v)
    for i, v in enumerate(np.asarray(Tlw, np.float32).reshape(-1)[:12]):
        m.Tlw[i] = float(v)
    m.fx, m.fy, m.cx, m.cy, m.bf, m.b = (float(np.float32(v)) for v in (fx, fy, cx, cy, bf, b))
    return m


class FrustumCamera(C.Structure):
    """Rows 0-2 of mTcw, fx, fy, cx, cy, mbf, image bounds, scale factor, levels."""
    _fields_ = [("Tcw", C.c_float * 12), ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float),
                ("cy", C.c_float), ("bf", C.c_float), ("min_x", C.c_float), ("max_x", C.c_float),
                ("min_y", C.c_float), ("max_y", C.c_float), ("scale_factor", C.c_float), ("nlevels", C.c_int)]


def make_frustum_camera(Tcw, fx, fy, cx, cy, bf, min_x, max_x, min_y, max_y, scale_factor=1.2, nlevels=8):
    c = FrustumCamera()
    for i, v in enumerate(np.asarray(Tcw, np.float32).reshape(-1)[:12]):
        c.Tcw[i] = float(v)
    (c.fx, c.fy, c.cx, c.cy, c.bf, c.min_x, c.max_x, c.min_y, c.max_y,
     c.scale_factor) = (float(np.float32(v)) for v in (fx, fy, cx, cy, bf, min_x, max_x, min_y, max_y, scale_factor))
    c.nlevels = int(nlevels)
    return c


class Params(C.Structure):
    _fields_ = [("nfeatures", C.c_int), ("scale_factor", C.c_float), ("nlevels", C.c_int),
                ("ini_th_fast", C.c_int), ("min_th_fast", C.c_int)]


@dataclass
class ExtractResult:
    keypoints: np.ndarray  # KP_DTYPE
    descriptors: np.ndarray  # N x 32 uint8
    pyramid: list  # unblurred levels (uint8 2-D arrays)


def build(ref=False) -> None:
    """Compile the restatement (and, with ref=True, the reference harness via
    oracle/Makefile; with ref="if-present", only where the reference sources
    are mounted -- the Makefile knows where)."""
    srcs = [os.path.join(HERE, "orb_oracle.cpp"), os.path.join(HERE, "cvshim", "cvshim_prims.cpp")]
    deps = srcs + [os.path.join(HERE, f) for f in ("orb_oracle.h", "orb_types.h", "orb_pattern_table.h")]
    deps.append(os.path.join(HERE, "cvshim", "cvshim_prims.h"))
    if not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < max(os.path.getmtime(d) for d in deps):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        subprocess.run(["g++", "-O3", "-std=c++11", "-ffp-contract=off", "-fPIC", "-shared", "-o", ORACLE_SO, *srcs,
                        "-lm", "-pthread"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref-if-present" if ref == "if-present" else "ref"], check=True)


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def level_sizes(w: int, h: int, nlevels: int, scale_factor: float):
    """Level dimensions exactly as src/ORBextractor.cc:1661-1663 computes them."""
    inv = scale_tables(nlevels, scale_factor)[1]
    return [(int(np.rint(np.float32(w) * inv[l])), int(np.rint(np.float32(h) * inv[l]))) for l in range(nlevels)]


def scale_tables(nlevels: int, scale_factor: float):
    """mvScaleFactor / mvInvScaleFactor (src/ORBextractor.cc:478-500): the
    running product is taken in double (scaleFactor is a double member) and
    stored as float."""
    sf = np.float64(np.float32(scale_factor))
    s = [np.float32(1.0)]
    for _ in range(1, nlevels):
        s.append(np.float32(np.float64(s[-1]) * sf))
    inv = [np.float32(np.float32(1.0) / x) for x in s]
    return s, inv


class _Base:
    def __init__(self, path: str):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.prefix = "ref_" if "ref_orb" in path else "orc_"

    def fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def extract(self, img: np.ndarray, nfeatures=1000, scale_factor=1.2, nlevels=8, ini_th=20, min_th=7,
                want_pyramid=True) -> ExtractResult:
        img = np.ascontiguousarray(img, dtype=np.uint8)
        h, w = img.shape
        p = Params(nfeatures, scale_factor, nlevels, ini_th, min_th)
        cap = max(4 * nfeatures + 64, 256)
        kps = np.zeros(cap, KP_DTYPE)
        desc = np.zeros((cap, 32), np.uint8)
        n = C.c_int(0)
        sizes = level_sizes(w, h, nlevels, scale_factor)
        tot = sum(a * b for a, b in sizes)
        pyr = np.zeros(tot, np.uint8) if want_pyramid else None
        rc = self.fn("extract")(_p(img), w, h, C.c_size_t(w), C.byref(p), _p(kps), _p(desc), cap, C.byref(n),
                                _p(pyr), C.c_size_t(tot))
        if rc != 0:
            raise RuntimeError(f"extract rc={rc}")
        levels = []
        if want_pyramid:
            off = 0
            for lw, lh in sizes:
                levels.append(pyr[off:off + lw * lh].reshape(lh, lw))
                off += lw * lh
        return ExtractResult(kps[:n.value].copy(), desc[:n.value].copy(), levels)

    def descriptor_distance(self, a: np.ndarray, b: np.ndarray) -> int:
        a = np.ascontiguousarray(a, np.uint8)
        b = np.ascontiguousarray(b, np.uint8)
        return int(self.fn("descriptor_distance")(_p(a), _p(b)))

    def features_in_area(self, kps, w, h, x, y, r, min_level=-1, max_level=-1, nlevels=8, scale_factor=1.2):
        kps = np.ascontiguousarray(kps, KP_DTYPE)
        p = Params(1000, scale_factor, nlevels, 20, 7)
        out = np.zeros(max(len(kps), 1), np.int32)
        f = self.fn("features_in_area")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                      C.c_int, C.c_int, C.c_void_p, C.c_int]
        n = f(C.byref(p), _p(kps), len(kps), w, h, x, y, r, min_level, max_level, _p(out), len(out))
        return out[:n].copy()

    def search_for_initialization(self, kps1, desc1, kps2, desc2, w, h, prev_xy=None, window=100, nnratio=0.9,
                                  check_ori=True, nlevels=8, scale_factor=1.2):
        kps1 = np.ascontiguousarray(kps1, KP_DTYPE)
        kps2 = np.ascontiguousarray(kps2, KP_DTYPE)
        desc1 = np.ascontiguousarray(desc1, np.uint8)
        desc2 = np.ascontiguousarray(desc2, np.uint8)
        if prev_xy is None:
            prev_xy = np.stack([kps1["x"], kps1["y"]], axis=1)
        prev = np.ascontiguousarray(prev_xy, np.float32).copy()
        m12 = np.zeros(max(len(kps1), 1), np.int32)
        p = Params(1000, scale_factor, nlevels, 20, 7)
        f = self.fn("search_for_initialization")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                      C.c_int, C.c_void_p, C.c_int, C.c_float, C.c_int, C.c_void_p]
        nm = f(C.byref(p), _p(kps1), _p(desc1), len(kps1), _p(kps2), _p(desc2), len(kps2), w, h, _p(prev),
               window, nnratio, int(check_ori), _p(m12))
        return int(nm), m12[:len(kps1)].copy(), prev

    def search_by_projection(self, kps, desc, w, h, mps, mp_desc, th=1.0, nnratio=0.8, uright=None, claimed=None,
                             nlevels=8, scale_factor=1.2):
        kps = np.ascontiguousarray(kps, KP_DTYPE)
        desc = np.ascontiguousarray(desc, np.uint8)
        mps = np.ascontiguousarray(mps, MP_DTYPE)
        mp_desc = np.ascontiguousarray(mp_desc, np.uint8)
        ur = None if uright is None else np.ascontiguousarray(uright, np.float32)
        cl = None if claimed is None else np.ascontiguousarray(claimed, np.uint8)
        out = np.zeros(max(len(kps), 1), np.int32)
        p = Params(1000, scale_factor, nlevels, 20, 7)
        f = self.fn("search_by_projection")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                      C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_void_p, C.c_void_p]
        nm = f(C.byref(p), _p(kps), _p(desc), _p(ur), len(kps), w, h, _p(mps), _p(mp_desc), len(mps), th, nnratio,
               _p(cl), _p(out))
        return int(nm), out[:len(kps)].copy()

    def search_by_projection_frame(self, kps, desc, w, h, last_kps, last_mps, last_mp_desc, motion, th=7.0,
                                   mono=True, check_ori=True, uright=None, claimed=None, nlevels=8,
                                   scale_factor=1.2):
        """SearchByProjection(CurrentFrame, LastFrame, th, bMono) -> (nmatches, match_out)."""
        kps = np.ascontiguousarray(kps, KP_DTYPE)
        desc = np.ascontiguousarray(desc, np.uint8)
        last_kps = np.ascontiguousarray(last_kps, KP_DTYPE)
        last_mps = np.ascontiguousarray(last_mps, FMP_DTYPE)
        last_mp_desc = np.ascontiguousarray(last_mp_desc, np.uint8)
        ur = None if uright is None else np.ascontiguousarray(uright, np.float32)
        cl = None if claimed is None else np.ascontiguousarray(claimed, np.uint8)
        out = np.zeros(max(len(kps), 1), np.int32)
        p = Params(1000, scale_factor, nlevels, 20, 7)
        f = self.fn("search_by_projection_frame")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int,
                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        nm = f(C.byref(p), _p(kps), _p(desc), _p(ur), len(kps), w, h, _p(last_kps), len(last_kps), _p(last_mps),
               _p(last_mp_desc), C.byref(motion), th, int(bool(mono)), int(bool(check_ori)), _p(cl), _p(out))
        return int(nm), out[:len(kps)].copy()

    def compute_stereo_matches(self, kpsL, descL, kpsR, descR, pyrL, pyrR, w, h, bf, fx, nlevels=8,
                               scale_factor=1.2):
        kpsL = np.ascontiguousarray(kpsL, KP_DTYPE)
        kpsR = np.ascontiguousarray(kpsR, KP_DTYPE)
        descL = np.ascontiguousarray(descL, np.uint8)
        descR = np.ascontiguousarray(descR, np.uint8)
        lw = np.array([l.shape[1] for l in pyrL], np.int32)
        lh = np.array([l.shape[0] for l in pyrL], np.int32)
        pl = np.ascontiguousarray(np.concatenate([l.ravel() for l in pyrL]))
        pr = np.ascontiguousarray(np.concatenate([l.ravel() for l in pyrR]))
        ur = np.zeros(max(len(kpsL), 1), np.float32)
        dp = np.zeros(max(len(kpsL), 1), np.float32)
        p = Params(1000, scale_factor, nlevels, 20, 7)
        f = self.fn("compute_stereo_matches")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p,
                      C.c_void_p]
        f(C.byref(p), _p(kpsL), _p(descL), len(kpsL), _p(kpsR), _p(descR), len(kpsR), _p(pl), _p(pr), _p(lw),
          _p(lh), w, h, bf, fx, _p(ur), _p(dp))
        return ur[:len(kpsL)].copy(), dp[:len(kpsL)].copy()

    def knn2(self, q, t):
        q = np.ascontiguousarray(q, np.uint8)
        t = np.ascontiguousarray(t, np.uint8)
        nq = len(q)
        outs = [np.zeros(max(nq, 1), np.int32) for _ in range(4)]
        self.fn("knn2")(_p(q), nq, _p(t), len(t), *[_p(o) for o in outs])
        return tuple(o[:nq].copy() for o in outs)


    def vocabulary_load(self, path):
        """TemplatedVocabulary::loadFromTextFile; the word count, -1 on failure."""
        f = self.fn("vocabulary_load")
        f.argtypes = [C.c_char_p]
        return int(f(path.encode()))

    def vocabulary_from_arrays(self, name, voc):
        """The tree of a synthetic.vocabulary dict, stored under name (oracle only)."""
        par = np.ascontiguousarray(voc["parents"], np.int32)
        lf = np.ascontiguousarray(voc["is_leaf"], np.uint8)
        d = np.ascontiguousarray(voc["descriptors"], np.uint8)
        w = np.ascontiguousarray(voc["weights"], np.float64)
        f = self.lib.orc_vocabulary_from_arrays
        f.argtypes = [C.c_char_p] + [C.c_int] * 5 + [C.c_void_p] * 4
        return int(f(name.encode(), int(voc["k"]), int(voc["L"]), int(voc["scoring"]), int(voc["weighting"]),
                     len(par) + 1, _p(par), _p(lf), _p(d), _p(w)))

    def bow_transform(self, path, desc, levelsup=4):
        """TemplatedVocabulary::transform(features, BowVector, FeatureVector,
        levelsup) with the vocabulary loaded from path."""
        desc = np.ascontiguousarray(desc, np.uint8).reshape(-1, 32)
        n = len(desc)
        m = max(n, 1)
        word, node = np.zeros(m, np.int32), np.zeros(m, np.int32)
        weight = np.zeros(m, np.float64)
        bw, bv = np.zeros(m, np.int32), np.zeros(m, np.float64)
        fn, fo, ff = np.zeros(m, np.int32), np.zeros(m + 1, np.int32), np.zeros(m, np.int32)
        bn, fnn = C.c_int(0), C.c_int(0)
        f = self.fn("bow_transform")
        f.argtypes = [C.c_char_p, C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 3 + [C.c_void_p] * 3 + \
            [C.c_void_p] * 4
        rc = f(path.encode(), _p(desc), n, levelsup, _p(word), _p(weight), _p(node), C.byref(bn), _p(bw), _p(bv),
               C.byref(fnn), _p(fn), _p(fo), _p(ff))
        if rc != 0:
            raise RuntimeError("vocabulary not loaded")
        b, q = bn.value, fnn.value
        return {"word": word[:n].copy(), "weight": weight[:n].copy(), "node": node[:n].copy(),
                "bow_words": bw[:b].copy(), "bow_values": bv[:b].copy(), "fv_nodes": fn[:q].copy(),
                "fv_offsets": fo[:q + 1].copy(), "fv_features": ff[:fo[q]].copy()}

    def search_by_projection_kf(self, kps, desc, w, h, Tcw, cam, kf_kps, mps, mp_desc, mp_state, th=10.0,
                                orbdist=100, check_ori=True, claimed=None, nlevels=8, scale_factor=1.2):
        """SearchByProjection(Frame&, KeyFrame*, sAlreadyFound, th, ORBdist)
        -> (nmatches, match_out).  mps: GEOM_DTYPE; mp_state 0 none, 1 usable,
        2 bad, 3 already found; cam: fx, fy, cx, cy."""
        kps = np.ascontiguousarray(kps, KP_DTYPE)
        desc = np.ascontiguousarray(desc, np.uint8)
        kf_kps = np.ascontiguousarray(kf_kps, KP_DTYPE)
        mps = np.ascontiguousarray(mps, GEOM_DTYPE)
        mpd = np.ascontiguousarray(mp_desc, np.uint8)
        st = np.ascontiguousarray(mp_state, np.uint8)
        T = np.ascontiguousarray(np.asarray(Tcw, np.float32).reshape(-1)[:12])
        cm = np.ascontiguousarray(cam, np.float32)
        cl = None if claimed is None else np.ascontiguousarray(claimed, np.uint8)
        out = np.zeros(max(len(kps), 1), np.int32)
        p = Params(1000, scale_factor, nlevels, 20, 7)
        f = self.fn("search_by_projection_kf")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                      C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_int, C.c_int,
                      C.c_void_p, C.c_void_p]
        nm = f(C.byref(p), _p(kps), _p(desc), len(kps), w, h, _p(T), _p(cm), _p(kf_kps), len(kf_kps), _p(mps),
               _p(mpd), _p(st), C.c_float(th), int(orbdist), int(bool(check_ori)), _p(cl), _p(out))
        return int(nm), out[:len(kps)].copy()

    def search_by_projection_sim3(self, kps, desc, w, h, Scw, cam, pts, pdesc, pstate, th=10, claimed=None,
                                  nlevels=8, scale_factor=1.2):
        """SearchByProjection(KeyFrame*, Scw, vpPoints, vpMatched, th) ->
        (nmatches, match_out per keyframe keypoint)."""
        kps = np.ascontiguousarray(kps, KP_DTYPE)
        desc = np.ascontiguousarray(desc, np.uint8)
        S = np.ascontiguousarray(np.asarray(Scw, np.float32).reshape(-1)[:12])
        cm = np.ascontiguousarray(cam, np.float32)
        pts = np.ascontiguousarray(pts, GEOM_DTYPE)
        pd = np.ascontiguousarray(pdesc, np.uint8)
        ps = np.ascontiguousarray(pstate, np.uint8)
        cl = None if claimed is None else np.ascontiguousarray(claimed, np.uint8)
        out = np.zeros(max(len(kps), 1), np.int32)
        p = Params(1000, scale_factor, nlevels, 20, 7)
        f = self.fn("search_by_projection_sim3")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        nm = f(C.byref(p), _p(kps), _p(desc), len(kps), w, h, _p(S), _p(cm), _p(pts), _p(pd), _p(ps), len(pts),
               int(th), _p(cl), _p(out))
        return int(nm), out[:len(kps)].copy()

    def fuse_candidates(self, kps, desc, uright, w, h, Tcw, cam, mps, mp_desc, mp_state, th=3.0, nlevels=8,
                        scale_factor=1.2):
        """Fuse(KeyFrame*, vpMapPoints, th): the keyframe feature each map point
        fuses with -> (count, target).  cam: fx, fy, cx, cy, bf."""
        kps = np.ascontiguousarray(kps, KP_DTYPE)
        desc = np.ascontiguousarray(desc, np.uint8)
        ur = None if uright is None else np.ascontiguousarray(uright, np.float32)
        T = np.ascontiguousarray(np.asarray(Tcw, np.float32).reshape(-1)[:12])
        cm = np.ascontiguousarray(cam, np.float32)
        mps = np.ascontiguousarray(mps, GEOM_DTYPE)
        mpd = np.ascontiguousarray(mp_desc, np.uint8)
        st = np.ascontiguousarray(mp_state, np.uint8)
        out = np.zeros(max(len(mps), 1), np.int32)
        p = Params(1000, scale_factor, nlevels, 20, 7)
        f = self.fn("fuse_candidates")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_void_p]
        nf = f(C.byref(p), _p(kps), _p(desc), _p(ur), len(kps), w, h, _p(T), _p(cm), _p(mps), _p(mpd), _p(st),
               len(mps), C.c_float(th), _p(out))
        return int(nf), out[:len(mps)].copy()

    def fuse_sim3_candidates(self, kps, desc, w, h, Scw, cam, pts, pdesc, pstate, th=4.0, nlevels=8,
                             scale_factor=1.2):
        """Fuse(KeyFrame*, Scw, vpPoints, th, vpReplacePoint): each point's
        choice -> (count, target).  cam: fx, fy, cx, cy."""
        kps = np.ascontiguousarray(kps, KP_DTYPE)
        desc = np.ascontiguousarray(desc, np.uint8)
        S = np.ascontiguousarray(np.asarray(Scw, np.float32).reshape(-1)[:12])
        cm = np.ascontiguousarray(cam, np.float32)
        pts = np.ascontiguousarray(pts, GEOM_DTYPE)
        pd = np.ascontiguousarray(pdesc, np.uint8)
        ps = np.ascontiguousarray(pstate, np.uint8)
        out = np.zeros(max(len(pts), 1), np.int32)
        p = Params(1000, scale_factor, nlevels, 20, 7)
        f = self.fn("fuse_sim3_candidates")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_void_p]
        nf = f(C.byref(p), _p(kps), _p(desc), len(kps), w, h, _p(S), _p(cm), _p(pts), _p(pd), _p(ps), len(pts),
               C.c_float(th), _p(out))
        return int(nf), out[:len(pts)].copy()

    def search_by_sim3(self, kps1, desc1, kps2, desc2, w, h, T1w, T2w, s12, R12, t12, cam, mps1, mpd1, st1, mps2,
                       mpd2, st2, th=7.5, nlevels=8, scale_factor=1.2, pre12=None):
        """SearchBySim3(pKF1, pKF2, vpMatches12, s12, R12, t12, th) ->
        (nfound, match12 over pKF1's features).  st1 / st2: 0 no map point,
        1 usable, 2 bad.  pre12: vpMatches12 entries already set (pKF2
        feature index, -1 none) -- the reference build receives them as map
        points (match12 then reports them), the restatement as skipped
        features on both sides (match12 -1 there)."""
        ref = self.prefix == "ref_"
        if pre12 is not None and not ref:
            pre = np.asarray(pre12)
            st1 = np.where(pre >= 0, 0, np.asarray(st1)).astype(np.uint8)
            st2 = np.asarray(st2).astype(np.uint8).copy()
            st2[pre[pre >= 0]] = 0
        a = [np.ascontiguousarray(kps1, KP_DTYPE), np.ascontiguousarray(desc1, np.uint8),
             np.ascontiguousarray(kps2, KP_DTYPE), np.ascontiguousarray(desc2, np.uint8)]
        fl = [np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1)) for x in (T1w, T2w, R12, t12, cam)]
        g1 = np.ascontiguousarray(mps1, GEOM_DTYPE)
        g2 = np.ascontiguousarray(mps2, GEOM_DTYPE)
        d1, d2 = np.ascontiguousarray(mpd1, np.uint8), np.ascontiguousarray(mpd2, np.uint8)
        s1, s2 = np.ascontiguousarray(st1, np.uint8), np.ascontiguousarray(st2, np.uint8)
        out = np.zeros(max(len(a[0]), 1), np.int32)
        p = Params(1000, scale_factor, nlevels, 20, 7)
        f = self.fn("search_by_sim3")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                      C.c_int, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p] + \
            [C.c_void_p] * 6 + [C.c_float] + ([C.c_void_p] if ref else []) + [C.c_void_p]
        pre = [_p(np.ascontiguousarray(pre12, np.int32)) if pre12 is not None else None] if ref else []
        nf = f(C.byref(p), _p(a[0]), _p(a[1]), len(a[0]), _p(a[2]), _p(a[3]), len(a[2]), w, h, _p(fl[0]), _p(fl[1]),
               C.c_float(s12), _p(fl[2]), _p(fl[3]), _p(fl[4]), _p(g1), _p(d1), _p(s1), _p(g2), _p(d2), _p(s2),
               C.c_float(th), *pre, _p(out))
        return int(nf), out[:len(a[0])].copy()

    def search_for_triangulation(self, kps1, desc1, mp1, ur1, fv1, kps2, desc2, mp2, ur2, fv2, Cw1, T2, K2, F12,
                                 scale, sigma2, only_stereo=False, check_ori=True):
        """SearchForTriangulation(pKF1, pKF2, F12, pairs, bOnlyStereo) ->
        (nmatches, match_out over pKF1's features)."""
        a1 = [np.ascontiguousarray(kps1, KP_DTYPE), np.ascontiguousarray(desc1, np.uint8),
              np.ascontiguousarray(mp1, np.uint8), np.ascontiguousarray(ur1, np.float32)]
        a2 = [np.ascontiguousarray(kps2, KP_DTYPE), np.ascontiguousarray(desc2, np.uint8),
              np.ascontiguousarray(mp2, np.uint8), np.ascontiguousarray(ur2, np.float32)]
        f1 = [np.ascontiguousarray(x, np.int32) for x in fv1]
        f2 = [np.ascontiguousarray(x, np.int32) for x in fv2]
        fl = [np.ascontiguousarray(np.asarray(x, np.float32).reshape(-1)) for x in (Cw1, T2, K2, F12)]
        sc = np.zeros(16, np.float32)
        sg = np.zeros(16, np.float32)
        sc[:len(scale)] = scale
        sg[:len(sigma2)] = sigma2
        out = np.zeros(max(len(a1[0]), 1), np.int32)
        f = self.fn("search_for_triangulation")
        f.argtypes = ([C.c_void_p] * 4 + [C.c_int] * 2 + [C.c_void_p] * 3) * 2 + [C.c_void_p] * 6 + \
            [C.c_int, C.c_int, C.c_void_p]
        nm = f(*[_p(x) for x in a1], len(a1[0]), len(f1[0]), *[_p(x) for x in f1],
               *[_p(x) for x in a2], len(a2[0]), len(f2[0]), *[_p(x) for x in f2],
               *[_p(x) for x in fl], _p(sc), _p(sg), int(bool(only_stereo)), int(bool(check_ori)), _p(out))
        return int(nm), out[:len(a1[0])].copy()

    def search_by_bow(self, kf_kps, kf_desc, kf_mp, kf_fv, f_kps, f_desc, f_fv, nnratio=0.75, check_ori=True):
        """ORBmatcher::SearchByBoW(KeyFrame*, Frame&, matches).  *_fv: (nodes,
        offsets, features) of the FeatureVector (bow_transform's fv_*);
        kf_mp: 0 none, 1 a map point, 2 a bad one.  -> (nmatches, match_out)."""
        kf_kps = np.ascontiguousarray(kf_kps, KP_DTYPE)
        f_kps = np.ascontiguousarray(f_kps, KP_DTYPE)
        kf_desc = np.ascontiguousarray(kf_desc, np.uint8)
        f_desc = np.ascontiguousarray(f_desc, np.uint8)
        kf_mp = np.ascontiguousarray(kf_mp, np.uint8)
        kn, ko, kfe = (np.ascontiguousarray(a, np.int32) for a in kf_fv)
        fn_, fo, ffe = (np.ascontiguousarray(a, np.int32) for a in f_fv)
        out = np.zeros(max(len(f_kps), 1), np.int32)
        f = self.fn("search_by_bow")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                      C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                      C.c_int, C.c_void_p]
        nm = f(_p(kf_kps), _p(kf_desc), _p(kf_mp), len(kf_kps), len(kn), _p(kn), _p(ko), _p(kfe), _p(f_kps),
               _p(f_desc), len(f_kps), len(fn_), _p(fn_), _p(fo), _p(ffe), C.c_float(nnratio), int(bool(check_ori)),
               _p(out))
        return int(nm), out[:len(f_kps)].copy()

    def search_by_bow_kf(self, kps1, desc1, mp1, fv1, kps2, desc2, mp2, fv2, nnratio=0.75, check_ori=True):
        """ORBmatcher::SearchByBoW(KeyFrame*, KeyFrame*, vpMatches12) ->
        (nmatches, match_out over pKF1's features: pKF2 feature or -1)."""
        kps1 = np.ascontiguousarray(kps1, KP_DTYPE)
        kps2 = np.ascontiguousarray(kps2, KP_DTYPE)
        d1 = np.ascontiguousarray(desc1, np.uint8)
        d2 = np.ascontiguousarray(desc2, np.uint8)
        m1 = np.ascontiguousarray(mp1, np.uint8)
        m2 = np.ascontiguousarray(mp2, np.uint8)
        a = [np.ascontiguousarray(x, np.int32) for x in fv1]
        b = [np.ascontiguousarray(x, np.int32) for x in fv2]
        out = np.zeros(max(len(kps1), 1), np.int32)
        f = self.fn("search_by_bow_kf")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                      C.c_float, C.c_int, C.c_void_p]
        nm = f(_p(kps1), _p(d1), _p(m1), len(kps1), len(a[0]), _p(a[0]), _p(a[1]), _p(a[2]), _p(kps2), _p(d2),
               _p(m2), len(kps2), len(b[0]), _p(b[0]), _p(b[1]), _p(b[2]), C.c_float(nnratio), int(bool(check_ori)),
               _p(out))
        return int(nm), out[:len(kps1)].copy()

    def undistort_keypoints(self, K4, dist, kps):
        """Frame::UndistortKeyPoints: the keypoints with undistorted x, y."""
        K = np.ascontiguousarray(K4, np.float32)
        d = np.ascontiguousarray(dist, np.float32)
        kps = np.ascontiguousarray(kps, KP_DTYPE)
        out = np.zeros(max(len(kps), 1), KP_DTYPE)
        f = self.fn("undistort_keypoints")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]
        f(_p(K), _p(d), len(d), _p(kps), len(kps), _p(out))
        return out[:len(kps)].copy()

    def compute_image_bounds(self, cols, rows, K4, dist):
        """Frame::ComputeImageBounds -> (mnMinX, mnMaxX, mnMinY, mnMaxY)."""
        K = np.ascontiguousarray(K4, np.float32)
        d = np.ascontiguousarray(dist, np.float32)
        b = np.zeros(4, np.float32)
        f = self.fn("compute_image_bounds")
        f.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        f(int(cols), int(rows), _p(K), _p(d), len(d), _p(b))
        return b

    def is_in_frustum(self, cam, mps, cos_limit=0.5, initial=None):
        """Frame::isInFrustum for every map point (GEOM_DTYPE records) of one
        frame; returns (MP_DTYPE records after the call, number in view)."""
        mps = np.ascontiguousarray(mps, GEOM_DTYPE)
        out = (np.zeros(max(len(mps), 1), MP_DTYPE) if initial is None
               else np.ascontiguousarray(np.array(initial, MP_DTYPE)))
        f = self.fn("is_in_frustum")
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_float, C.c_void_p]
        n = f(C.byref(cam), _p(mps), len(mps), C.c_float(cos_limit), _p(out))
        return out[:len(mps)].copy(), int(n)

    def distinctive_descriptors(self, pool, offsets, rows, initial=None):
        """MapPoint::ComputeDistinctiveDescriptors over ragged observation lists
        (src/MapPoint.cc:365-447); returns (best_rows, descriptors)."""
        pool = np.ascontiguousarray(pool, np.uint8).reshape(-1, 32)
        offsets = np.ascontiguousarray(offsets, np.int32)
        rows = np.ascontiguousarray(rows, np.int32)
        m = len(offsets) - 1
        best = np.zeros(max(m, 1), np.int32)
        desc = (np.zeros((max(m, 1), 32), np.uint8) if initial is None
                else np.ascontiguousarray(np.array(initial, np.uint8).reshape(-1, 32)))
        f = self.fn("distinctive_descriptors")
        f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        f(_p(pool), len(pool), _p(offsets), _p(rows), m, _p(best), _p(desc))
        return best[:m].copy(), desc[:m].copy()


class Oracle(_Base):
    def __init__(self, path: str = ORACLE_SO):
        super().__init__(path)

    def predict_scale(self, ratio, scale_factor=1.2, nlevels=8):
        """MapPoint::PredictScale on ratios mfMaxDistance / currentDist."""
        r = np.ascontiguousarray(ratio, np.float32)
        out = np.zeros(max(len(r), 1), np.int32)
        f = self.lib.orc_predict_scale
        f.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_int, C.c_void_p]
        f(_p(r), len(r), C.c_float(scale_factor), nlevels, _p(out))
        return out[:len(r)].copy()


class RefOracle(_Base):
    def __init__(self, path: str = REF_SO):
        super().__init__(path)


def ref_available() -> bool:
    return os.path.exists(REF_SO)
