"""ORBmatcher and Frame::ComputeStereoMatches on the GPU, with the
reference's interfaces (include/ORBmatcher.h, src/Frame.cc:831)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._lib import (FRAME_MAPPOINT_DTYPE, KEYPOINT_DTYPE, MAPPOINT_DTYPE, MEM_DEVICE, MEM_HOST, FrameStruct,
                   MotionStruct, check, lib, ptr)


def _is_cuda(a) -> bool:
    return hasattr(a, "is_cuda") and bool(a.is_cuda)


def _cpu(a):
    return a.cpu().numpy() if _is_cuda(a) else a


@dataclass
class FrameView:
    """The fields of ORB_SLAM2::Frame that the searches read.

    keypoints: structured KEYPOINT_DTYPE array (host) or an (n, 7) float32
    CUDA tensor with the same 28-byte records; descriptors: n x 32 uint8.
    width/height: image bounds of the 64 x 48 grid (no distortion).
    """
    keypoints: object
    descriptors: object
    width: int
    height: int
    scale_factors: object
    uright: object = None
    # read by SearchByProjection(CurrentFrame, LastFrame, th, bMono) only:
    # pose (rows 0-2 of mTcw), intrinsics and stereo constants of the frame,
    # its map points (FRAME_MAPPOINT_DTYPE records, one per keypoint) with
    # their descriptors, and which keypoints already hold an observed map point
    Tcw: object = None
    fx: float = 0.0
    fy: float = 0.0
    cx: float = 0.0
    cy: float = 0.0
    mbf: float = 0.0
    mb: float = 0.0
    mappoints: object = None
    mp_descriptors: object = None
    claimed: object = None
    _keep: list = field(default_factory=list, repr=False)

    def struct(self) -> FrameStruct:
        dev = _is_cuda(self.descriptors)
        kps = self.keypoints
        desc = self.descriptors
        ur = self.uright
        if not dev:
            kps = np.ascontiguousarray(kps, KEYPOINT_DTYPE)
            desc = np.ascontiguousarray(desc, np.uint8)
            ur = None if ur is None else np.ascontiguousarray(ur, np.float32)
        self._keep = [kps, desc, ur]
        s = FrameStruct()
        s.keypoints = ptr(kps).value
        s.descriptors = ptr(desc).value
        s.uright = ptr(ur).value if ur is not None else None
        s.n = int(kps.shape[0])
        s.width = int(self.width)
        s.height = int(self.height)
        sf = np.asarray(self.scale_factors, np.float32)
        s.nlevels = int(len(sf))
        for i, v in enumerate(sf[:16]):
            s.scale_factors[i] = float(v)
        s.mem = MEM_DEVICE if dev else MEM_HOST
        return s


class ORBmatcher:
    """ORB_SLAM2::ORBmatcher(nnratio=0.6, checkOri=true)."""

    TH_HIGH = 100
    TH_LOW = 50
    HISTO_LENGTH = 30

    def __init__(self, nnratio: float = 0.6, checkOri: bool = True, stream=None):
        self._h = C.c_void_p()
        st = C.c_void_p(0 if stream is None else int(stream))
        check(lib().orbgpu_matcher_create(C.c_float(nnratio), int(bool(checkOri)), st, C.byref(self._h)),
              "orbgpu_matcher_create")
        self.mfNNratio = nnratio
        self.mbCheckOrientation = checkOri

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            try:
                lib().orbgpu_matcher_destroy(h)
            except Exception:
                pass
            self._h = None

    @property
    def handle(self):
        return self._h

    def SearchForInitialization(self, F1: FrameView, F2: FrameView, vbPrevMatched, windowSize: int = 10):
        """Returns (nmatches, vnMatches12, vbPrevMatched updated) -- src/ORBmatcher.cc:573-717."""
        s1, s2 = F1.struct(), F2.struct()
        prev = np.ascontiguousarray(vbPrevMatched, np.float32).copy()
        m12 = np.full(max(s1.n, 1), -1, np.int32)
        nm = C.c_int(0)
        check(lib().orbgpu_search_for_initialization(self._h, C.byref(s1), C.byref(s2), ptr(prev), ptr(m12),
                                                     int(windowSize), C.byref(nm)),
              "orbgpu_search_for_initialization")
        return nm.value, m12[:s1.n], prev

    def SearchByProjection(self, F: FrameView, second, *args, **kw):
        """The two SearchByProjection overloads on a Frame:

        SearchByProjection(F, mappoints, mp_descriptors, th=1.0, claimed=None)
            -- (Frame&, vector<MapPoint*>, th), src/ORBmatcher.cc:72-183;
            match[i] = map point index assigned to keypoint i (-2 pre-claimed,
            -1 none).
        SearchByProjection(CurrentFrame, LastFrame, th, bMono)
            -- (Frame&, const Frame&, th, bMono), src/ORBmatcher.cc:1710-1879;
            match[i] = LastFrame keypoint whose map point fills
            CurrentFrame.mvpMapPoints[i] (-1 not assigned, -2 pre-claimed, -4
            reset by the rotation check).
        Both return (nmatches, match)."""
        if isinstance(second, FrameView):
            return self._search_by_projection_frame(F, second, *args, **kw)
        return self._search_by_projection_mappoints(F, second, *args, **kw)

    def _search_by_projection_frame(self, CF: FrameView, LF: FrameView, th: float, bMono: bool):
        sc, sl = CF.struct(), LF.struct()
        dev = sc.mem == MEM_DEVICE
        mo = MotionStruct()
        for i, v in enumerate(np.asarray(_cpu(CF.Tcw), np.float32).reshape(-1)[:12]):
            mo.Tcw[i] = float(v)
        for i, v in enumerate(np.asarray(_cpu(LF.Tcw), np.float32).reshape(-1)[:12]):
            mo.Tlw[i] = float(v)
        mo.fx, mo.fy, mo.cx, mo.cy, mo.bf, mo.b = (float(np.float32(v)) for v in
                                                   (CF.fx, CF.fy, CF.cx, CF.cy, CF.mbf, CF.mb))
        nm = C.c_int(0)
        if dev:
            import torch
            out = torch.empty(max(sc.n, 1), dtype=torch.int32, device="cuda")
            mps, mpd, cl = LF.mappoints, LF.mp_descriptors, CF.claimed
        else:
            out = np.zeros(max(sc.n, 1), np.int32)
            mps = np.ascontiguousarray(LF.mappoints, FRAME_MAPPOINT_DTYPE)
            mpd = np.ascontiguousarray(LF.mp_descriptors, np.uint8)
            cl = None if CF.claimed is None else np.ascontiguousarray(CF.claimed, np.uint8)
        if sl.n and (int(mpd.shape[0]) < sl.n or
                     (mps.nbytes if isinstance(mps, np.ndarray) else mps.numel() * mps.element_size()) < sl.n * 16):
            raise ValueError("LastFrame needs one map point record and descriptor per keypoint")
        check(lib().orbgpu_search_by_projection_frame(self._h, C.byref(sc), C.byref(sl), ptr(mps), ptr(mpd),
                                                      C.byref(mo), C.c_float(th), int(bool(bMono)), ptr(cl), ptr(out),
                                                      MEM_DEVICE if dev else MEM_HOST, C.byref(nm)),
              "orbgpu_search_by_projection_frame")
        return nm.value, out[:sc.n]

    def SearchByProjectionKeyFrame(self, F: FrameView, pose, kf_keypoints, mappoints, mp_descriptors, usable,
                                   th: float, orbdist: int, claimed=None):
        """SearchByProjection(Frame& CurrentFrame, KeyFrame* pKF, const
        set<MapPoint*>& sAlreadyFound, th, ORBdist) -- src/ORBmatcher.cc:1891-2010.

        pose: CurrentFrame's FRUSTUM_FRAME_DTYPE record (frustum_frame);
        per keyframe feature: kf_keypoints (KEYPOINT_DTYPE), mappoints
        (MAPPOINT_GEOMETRY_DTYPE rows), mp_descriptors (m x 32), usable (1
        where the map point exists, is not bad and not already found).  Host
        arrays, or CUDA tensors when F is on the device.  Returns (nmatches,
        match): per keypoint the keyframe feature whose map point it got, -1,
        -2 claimed before, -4 reset by the rotation check."""
        from ._lib import FRUSTUM_FRAME_DTYPE
        s = F.struct()
        dev = s.mem == MEM_DEVICE
        nm = C.c_int(0)
        rec = np.ascontiguousarray(np.array(pose, FRUSTUM_FRAME_DTYPE).reshape(-1)[:1])
        if dev:
            import torch
            out = torch.empty(max(s.n, 1), dtype=torch.int32, device="cuda")
            kk, mps, mpd, use, cl = kf_keypoints, mappoints, mp_descriptors, usable, claimed
            m = int(mpd.shape[0])
        else:
            out = np.zeros(max(s.n, 1), np.int32)
            kk = np.ascontiguousarray(kf_keypoints, KEYPOINT_DTYPE)
            mps = np.ascontiguousarray(np.asarray(mappoints, np.float32).reshape(-1, 8))
            mpd = np.ascontiguousarray(mp_descriptors, np.uint8)
            use = np.ascontiguousarray(usable, np.uint8)
            cl = None if claimed is None else np.ascontiguousarray(claimed, np.uint8)
            m = len(mpd)
            assert mps.shape[0] == m and len(kk) == m and len(use) == m
        check(lib().orbgpu_search_by_projection_keyframe(self._h, C.byref(s), ptr(rec), ptr(kk), ptr(mps), ptr(mpd),
                                                         ptr(use), m, C.c_float(th), int(orbdist), ptr(cl), ptr(out),
                                                         MEM_DEVICE if dev else MEM_HOST, C.byref(nm)),
              "orbgpu_search_by_projection_keyframe")
        return nm.value, out[:s.n]

    def SearchByProjectionSim3(self, KF: FrameView, Scw, fx, fy, cx, cy, points, point_descriptors, usable, th: int,
                               matched=None, scale_factor: float = 1.2, nlevels: int = 8):
        """SearchByProjection(KeyFrame* pKF, cv::Mat Scw, vpPoints, vpMatched, th)
        -- src/ORBmatcher.cc:423-560 (loop closing).  KF: the keyframe's
        keypoints / descriptors; Scw rows 0-2; points (MAPPOINT_GEOMETRY_DTYPE
        rows incl. normals), point_descriptors, usable (not bad, not already
        in vpMatched); matched: keypoints whose vpMatched entry is set.
        Returns (nmatches, match): per keypoint the point index now in
        vpMatched, -2 set before, -1 none."""
        s = KF.struct()
        dev = s.mem == MEM_DEVICE
        nm = C.c_int(0)
        S = np.ascontiguousarray(np.asarray(Scw, np.float32).reshape(-1)[:12])
        if dev:
            import torch
            out = torch.empty(max(s.n, 1), dtype=torch.int32, device="cuda")
            pts, pd, use, cl = points, point_descriptors, usable, matched
            m = int(pd.shape[0])
        else:
            out = np.zeros(max(s.n, 1), np.int32)
            pts = np.ascontiguousarray(np.asarray(points, np.float32).reshape(-1, 8))
            pd = np.ascontiguousarray(point_descriptors, np.uint8)
            use = np.ascontiguousarray(usable, np.uint8)
            cl = None if matched is None else np.ascontiguousarray(matched, np.uint8)
            m = len(pd)
        check(lib().orbgpu_search_by_projection_sim3(self._h, C.byref(s), ptr(S), C.c_float(fx), C.c_float(fy),
                                                     C.c_float(cx), C.c_float(cy), C.c_float(scale_factor),
                                                     int(nlevels), ptr(pts), ptr(pd), ptr(use), m, int(th), ptr(cl),
                                                     ptr(out), MEM_DEVICE if dev else MEM_HOST, C.byref(nm)),
              "orbgpu_search_by_projection_sim3")
        return nm.value, out[:s.n]

    def FuseCandidates(self, KF: FrameView, Tcw, fx, fy, cx, cy, bf, inv_level_sigma2, mappoints, mp_descriptors,
                       usable, th: float = 3.0, scale_factor: float = 1.2, nlevels: int = 8):
        """The search half of Fuse(KeyFrame* pKF, vpMapPoints, th) --
        src/ORBmatcher.cc:1107-1245: per map point the keyframe feature it
        fuses with (-1 none) and the distance.  KF carries pKF's keypoints,
        descriptors and mvuRight; the map updates (Replace / AddObservation)
        are applied by the caller in vpMapPoints order.  Host arrays, or CUDA
        tensors when KF is on the device.  Returns (target, dist)."""
        s = KF.struct()
        dev = s.mem == MEM_DEVICE
        T = np.ascontiguousarray(np.asarray(Tcw, np.float32).reshape(-1)[:12])
        isg = np.ascontiguousarray(inv_level_sigma2, np.float32)
        if dev:
            import torch
            mps, mpd, use = mappoints, mp_descriptors, usable
            m = int(mpd.shape[0])
            target = torch.empty(max(m, 1), dtype=torch.int32, device="cuda")
            dist = torch.empty(max(m, 1), dtype=torch.int32, device="cuda")
        else:
            mps = np.ascontiguousarray(np.asarray(mappoints, np.float32).reshape(-1, 8))
            mpd = np.ascontiguousarray(mp_descriptors, np.uint8)
            use = np.ascontiguousarray(usable, np.uint8)
            m = len(mpd)
            target = np.zeros(max(m, 1), np.int32)
            dist = np.zeros(max(m, 1), np.int32)
        check(lib().orbgpu_fuse_candidates(self._h, C.byref(s), ptr(T), C.c_float(fx), C.c_float(fy), C.c_float(cx),
                                           C.c_float(cy), C.c_float(bf), C.c_float(scale_factor), int(nlevels),
                                           ptr(isg), ptr(mps), ptr(mpd), ptr(use), m, C.c_float(th), ptr(target),
                                           ptr(dist), MEM_DEVICE if dev else MEM_HOST),
              "orbgpu_fuse_candidates")
        return target[:m], dist[:m]

    def FuseSim3Candidates(self, KF: FrameView, Scw, fx, fy, cx, cy, points, point_descriptors, usable,
                           th: float = 4.0, scale_factor: float = 1.2, nlevels: int = 8):
        """The search half of Fuse(KeyFrame* pKF, cv::Mat Scw, vpPoints, th,
        vpReplacePoint) -- src/ORBmatcher.cc:1290-1380: per point the keyframe
        feature it fuses with (-1 none) and the distance; the caller fills
        vpReplacePoint / adds observations in order.  Returns (target, dist)."""
        s = KF.struct()
        dev = s.mem == MEM_DEVICE
        S = np.ascontiguousarray(np.asarray(Scw, np.float32).reshape(-1)[:12])
        if dev:
            import torch
            pts, pd, use = points, point_descriptors, usable
            m = int(pd.shape[0])
            target = torch.empty(max(m, 1), dtype=torch.int32, device="cuda")
            dist = torch.empty(max(m, 1), dtype=torch.int32, device="cuda")
        else:
            pts = np.ascontiguousarray(np.asarray(points, np.float32).reshape(-1, 8))
            pd = np.ascontiguousarray(point_descriptors, np.uint8)
            use = np.ascontiguousarray(usable, np.uint8)
            m = len(pd)
            target = np.zeros(max(m, 1), np.int32)
            dist = np.zeros(max(m, 1), np.int32)
        check(lib().orbgpu_fuse_sim3_candidates(self._h, C.byref(s), ptr(S), C.c_float(fx), C.c_float(fy),
                                                C.c_float(cx), C.c_float(cy), C.c_float(scale_factor), int(nlevels),
                                                ptr(pts), ptr(pd), ptr(use), m, C.c_float(th), ptr(target), ptr(dist),
                                                MEM_DEVICE if dev else MEM_HOST),
              "orbgpu_fuse_sim3_candidates")
        return target[:m], dist[:m]

    def SearchBySim3(self, KF1: FrameView, KF2: FrameView, T1w, T2w, s12, R12, t12, fx, fy, cx, cy, mps1, mpd1,
                     usable1, mps2, mpd2, usable2, th: float = 7.5, scale_factor: float = 1.2, nlevels: int = 8):
        """SearchBySim3(pKF1, pKF2, vpMatches12, s12, R12, t12, th) --
        src/ORBmatcher.cc:1441-1640 (host arrays).  Returns (nfound, match12:
        per pKF1 feature the pKF2 feature whose map point vpMatches12 gets, or
        -1)."""
        s1, s2 = KF1.struct(), KF2.struct()
        out = np.zeros(max(s1.n, 1), np.int32)
        nf = C.c_int(0)
        arrs = [np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1)) for a in (T1w, T2w, R12, t12)]
        g1 = np.ascontiguousarray(np.asarray(mps1, np.float32).reshape(-1, 8))
        g2 = np.ascontiguousarray(np.asarray(mps2, np.float32).reshape(-1, 8))
        d1, d2 = np.ascontiguousarray(mpd1, np.uint8), np.ascontiguousarray(mpd2, np.uint8)
        u1, u2 = np.ascontiguousarray(usable1, np.uint8), np.ascontiguousarray(usable2, np.uint8)
        check(lib().orbgpu_search_by_sim3(self._h, C.byref(s1), C.byref(s2), ptr(arrs[0]), ptr(arrs[1]),
                                          C.c_float(s12), ptr(arrs[2]), ptr(arrs[3]), C.c_float(fx), C.c_float(fy),
                                          C.c_float(cx), C.c_float(cy), C.c_float(scale_factor), int(nlevels), ptr(g1),
                                          ptr(d1), ptr(u1), ptr(g2), ptr(d2), ptr(u2), C.c_float(th), ptr(out),
                                          C.byref(nf)), "orbgpu_search_by_sim3")
        return nf.value, out[:s1.n]

    def _search_by_projection_mappoints(self, F: FrameView, mappoints, mp_descriptors, th: float = 1.0,
                                        claimed=None):
        s = F.struct()
        dev = s.mem == MEM_DEVICE
        nm = C.c_int(0)
        if dev:
            import torch
            out = torch.empty(max(s.n, 1), dtype=torch.int32, device="cuda")
            mps, mpd, cl = mappoints, mp_descriptors, claimed
        else:
            out = np.zeros(max(s.n, 1), np.int32)
            mps = np.ascontiguousarray(mappoints, MAPPOINT_DTYPE)
            mpd = np.ascontiguousarray(mp_descriptors, np.uint8)
            cl = None if claimed is None else np.ascontiguousarray(claimed, np.uint8)
        # the map point count comes from the descriptor rows (M x 32), so a raw
        # byte view of the records cannot be mistaken for more map points
        n_mp = int(mpd.shape[0])
        if (mps.nbytes if isinstance(mps, np.ndarray) else mps.numel() * mps.element_size()) < n_mp * 32:
            raise ValueError("mappoints buffer holds fewer records than mp_descriptors rows")
        check(lib().orbgpu_search_by_projection(self._h, C.byref(s), ptr(mps), ptr(mpd), n_mp,
                                                C.c_float(th), ptr(cl), ptr(out), MEM_DEVICE if dev else MEM_HOST,
                                                C.byref(nm)),
              "orbgpu_search_by_projection")
        return nm.value, out[:s.n]

    def knn2(self, query, train, algo: int = 0, ratio: float | None = None):
        """Brute-force k=2 over DescriptorDistance (device tensors) -> (idx1, d1, idx2, d2),
        plus the ratio test's accept mask (uint8) when 'ratio' is given.

        algo 0: popcount kernel; 1: tensor cores (+-1 FP8 dot products); -1:
        automatic (tuned crossover).  All give the same (distance, lower index
        first) results."""
        import torch
        nq = int(query.shape[0])
        outs = [torch.empty(max(nq, 1), dtype=torch.int32, device=query.device) for _ in range(4)]
        check(lib().orbgpu_knn2(self._h, ptr(query), nq, ptr(train), int(train.shape[0]), *[ptr(o) for o in outs],
                                int(algo)),
              "orbgpu_knn2")
        res = tuple(o[:nq] for o in outs)
        if ratio is None:
            return res
        accept = torch.empty(max(nq, 1), dtype=torch.uint8, device=query.device)
        check(lib().orbgpu_knn2_accept(ptr(outs[1]), ptr(outs[3]), nq, C.c_float(ratio), ptr(accept),
                                       C.c_void_p(torch.cuda.current_stream().cuda_stream)),
              "orbgpu_knn2_accept")
        return res + (accept[:nq],)

    @staticmethod
    def DescriptorDistance(a, b):
        """ORBmatcher::DescriptorDistance over rows of two device tensors."""
        import torch
        n = int(a.shape[0])
        out = torch.empty(max(n, 1), dtype=torch.int32, device=a.device)
        check(lib().orbgpu_descriptor_distance(ptr(a), ptr(b), n, ptr(out), C.c_void_p(0)), "orbgpu_descriptor_distance")
        torch.cuda.synchronize()
        return out[:n]


def compute_stereo_matches(matcher: ORBmatcher, left_extractor, right_extractor, FL: FrameView, FR: FrameView,
                           bf: float, fx: float):
    """Frame::ComputeStereoMatches (src/Frame.cc:831-1082): (mvuRight, mvDepth).

    The extractors must be the ones that produced FL / FR (their pyramids are
    read in place)."""
    sl, sr = FL.struct(), FR.struct()
    dev = sl.mem == MEM_DEVICE
    if dev:
        import torch
        ur = torch.empty(max(sl.n, 1), dtype=torch.float32, device="cuda")
        dp = torch.empty(max(sl.n, 1), dtype=torch.float32, device="cuda")
    else:
        ur = np.zeros(max(sl.n, 1), np.float32)
        dp = np.zeros(max(sl.n, 1), np.float32)
    check(lib().orbgpu_compute_stereo_matches(matcher.handle, left_extractor.handle, right_extractor.handle,
                                              C.byref(sl), C.byref(sr), C.c_float(bf), C.c_float(fx), ptr(ur), ptr(dp),
                                              MEM_DEVICE if dev else MEM_HOST),
          "orbgpu_compute_stereo_matches")
    return ur[:sl.n], dp[:sl.n]
