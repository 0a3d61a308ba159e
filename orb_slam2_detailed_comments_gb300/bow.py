"""DBoW2's vocabulary on the GPU: ORBVocabulary (include/ORBVocabulary.h) and
Frame::ComputeBoW (src/Frame.cc:704-718) for many frames at once
(orbgpu_vocabulary_* / orbgpu_bow_transform in include/orbgpu.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import OrbGpuError, check, lib, ptr


class Vocabulary:
    """A DBoW2 vocabulary tree resident on the device.

    Vocabulary(path) reads the text format of
    TemplatedVocabulary::loadFromTextFile; Vocabulary.from_arrays builds the
    same tree from arrays (node i + 1 described by entry i, parents first).
    """

    def __init__(self, path: str | None = None, _handle=None):
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = _handle
        else:
            check(lib().orbgpu_vocabulary_load_text(str(path).encode(), C.byref(self._h)),
                  "orbgpu_vocabulary_load_text")

    @classmethod
    def from_arrays(cls, k, L, scoring, weighting, parents, is_leaf, descriptors, weights):
        h = C.c_void_p()
        par = np.ascontiguousarray(parents, np.int32)
        lf = np.ascontiguousarray(is_leaf, np.uint8)
        d = np.ascontiguousarray(descriptors, np.uint8).reshape(-1, 32)
        w = np.ascontiguousarray(weights, np.float64)
        if not (len(par) == len(lf) == len(d) == len(w)):
            raise ValueError("parents, is_leaf, descriptors and weights need one entry per node after the root")
        check(lib().orbgpu_vocabulary_create(int(k), int(L), int(scoring), int(weighting), len(par) + 1, ptr(par),
                                             ptr(lf), ptr(d), ptr(w), C.byref(h)), "orbgpu_vocabulary_create")
        return cls(_handle=h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            try:
                lib().orbgpu_vocabulary_destroy(h)
            except Exception:
                pass

    def size(self) -> int:
        """TemplatedVocabulary::size(): the number of words."""
        nw, nn = C.c_int(0), C.c_int(0)
        check(lib().orbgpu_vocabulary_size(self._h, C.byref(nw), C.byref(nn)), "orbgpu_vocabulary_size")
        return nw.value

    def transform(self, descriptors, offsets, levelsup: int = 4, stream=None):
        """TemplatedVocabulary::transform(features, BowVector, FeatureVector,
        levelsup) for every frame of a batch: descriptors an (n, 32) uint8
        tensor (device or page-locked host), offsets an (nframes + 1,) int32
        tensor.  Returns a dict of device tensors (see orbgpu_bow_transform):
        word, weight, node per feature; bow_counts, bow_words, bow_values,
        fv_counts, fv_nodes, fv_starts, fv_sizes, fv_features with frame f's
        entries from offsets[f] on.  Asynchronous on the current stream."""
        import torch
        n = int(descriptors.shape[0])
        nf = int(offsets.shape[0]) - 1
        dev = torch.device("cuda")
        m = max(n, 1)
        out = {"word": torch.empty(m, dtype=torch.int32, device=dev),
               "weight": torch.empty(m, dtype=torch.float64, device=dev),
               "node": torch.empty(m, dtype=torch.int32, device=dev),
               "bow_counts": torch.empty(max(nf, 1), dtype=torch.int32, device=dev),
               "bow_words": torch.empty(m, dtype=torch.int32, device=dev),
               "bow_values": torch.empty(m, dtype=torch.float64, device=dev),
               "fv_counts": torch.empty(max(nf, 1), dtype=torch.int32, device=dev),
               "fv_nodes": torch.empty(m, dtype=torch.int32, device=dev),
               "fv_starts": torch.empty(m, dtype=torch.int32, device=dev),
               "fv_sizes": torch.empty(m, dtype=torch.int32, device=dev),
               "fv_features": torch.empty(m, dtype=torch.int32, device=dev)}
        st = torch.cuda.current_stream().cuda_stream if stream is None else int(stream)
        keys = ("word", "weight", "node", "bow_counts", "bow_words", "bow_values", "fv_counts", "fv_nodes",
                "fv_starts", "fv_sizes", "fv_features")
        check(lib().orbgpu_bow_transform(self._h, ptr(descriptors), ptr(offsets), nf, int(levelsup),
                                         *[ptr(out[k]) for k in keys], C.c_void_p(st)), "orbgpu_bow_transform")
        return out

    def ComputeBoW(self, descriptors, levelsup: int = 4):
        """Frame::ComputeBoW for one frame: (BowVector as {word: value},
        FeatureVector as {node: [feature indices]}) on the host."""
        import torch
        n = int(descriptors.shape[0])
        offs = torch.tensor([0, n], dtype=torch.int32, device="cuda")
        r = self.transform(descriptors, offs, levelsup)
        nb, nv = int(r["bow_counts"][0].item()), int(r["fv_counts"][0].item())
        if nb < 0:
            raise OrbGpuError(1, "ComputeBoW", "more than 8192 features in one frame")
        words = r["bow_words"][:nb].cpu().numpy()
        values = r["bow_values"][:nb].cpu().numpy()
        nodes = r["fv_nodes"][:nv].cpu().numpy()
        starts = r["fv_starts"][:nv].cpu().numpy()
        sizes = r["fv_sizes"][:nv].cpu().numpy()
        feats = r["fv_features"][:n].cpu().numpy()
        return ({int(w): float(v) for w, v in zip(words, values)},
                {int(nd): feats[s:s + z].tolist() for nd, s, z in zip(nodes, starts, sizes)})


def search_by_bow(keypoints, descriptors, offsets, bow, kf_mappoints, pairs, nnratio: float = 0.75,
                  check_orientation: bool = True, stream=None, keyframes: bool = False):
    """ORBmatcher::SearchByBoW(KeyFrame*, Frame&, vpMapPointMatches)
    (src/ORBmatcher.cc:247-380) for many (keyframe, frame) pairs in one launch.

    keypoints (n, 7) float32, descriptors (n, 32) uint8 and offsets (S + 1,)
    int32 tensors hold a set of S keyframes and frames back to back; bow is
    Vocabulary.transform's result on that set; kf_mappoints (n,) uint8, 1
    where a keyframe feature has a map point that is not bad; pairs (P, 2)
    host ints (keyframe entry, frame entry).  Returns (nmatches (P,), list of
    P match tensors: per frame feature the keyframe feature whose map point it
    receives, or -1).  With keyframes=True it is SearchByBoW(KeyFrame* pKF1,
    KeyFrame* pKF2, vpMatches12) (src/ORBmatcher.cc:729-880): pairs hold
    (pKF1, pKF2), kf_mappoints is read for both, and the matches are per pKF1
    feature (the pKF2 feature or -1)."""
    import torch
    pr = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    offs = offsets.cpu().numpy() if offsets.is_cuda else np.asarray(offsets)
    side = 0 if keyframes else 1
    sizes = offs[pr[:, side] + 1] - offs[pr[:, side]]
    out_off = np.zeros(len(pr) + 1, np.int32)
    out_off[1:] = np.cumsum(sizes)
    dev = torch.device("cuda")
    P = torch.from_numpy(pr.reshape(-1).copy()).to(dev)
    OO = torch.from_numpy(out_off[:-1].copy()).to(dev)
    match = torch.empty(max(int(out_off[-1]), 1), dtype=torch.int32, device=dev)
    nm = torch.empty(max(len(pr), 1), dtype=torch.int32, device=dev)
    st = torch.cuda.current_stream().cuda_stream if stream is None else int(stream)
    fn = lib().orbgpu_search_by_bow_keyframes if keyframes else lib().orbgpu_search_by_bow
    check(fn(ptr(keypoints), ptr(descriptors), ptr(offsets), ptr(bow["fv_counts"]),
                                     ptr(bow["fv_nodes"]), ptr(bow["fv_starts"]), ptr(bow["fv_sizes"]),
                                     ptr(bow["fv_features"]), ptr(kf_mappoints), ptr(P), len(pr), C.c_float(nnratio),
                                     int(bool(check_orientation)), ptr(OO), ptr(match), ptr(nm), C.c_void_p(st)),
          "orbgpu_search_by_bow")
    return nm[:len(pr)], [match[out_off[i]:out_off[i + 1]] for i in range(len(pr))]


def search_for_triangulation(keypoints, descriptors, offsets, bow, has_mappoint, uright, pairs, geometry,
                             scale_factors, level_sigma2, only_stereo: bool = False, check_orientation: bool = True,
                             stream=None):
    """ORBmatcher::SearchForTriangulation(pKF1, pKF2, F12, vMatchedPairs,
    bOnlyStereo) (src/ORBmatcher.cc:884-1040) for many keyframe pairs.

    The set as for search_by_bow; has_mappoint (n,) uint8 (GetMapPoint(i) not
    NULL), uright (n,) float32 tensors; pairs (P, 2) host ints (pKF1, pKF2);
    geometry: per pair (Cw1, T2 (3 x 4), K2 (fx, fy, cx, cy), F12 (3 x 3))
    on the host; scale_factors / level_sigma2: pKF2's tables.  Returns
    (nmatches (P,), list of P tensors: per pKF1 feature the paired pKF2
    feature or -1)."""
    import torch
    pr = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
    params = np.zeros((len(pr), 11), np.float32)
    for i, (Cw1, T2, K2, F12) in enumerate(geometry):
        ex, ey = C.c_float(0), C.c_float(0)
        c = np.ascontiguousarray(Cw1, np.float32)
        t = np.ascontiguousarray(np.asarray(T2, np.float32).reshape(-1)[:12])
        k = np.ascontiguousarray(K2, np.float32)
        check(lib().orbgpu_triangulation_epipole(ptr(c), ptr(t), ptr(k), C.byref(ex), C.byref(ey)),
              "orbgpu_triangulation_epipole")
        params[i, :9] = np.asarray(F12, np.float32).reshape(-1)[:9]
        params[i, 9], params[i, 10] = ex.value, ey.value
    offs = offsets.cpu().numpy() if offsets.is_cuda else np.asarray(offsets)
    sizes = offs[pr[:, 0] + 1] - offs[pr[:, 0]]
    out_off = np.zeros(len(pr) + 1, np.int32)
    out_off[1:] = np.cumsum(sizes)
    dev = torch.device("cuda")
    P = torch.from_numpy(pr.reshape(-1).copy()).to(dev)
    PP = torch.from_numpy(params.reshape(-1).copy()).to(dev)
    OO = torch.from_numpy(out_off[:-1].copy()).to(dev)
    sc = np.ascontiguousarray(scale_factors, np.float32)
    sg = np.ascontiguousarray(level_sigma2, np.float32)
    match = torch.empty(max(int(out_off[-1]), 1), dtype=torch.int32, device=dev)
    nm = torch.empty(max(len(pr), 1), dtype=torch.int32, device=dev)
    st = torch.cuda.current_stream().cuda_stream if stream is None else int(stream)
    check(lib().orbgpu_search_for_triangulation(ptr(keypoints), ptr(descriptors), ptr(offsets), ptr(bow["fv_counts"]),
                                                ptr(bow["fv_nodes"]), ptr(bow["fv_starts"]), ptr(bow["fv_sizes"]),
                                                ptr(bow["fv_features"]), ptr(has_mappoint), ptr(uright), ptr(P),
                                                len(pr), ptr(PP), ptr(sc), ptr(sg), len(sc), int(bool(only_stereo)),
                                                int(bool(check_orientation)), ptr(OO), ptr(match), ptr(nm),
                                                C.c_void_p(st)), "orbgpu_search_for_triangulation")
    return nm[:len(pr)], [match[out_off[i]:out_off[i + 1]] for i in range(len(pr))]
