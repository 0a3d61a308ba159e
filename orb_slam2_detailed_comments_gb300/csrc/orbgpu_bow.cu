// orbgpu_bow.cu -- DBoW2's vocabulary transform (Frame::ComputeBoW,
// src/Frame.cc:704-718: ORBVocabulary::transform(descriptors, mBowVec,
// mFeatVec, 4)) for the features of many frames.
//
// The vocabulary tree lives in HBM with every node's children contiguous
// (grouped by parent in node-id order, the order loadFromTextFile appends
// them), so one descent level reads the k child descriptors of one node as
// consecutive 32-byte rows.  k_bow_descend: one thread per feature walks the
// tree (TemplatedVocabulary.h:1240-1290: at every level the first child with
// the least Hamming distance, strict <; the node of level L - levelsup kept
// for the feature vector; stop at a node without children) and writes the
// word, its weight and that node.  k_bow_assemble: two blocks per frame sort
// the kept features (weight > 0) by word and by node in shared memory and
// writes BowVector (BowVector::addWeight / addIfNotExist, then normalize,
// BowVector.cpp:40-95) and FeatureVector (FeatureVector::addFeature,
// FeatureVector.cpp:37-53).  The doubles are the reference's: a word seen c
// times sums its weight c times in sequence (the reference adds them in
// feature order, and they are equal), and the norm is one sequential sum in
// ascending word order, as std::map iterates.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "orbgpu_host.h"

struct orbgpu_vocabulary {
    int k, L, scoring, weighting, nnodes, nwords;
    uint4* child_desc;   // one 32-byte row per non-root node, grouped by parent
    int* child_start;    // nnodes + 1: children of node p at positions [child_start[p], child_start[p + 1])
    int* pos_node;       // node id at each position
    int* node_word;      // word id of every node (0 where none, as DBoW2's Node default)
    double* node_weight;
};

namespace orbgpu {

#define BOW_THREADS 256
#define BOW_ASM_THREADS 1024
#define BOW_MAX_FEATURES 8192  // per frame (the assembly sorts a frame in shared memory)

__global__ void __launch_bounds__(BOW_THREADS) k_bow_descend(const uint4* __restrict__ desc, const int* __restrict__ offsets,
                                                             int nframes, const uint4* __restrict__ child_desc,
                                                             const int* __restrict__ child_start,
                                                             const int* __restrict__ pos_node,
                                                             const int* __restrict__ node_word,
                                                             const double* __restrict__ node_weight, int nid_level,
                                                             int* __restrict__ word_out, double* __restrict__ weight_out,
                                                             int* __restrict__ node_out) {
    const int first = __ldg(offsets), last = __ldg(offsets + nframes);
    if (first < 0) return;
    for (int i = first + blockIdx.x * BOW_THREADS + threadIdx.x; i < last; i += gridDim.x * BOW_THREADS) {
        const uint4 f0 = __ldg(desc + 2 * (size_t)i), f1 = __ldg(desc + 2 * (size_t)i + 1);
        int node = 0, level = 0, nid = 0;
        int s = __ldg(child_start), e = __ldg(child_start + 1);
        while (s < e) {
            ++level;
            int best = s;
            int best_d = hamming256(f0, f1, __ldg(child_desc + 2 * (size_t)s), __ldg(child_desc + 2 * (size_t)s + 1));
            for (int p = s + 1; p < e; p++) {
                const int d = hamming256(f0, f1, __ldg(child_desc + 2 * (size_t)p), __ldg(child_desc + 2 * (size_t)p + 1));
                if (d < best_d) {
                    best_d = d;
                    best = p;
                }
            }
            node = __ldg(pos_node + best);
            if (level == nid_level) nid = node;
            s = __ldg(child_start + node);
            e = __ldg(child_start + node + 1);
        }
        word_out[i] = __ldg(node_word + node);
        weight_out[i] = __ldg(node_weight + node);
        node_out[i] = nid;
    }
}

// Ascending bitonic sort of n2 (a power of two) 64-bit keys in shared memory.
__device__ void bow_block_sort(unsigned long long* keys, int n2) {
    for (int k = 2; k <= n2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const unsigned long long a = keys[i], b = keys[l];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        keys[i] = b;
                        keys[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Two blocks per frame (block 2f builds frame f's BowVector, block 2f + 1 its
// FeatureVector).  Shared memory: BOW_MAX_FEATURES 64-bit keys per block.
__global__ void __launch_bounds__(BOW_ASM_THREADS) k_bow_assemble(
    const int* __restrict__ offsets, const int* __restrict__ word, const double* __restrict__ weight,
    const int* __restrict__ node, int weighting, int scoring, int* __restrict__ bow_counts,
    int* __restrict__ bow_words, double* __restrict__ bow_values, int* __restrict__ fv_counts,
    int* __restrict__ fv_nodes, int* __restrict__ fv_starts, int* __restrict__ fv_sizes,
    int* __restrict__ fv_features) {
    extern __shared__ unsigned long long keys[];
    __shared__ int s_nkept, s_nruns;
    __shared__ double s_norm;
    // two blocks per frame: pass 0 the BowVector (keys word << 32 | feature),
    // pass 1 the FeatureVector (node << 32 | feature)
    const int f = blockIdx.x >> 1, pass = blockIdx.x & 1;
    const int o0 = offsets[f], o1 = offsets[f + 1];
    const int n = o1 - o0;
    if (o0 < 0 || n < 0 || n > BOW_MAX_FEATURES) {
        if (threadIdx.x == 0) (pass == 0 ? bow_counts : fv_counts)[f] = -1;
        return;
    }
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    const unsigned long long pad = ~0ull;
    {
        for (int i = threadIdx.x; i < n2; i += blockDim.x) {
            unsigned long long key = pad;
            if (i < n && weight[o0 + i] > 0.0) {
                const unsigned hi = pass == 0 ? (unsigned)word[o0 + i] : (unsigned)node[o0 + i];
                key = ((unsigned long long)hi << 32) | (unsigned)i;
            }
            keys[i] = key;
        }
        if (threadIdx.x == 0) {
            s_nkept = 0;
            s_nruns = 0;
        }
        __syncthreads();
        bow_block_sort(keys, n2);
        // kept features sort first; runs of equal high words are the entries
        int kept = 0;
        for (int i = threadIdx.x; i < n2; i += blockDim.x) kept += keys[i] != pad ? 1 : 0;
        kept = __reduce_add_sync(0xffffffffu, kept);
        if ((threadIdx.x & 31) == 0 && kept) atomicAdd(&s_nkept, kept);
        __syncthreads();
        const int nk = s_nkept;
        // run starts in ascending order: a block-wide exclusive scan of the flags
        __shared__ int s_warp[BOW_ASM_THREADS / 32];
        for (int base = 0; base < nk; base += blockDim.x) {
            const int i = base + threadIdx.x;
            const bool start = i < nk && (i == 0 || (keys[i] >> 32) != (keys[i - 1] >> 32));
            const unsigned bal = __ballot_sync(0xffffffffu, start);
            const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
            if (lane == 0) s_warp[w] = __popc(bal);
            __syncthreads();
            if (threadIdx.x == 0) {
                int acc = s_nruns;
                for (int q = 0; q < (int)(blockDim.x >> 5); q++) {
                    const int c = s_warp[q];
                    s_warp[q] = acc;
                    acc += c;
                }
                s_nruns = acc;
            }
            __syncthreads();
            if (start) {
                const int r = s_warp[w] + __popc(bal & ((1u << lane) - 1u));
                int end = i + 1;
                while (end < nk && (keys[end] >> 32) == (keys[i] >> 32)) end++;
                const unsigned hi = (unsigned)(keys[i] >> 32);
                if (pass == 0) {
                    const double w0 = weight[o0 + (int)(keys[i] & 0xffffffffu)];
                    double v = w0;
                    if (weighting == 0 || weighting == 1)  // TF_IDF, TF: addWeight per occurrence
                        for (int q = i + 1; q < end; q++) v = __dadd_rn(v, w0);
                    bow_words[o0 + r] = (int)hi;
                    bow_values[o0 + r] = v;
                } else {
                    fv_nodes[o0 + r] = (int)hi;
                    fv_starts[o0 + r] = o0 + i;
                    fv_sizes[o0 + r] = end - i;
                }
            }
            __syncthreads();
        }
        const int nruns = s_nruns;
        if (pass == 1) {
            // the features of every node, in feature order (the sort's low words)
            for (int i = threadIdx.x; i < nk; i += blockDim.x) fv_features[o0 + i] = (int)(keys[i] & 0xffffffffull);
            if (threadIdx.x == 0) fv_counts[f] = nruns;
            return;
        }
        // normalisation (ScoringObject.h:84-89: L1 for L1 / chi-square / KL /
        // Bhattacharyya, L2 for L2, none for the dot product, where TF divides
        // by the number of words instead)
        if (threadIdx.x == 0) {
            double norm = 0.0;
            if (scoring == 5) {
                norm = (weighting == 0 || weighting == 1) && nruns > 0 ? (double)nruns : 0.0;
            } else if (scoring == 1) {
                for (int r = 0; r < nruns; r++) norm = __dadd_rn(norm, __dmul_rn(bow_values[o0 + r], bow_values[o0 + r]));
                norm = __dsqrt_rn(norm);
            } else {
                for (int r = 0; r < nruns; r++) norm = __dadd_rn(norm, fabs(bow_values[o0 + r]));
            }
            s_norm = norm;
            bow_counts[f] = nruns;
        }
        __syncthreads();
        const double norm = s_norm;
        if (norm > 0.0)
            for (int r = threadIdx.x; r < nruns; r += blockDim.x) bow_values[o0 + r] = __ddiv_rn(bow_values[o0 + r], norm);
        __syncthreads();
    }
}

// ORBmatcher::SearchByBoW(KeyFrame* pKF, Frame& F, vpMapPointMatches),
// src/ORBmatcher.cc:247-380, one block per (keyframe, frame) pair.  A frame
// feature belongs to one FeatureVector node and so does a keyframe feature:
// the nodes both vectors hold are independent, and one warp takes one node
// (found by binary search in the keyframe's sorted node list).  Inside a node
// the keyframe features run in list order, as in the reference: each takes,
// among the node's frame features not matched yet (a shared bitmap), the
// first at the least distance, with the second-best over the rest; kept when
// best <= TH_LOW and best < nnratio * second.  Then the rotation histogram,
// ComputeThreeMaxima (src/ORBmatcher.cc:2035-2077) and the resets.  With
// 'keyframes' it is SearchByBoW(KeyFrame* pKF1, KeyFrame* pKF2, vpMatches12)
// (src/ORBmatcher.cc:729-880): candidates need a map point that is not bad,
// TH_LOW is exclusive, and the result is per pKF1 feature.
#define SBB_THREADS 1024
#define SBB_TH_LOW 50

// SearchForTriangulation's per-call constants: pKF2's scale tables (read at
// the candidate's octave) and bOnlyStereo.
struct TriangulationDev {
    float scale[16];
    float sigma2[16];
    int only_stereo;
};

__global__ void __launch_bounds__(SBB_THREADS) k_search_by_bow(
    const orbgpu_keypoint* __restrict__ kps, const uint4* __restrict__ desc, const int* __restrict__ offsets,
    const int* __restrict__ fv_counts, const int* __restrict__ fv_nodes, const int* __restrict__ fv_starts,
    const int* __restrict__ fv_sizes, const int* __restrict__ fv_features, const uint8_t* __restrict__ kf_mp,
    const int* __restrict__ pairs, float nnratio, int check_ori, int keyframes, const float* __restrict__ pair_params,
    const float* __restrict__ uright, TriangulationDev tri, const int* __restrict__ out_offsets,
    int* __restrict__ match_out, int* __restrict__ nmatches) {
    __shared__ unsigned s_taken[BOW_MAX_FEATURES / 32];
    __shared__ unsigned char s_bin[BOW_MAX_FEATURES];
    __shared__ int hist[ORBGPU_HISTO_LENGTH];
    __shared__ int s_ind[3], s_nm;
    const int p = blockIdx.x;
    const int kf = pairs[2 * p], fr = pairs[2 * p + 1];
    const int ok0 = offsets[kf], of0 = offsets[fr];
    const int kn = offsets[kf + 1] - ok0, frn = offsets[fr + 1] - of0;
    // the output (and bins) are per frame feature, or per first-keyframe
    // feature for two keyframes (vpMatches12)
    const int fn = keyframes ? kn : frn;
    const int ckf = fv_counts[kf], cf = fv_counts[fr];
    int* out = match_out + out_offsets[p];
    if (kn < 0 || kn > BOW_MAX_FEATURES || frn < 0 || frn > BOW_MAX_FEATURES || ckf < 0 || cf < 0) {
        if (threadIdx.x == 0) nmatches[p] = -1;
        return;
    }
    for (int i = threadIdx.x; i < fn; i += blockDim.x) out[i] = -1;
    for (int i = threadIdx.x; i < BOW_MAX_FEATURES / 32; i += blockDim.x) s_taken[i] = 0;
    if (threadIdx.x < ORBGPU_HISTO_LENGTH) hist[threadIdx.x] = 0;
    if (threadIdx.x == 0) s_nm = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    // mode 2: SearchForTriangulation -- F12 (row-major) and the epipole in pKF2
    const bool triang = keyframes == 2;
    float F[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, ex = 0.f, ey = 0.f;
    if (triang) {
#pragma unroll
        for (int q = 0; q < 9; q++) F[q] = pair_params[11 * p + q];
        ex = pair_params[11 * p + 9];
        ey = pair_params[11 * p + 10];
    }
    const float factor = __fdiv_rn((float)ORBGPU_HISTO_LENGTH, 360.0f);
    const unsigned INF = 0x7fffffffu;
    for (int j = warp; j < cf; j += nwarps) {
        const int node = fv_nodes[of0 + j];
        int lo = 0, hi = ckf - 1, jk = -1;
        while (lo <= hi) {
            const int mid = (lo + hi) >> 1;
            const int v = fv_nodes[ok0 + mid];
            if (v == node) {
                jk = mid;
                break;
            }
            if (v < node) lo = mid + 1;
            else hi = mid - 1;
        }
        if (jk < 0) continue;
        const int* flist = fv_features + fv_starts[of0 + j];
        const int fcount = fv_sizes[of0 + j];
        const int* klist = fv_features + fv_starts[ok0 + jk];
        const int kcount = fv_sizes[ok0 + jk];
        for (int t = 0; t < kcount; t++) {
            const int ikf = klist[t];
            bool st1 = false;
            float x1 = 0.f, y1 = 0.f, la = 0.f, lb = 0.f, lc = 0.f;
            if (triang) {
                // features without a map point (bad or not), stereo ones only with bOnlyStereo
                if (kf_mp[ok0 + ikf] != 0) continue;
                st1 = uright[ok0 + ikf] >= 0.0f;
                if (tri.only_stereo && !st1) continue;
                x1 = kps[ok0 + ikf].x;
                y1 = kps[ok0 + ikf].y;
                // CheckDistEpipolarLine (src/ORBmatcher.cc:205-232): the line of kp1 in pKF2
                la = __fadd_rn(__fadd_rn(__fmul_rn(x1, F[0]), __fmul_rn(y1, F[3])), F[6]);
                lb = __fadd_rn(__fadd_rn(__fmul_rn(x1, F[1]), __fmul_rn(y1, F[4])), F[7]);
                lc = __fadd_rn(__fadd_rn(__fmul_rn(x1, F[2]), __fmul_rn(y1, F[5])), F[8]);
            } else if (kf_mp[ok0 + ikf] != 1) {
                continue;
            }
            const uint4 a0 = desc[2 * (size_t)(ok0 + ikf)], a1 = desc[2 * (size_t)(ok0 + ikf) + 1];
            unsigned b1 = INF;
            int b2 = 256;
            for (int c = 0; c < fcount; c += 32) {
                unsigned key = INF;
                int d = 256;
                if (c + lane < fcount) {
                    const int jf = flist[c + lane];
                    const bool free2 = !((s_taken[jf >> 5] >> (jf & 31)) & 1u);
                    if (triang) {
                        const bool st2 = uright[of0 + jf] >= 0.0f;
                        if (free2 && kf_mp[of0 + jf] == 0 && (!tri.only_stereo || st2)) {
                            const int dd = hamming256(a0, a1, desc[2 * (size_t)(of0 + jf)],
                                                      desc[2 * (size_t)(of0 + jf) + 1]);
                            const orbgpu_keypoint k2 = kps[of0 + jf];
                            bool ok = dd <= SBB_TH_LOW && k2.octave >= 0 && k2.octave < 16;
                            if (ok && !st1 && !st2) {
                                const float dx = __fsub_rn(ex, k2.x), dy = __fsub_rn(ey, k2.y);
                                if (__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) <
                                    __fmul_rn(100.0f, tri.scale[k2.octave]))
                                    ok = false;
                            }
                            if (ok) {
                                const float num = __fadd_rn(__fadd_rn(__fmul_rn(la, k2.x), __fmul_rn(lb, k2.y)), lc);
                                const float den = __fadd_rn(__fmul_rn(la, la), __fmul_rn(lb, lb));
                                ok = den != 0.0f &&
                                     (double)__fdiv_rn(__fmul_rn(num, num), den) <
                                         __dmul_rn(3.84, (double)tri.sigma2[k2.octave]);
                            }
                            if (ok) {
                                // the last candidate at the least distance wins ("dist > bestDist" skips)
                                d = dd;
                                key = ((unsigned)dd << 13) | (unsigned)(8191 - (c + lane));
                            }
                        }
                    } else if (free2 && (!keyframes || kf_mp[of0 + jf] == 1)) {
                        d = hamming256(a0, a1, desc[2 * (size_t)(of0 + jf)], desc[2 * (size_t)(of0 + jf) + 1]);
                        key = ((unsigned)d << 13) | (unsigned)(c + lane);
                    }
                }
                const unsigned c1 = __reduce_min_sync(0xffffffffu, key);
                const int c2 = (int)__reduce_min_sync(0xffffffffu, (unsigned)(key == c1 ? 256 : d));
                if (c1 < b1) {
                    b2 = min(b1 == INF ? 256 : (int)(b1 >> 13), c2);
                    b1 = c1;
                } else {
                    b2 = min(b2, c1 == INF ? 256 : (int)(c1 >> 13));
                }
            }
            const int best1 = b1 == INF ? 256 : (int)(b1 >> 13);
            // TH_LOW inclusive for (keyframe, frame), exclusive for two
            // keyframes; triangulation: any candidate left (no ratio test)
            const bool take = triang ? b1 != INF
                                     : (keyframes ? best1 < SBB_TH_LOW : best1 <= SBB_TH_LOW) &&
                                           (float)best1 < __fmul_rn(nnratio, (float)b2);
            if (take) {
                if (lane == 0) {
                    const int jf = flist[triang ? 8191u - (b1 & 8191u) : (b1 & 8191u)];
                    atomicOr(&s_taken[jf >> 5], 1u << (jf & 31));
                    const int slot = keyframes ? ikf : jf;
                    out[slot] = keyframes ? jf : ikf;  // modes 1 and 2 report per first-keyframe feature
                    if (check_ori) {
                        float rot = __fsub_rn(kps[ok0 + ikf].angle, kps[of0 + jf].angle);
                        if (rot < 0.0f) rot = __fadd_rn(rot, 360.0f);
                        int bin = (int)roundf(__fmul_rn(rot, factor));
                        if (bin == ORBGPU_HISTO_LENGTH) bin = 0;
                        s_bin[slot] = (unsigned char)bin;
                        atomicAdd(&hist[bin], 1);
                    }
                }
                __syncwarp();
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int ind1 = -1, ind2 = -1, ind3 = -1;
        if (check_ori) {
            int max1 = 0, max2 = 0, max3 = 0;
            for (int b = 0; b < ORBGPU_HISTO_LENGTH; b++) {  // ComputeThreeMaxima, src/ORBmatcher.cc:2035-2077
                const int sz = hist[b];
                if (sz > max1) {
                    max3 = max2; max2 = max1; max1 = sz;
                    ind3 = ind2; ind2 = ind1; ind1 = b;
                } else if (sz > max2) {
                    max3 = max2; max2 = sz;
                    ind3 = ind2; ind2 = b;
                } else if (sz > max3) {
                    max3 = sz;
                    ind3 = b;
                }
            }
            if ((float)max2 < __fmul_rn(0.1f, (float)max1)) {
                ind2 = -1;
                ind3 = -1;
            } else if ((float)max3 < __fmul_rn(0.1f, (float)max1)) {
                ind3 = -1;
            }
        }
        s_ind[0] = ind1;
        s_ind[1] = ind2;
        s_ind[2] = ind3;
    }
    __syncthreads();
    int kept = 0;
    for (int i = threadIdx.x; i < fn; i += blockDim.x) {
        if (out[i] < 0) continue;
        if (check_ori) {
            const int b = s_bin[i];
            if (b != s_ind[0] && b != s_ind[1] && b != s_ind[2]) {
                out[i] = -1;
                continue;
            }
        }
        kept++;
    }
    kept = __reduce_add_sync(0xffffffffu, kept);
    if (lane == 0 && kept) atomicAdd(&s_nm, kept);
    __syncthreads();
    if (threadIdx.x == 0) nmatches[p] = s_nm;
}

}  // namespace orbgpu

using namespace orbgpu;

static int search_by_bow(const orbgpu_keypoint* kps, const uint8_t* desc, const int* offsets, const int* fv_counts,
                         const int* fv_nodes, const int* fv_starts, const int* fv_sizes, const int* fv_features,
                         const uint8_t* kf_mappoints, const int* pairs, int npairs, float nnratio, int check_ori,
                         int keyframes, const int* out_offsets, int* match_out, int* nmatches, void* stream,
                         const float* pair_params = nullptr, const float* uright = nullptr,
                         const TriangulationDev* tri = nullptr) {
    if (npairs < 0 || (npairs > 0 && (!kps || !desc || !offsets || !fv_counts || !fv_nodes || !fv_starts ||
                                      !fv_sizes || !fv_features || !kf_mappoints || !pairs || !out_offsets ||
                                      !match_out || !nmatches)) ||
        ((uintptr_t)desc & 15)) {
        orbgpu_set_last_error("orbgpu_search_by_bow: bad arguments", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (npairs == 0) return ORBGPU_OK;
    k_search_by_bow<<<npairs, SBB_THREADS, 0, (cudaStream_t)stream>>>(
        kps, reinterpret_cast<const uint4*>(desc), offsets, fv_counts, fv_nodes, fv_starts, fv_sizes, fv_features,
        kf_mappoints, pairs, nnratio, check_ori, keyframes, pair_params, uright, tri ? *tri : TriangulationDev{},
        out_offsets, match_out, nmatches);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    return ORBGPU_OK;
}

extern "C" int orbgpu_search_by_bow(const orbgpu_keypoint* kps, const uint8_t* desc, const int* offsets,
                                    const int* fv_counts, const int* fv_nodes, const int* fv_starts,
                                    const int* fv_sizes, const int* fv_features, const uint8_t* kf_mappoints,
                                    const int* pairs, int npairs, float nnratio, int check_ori,
                                    const int* out_offsets, int* match_out, int* nmatches, void* stream) {
    return search_by_bow(kps, desc, offsets, fv_counts, fv_nodes, fv_starts, fv_sizes, fv_features, kf_mappoints,
                         pairs, npairs, nnratio, check_ori, 0, out_offsets, match_out, nmatches, stream);
}

extern "C" int orbgpu_search_by_bow_keyframes(const orbgpu_keypoint* kps, const uint8_t* desc, const int* offsets,
                                              const int* fv_counts, const int* fv_nodes, const int* fv_starts,
                                              const int* fv_sizes, const int* fv_features,
                                              const uint8_t* kf_mappoints, const int* pairs, int npairs,
                                              float nnratio, int check_ori, const int* out_offsets, int* match_out,
                                              int* nmatches, void* stream) {
    return search_by_bow(kps, desc, offsets, fv_counts, fv_nodes, fv_starts, fv_sizes, fv_features, kf_mappoints,
                         pairs, npairs, nnratio, check_ori, 1, out_offsets, match_out, nmatches, stream);
}

extern "C" int orbgpu_vocabulary_create(int k, int L, int scoring, int weighting, int nnodes, const int* parents,
                                        const uint8_t* is_leaf, const uint8_t* descriptors, const double* weights,
                                        orbgpu_vocabulary** out) {
    if (!out || k < 0 || k > 20 || L < 1 || L > 10 || scoring < 0 || scoring > 5 || weighting < 0 || weighting > 3 ||
        nnodes < 1 || (nnodes > 1 && (!parents || !is_leaf || !descriptors || !weights))) {
        orbgpu_set_last_error("orbgpu_vocabulary_create: bad arguments", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    *out = nullptr;
    const int nc = nnodes - 1;  // nodes after the root; node i + 1 is described by entry i
    std::vector<int> count(nnodes + 1, 0);
    for (int i = 0; i < nc; i++) {
        const int p = parents[i];
        if (p < 0 || p > i) {  // a parent must precede its child (the reference indexes m_nodes[pid])
            orbgpu_set_last_error("orbgpu_vocabulary_create: a node's parent does not precede it", __FILE__, __LINE__);
            return ORBGPU_ERR_BAD_ARG;
        }
        count[p + 1]++;
    }
    std::vector<int> start(nnodes + 1, 0);
    for (int p = 0; p < nnodes; p++) start[p + 1] = start[p] + count[p + 1];
    std::vector<int> fill(start.begin(), start.end() - 1), pos_node(std::max(nc, 1));
    std::vector<uint8_t> cdesc((size_t)std::max(nc, 1) * 32);
    std::vector<int> word(nnodes, 0);
    std::vector<double> w(nnodes, 0.0);
    int nwords = 0;
    for (int i = 0; i < nc; i++) {
        const int node = i + 1, pos = fill[parents[i]]++;
        pos_node[pos] = node;
        std::memcpy(&cdesc[(size_t)pos * 32], descriptors + (size_t)i * 32, 32);
        w[node] = weights[i];
        if (is_leaf[i]) word[node] = nwords++;
    }
    orbgpu_vocabulary* v = new orbgpu_vocabulary();
    v->k = k;
    v->L = L;
    v->scoring = scoring;
    v->weighting = weighting;
    v->nnodes = nnodes;
    v->nwords = nwords;
    v->child_desc = nullptr;
    v->child_start = v->pos_node = v->node_word = nullptr;
    v->node_weight = nullptr;
    cudaError_t e = cudaMalloc(&v->child_desc, cdesc.size());
    if (e == cudaSuccess) e = cudaMalloc(&v->child_start, sizeof(int) * (nnodes + 1));
    if (e == cudaSuccess) e = cudaMalloc(&v->pos_node, sizeof(int) * pos_node.size());
    if (e == cudaSuccess) e = cudaMalloc(&v->node_word, sizeof(int) * nnodes);
    if (e == cudaSuccess) e = cudaMalloc(&v->node_weight, sizeof(double) * nnodes);
    if (e == cudaSuccess) e = cudaMemcpy(v->child_desc, cdesc.data(), cdesc.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(v->child_start, start.data(), sizeof(int) * (nnodes + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(v->pos_node, pos_node.data(), sizeof(int) * pos_node.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(v->node_word, word.data(), sizeof(int) * nnodes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(v->node_weight, w.data(), sizeof(double) * nnodes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        orbgpu_vocabulary_destroy(v);
        orbgpu_set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
        return e == cudaErrorMemoryAllocation ? ORBGPU_ERR_OOM : ORBGPU_ERR_CUDA;
    }
    *out = v;
    return ORBGPU_OK;
}

extern "C" int orbgpu_vocabulary_load_text(const char* path, orbgpu_vocabulary** out) {
    // TemplatedVocabulary::loadFromTextFile (TemplatedVocabulary.h:1368-1460):
    // "k L scoring weighting", then "parent is_leaf d0 .. d31 weight" per node
    std::ifstream f(path ? path : "");
    std::string line;
    if (!out || !f.is_open() || !std::getline(f, line)) {
        orbgpu_set_last_error("orbgpu_vocabulary_load_text: cannot read the file", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    int k = -1, L = -1, n1 = -1, n2 = -1;
    {
        std::stringstream hs(line);
        hs >> k >> L >> n1 >> n2;
    }
    std::vector<int> parents;
    std::vector<uint8_t> leaf, desc;
    std::vector<double> weights;
    while (std::getline(f, line)) {
        std::stringstream ls(line);
        int pid = -1, lf = 0;
        ls >> pid >> lf;
        uint8_t d[32];
        for (int i = 0; i < 32; i++) {
            int b = 0;
            ls >> b;
            d[i] = (uint8_t)b;
        }
        double w = 0;
        ls >> w;
        if (line.empty() || ls.fail()) {
            // an empty or short line: the reference appends a node whose
            // descriptor bytes are left unset
            orbgpu_set_last_error("orbgpu_vocabulary_load_text: malformed node line", __FILE__, __LINE__);
            return ORBGPU_ERR_BAD_ARG;
        }
        parents.push_back(pid);
        leaf.push_back(lf > 0 ? 1 : 0);
        desc.insert(desc.end(), d, d + 32);
        weights.push_back(w);
    }
    return orbgpu_vocabulary_create(k, L, n1, n2, (int)parents.size() + 1, parents.data(), leaf.data(), desc.data(),
                                    weights.data(), out);
}

extern "C" int orbgpu_vocabulary_destroy(orbgpu_vocabulary* v) {
    if (!v) return ORBGPU_OK;
    // transforms run on the caller's streams: all of them are done before the
    // tree is freed
    cudaDeviceSynchronize();
    cudaFree(v->child_desc);
    cudaFree(v->child_start);
    cudaFree(v->pos_node);
    cudaFree(v->node_word);
    cudaFree(v->node_weight);
    delete v;
    return ORBGPU_OK;
}

extern "C" int orbgpu_vocabulary_size(const orbgpu_vocabulary* v, int* nwords, int* nnodes) {
    if (!v) return ORBGPU_ERR_BAD_ARG;
    if (nwords) *nwords = v->nwords;
    if (nnodes) *nnodes = v->nnodes;
    return ORBGPU_OK;
}

extern "C" int orbgpu_bow_transform(const orbgpu_vocabulary* v, const uint8_t* desc, const int* offsets, int nframes,
                                    int levelsup, int* word_ids, double* weights, int* node_ids, int* bow_counts,
                                    int* bow_words, double* bow_values, int* fv_counts, int* fv_nodes, int* fv_starts,
                                    int* fv_sizes, int* fv_features, void* stream) {
    if (!v || nframes < 0 ||
        (nframes > 0 && (!desc || !offsets || !word_ids || !weights || !node_ids || !bow_counts || !bow_words ||
                         !bow_values || !fv_counts || !fv_nodes || !fv_starts || !fv_sizes || !fv_features)) ||
        ((uintptr_t)desc & 15)) {
        orbgpu_set_last_error("orbgpu_bow_transform: bad arguments", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (nframes == 0) return ORBGPU_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (v->nwords == 0) {
        // TemplatedVocabulary::transform returns empty vectors for an empty vocabulary
        ORBGPU_CUDA_TRY(cudaMemsetAsync(bow_counts, 0, sizeof(int) * nframes, st));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(fv_counts, 0, sizeof(int) * nframes, st));
        return ORBGPU_OK;
    }
    ORBGPU_CUDA_TRY(allow_max_dynamic_smem(k_bow_assemble));
    const int blocks = nsm_of_current_device() * 8;
    k_bow_descend<<<blocks, BOW_THREADS, 0, st>>>(reinterpret_cast<const uint4*>(desc), offsets, nframes,
                                                  v->child_desc, v->child_start, v->pos_node, v->node_word,
                                                  v->node_weight, v->L - levelsup, word_ids, weights, node_ids);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    k_bow_assemble<<<2 * nframes, BOW_ASM_THREADS, BOW_MAX_FEATURES * 8, st>>>(
        offsets, word_ids, weights, node_ids, v->weighting, v->scoring, bow_counts, bow_words, bow_values, fv_counts,
        fv_nodes, fv_starts, fv_sizes, fv_features);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    return ORBGPU_OK;
}

extern "C" int orbgpu_triangulation_epipole(const float* Cw1, const float* T2, const float* K2, float* ex,
                                            float* ey) {
    if (!Cw1 || !T2 || !K2 || !ex || !ey) return ORBGPU_ERR_BAD_ARG;
    // C2 = R2w * Cw + t2w (src/ORBmatcher.cc:897-901): the 3 x 3 product
    // accumulated in double and rounded to float, then a float add
    float C2[3];
    for (int r = 0; r < 3; r++) {
        double s = 0.0;
        for (int k = 0; k < 3; k++) s += (double)T2[4 * r + k] * (double)Cw1[k];
        C2[r] = (float)s + T2[4 * r + 3];
    }
    const float invz = 1.0f / C2[2];
    *ex = K2[0] * C2[0] * invz + K2[2];
    *ey = K2[1] * C2[1] * invz + K2[3];
    return ORBGPU_OK;
}

extern "C" int orbgpu_search_for_triangulation(const orbgpu_keypoint* kps, const uint8_t* desc, const int* offsets,
                                               const int* fv_counts, const int* fv_nodes, const int* fv_starts,
                                               const int* fv_sizes, const int* fv_features,
                                               const uint8_t* has_mappoint, const float* uright, const int* pairs,
                                               int npairs, const float* pair_params, const float* scale_factors,
                                               const float* level_sigma2, int nlevels, int only_stereo,
                                               int check_ori, const int* out_offsets, int* match_out,
                                               int* nmatches, void* stream) {
    if (!uright || (npairs > 0 && !pair_params) || !scale_factors || !level_sigma2 || nlevels < 1 || nlevels > 16) {
        orbgpu_set_last_error("orbgpu_search_for_triangulation: bad arguments", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    TriangulationDev tri;
    std::memset(&tri, 0, sizeof(tri));
    for (int l = 0; l < nlevels; l++) {
        tri.scale[l] = scale_factors[l];
        tri.sigma2[l] = level_sigma2[l];
    }
    // octaves past nlevels read the reference's vectors out of range: they are rejected here
    for (int l = nlevels; l < 16; l++) tri.scale[l] = tri.sigma2[l] = 0.0f;
    tri.only_stereo = only_stereo ? 1 : 0;
    return search_by_bow(kps, desc, offsets, fv_counts, fv_nodes, fv_starts, fv_sizes, fv_features, has_mappoint,
                         pairs, npairs, 0.0f, check_ori, 2, out_offsets, match_out, nmatches, stream, pair_params,
                         uright, &tri);
}
