// orbgpu_stereo.cuh -- Frame::ComputeStereoMatches (src/Frame.cc:831-1082) as
// device functions, shared by the per-frame entry (orbgpu_match.cu) and the
// batched one over a batch's resident pyramids (orbgpu_batch.cu).
//
//   row index    every right keypoint is listed under the image rows of its
//                band [y - 2 scale, y + 2 scale] (src/Frame.cc:875-881)
//   match        one warp per left keypoint: the row band's best descriptor
//                distance (octave within one level, uR in [uL - maxD, uL]),
//                accepted below (TH_HIGH + TH_LOW) / 2; then the SAD of the
//                centre-subtracted 11 x 11 patch at 11 offsets (22 lanes: each
//                offset's rows in two halves), the first minimum, the
//                parabola, disparity and depth (src/Frame.cc:884-1064)
//   median cut   one block per frame: SADs of the accepted matches sorted,
//                those at or above 1.5 * 1.4 * median discarded
//                (src/Frame.cc:1069-1081)
#pragma once

#include "orbgpu_common.cuh"
#include "orbgpu_ext.h"

namespace orbgpu {

struct StereoLevels {
    const uint8_t* left[16];
    const uint8_t* right[16];
    int w[16], h[16], pitch[16];
    float scale[16], inv_scale[16];
    int nlevels;
};

// Rows [lo, hi] (clipped to [0, nRows)) whose band holds right keypoint kp;
// false for an octave outside the pyramid.
__device__ __forceinline__ bool stereo_rows_of(const orbgpu_keypoint& kp, const StereoLevels& lv, int nRows, int& lo,
                                               int& hi) {
    if (kp.octave < 0 || kp.octave >= lv.nlevels) return false;
    const float r = __fmul_rn(2.0f, lv.scale[kp.octave]);
    hi = min((int)ceilf(__fadd_rn(kp.y, r)), nRows - 1);
    lo = max((int)floorf(__fsub_rn(kp.y, r)), 0);
    return true;
}

// The match of left keypoint iL, by the calling warp.  Writes uright[iL],
// depth[iL] (-1 when unmatched) and sad_out[iL] (the accepted SAD, -1 none).
__device__ __forceinline__ void stereo_match_warp(int iL, const orbgpu_keypoint* kpsL, const uint8_t* descL,
                                                  const orbgpu_keypoint* kpsR, const uint8_t* descR,
                                                  const StereoLevels& lv, int nRows, const int* row_start,
                                                  const int* row_keys, float bf, float fx, float* uright,
                                                  float* depth, int* sad_out, int* status) {
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        uright[iL] = -1.0f;
        depth[iL] = -1.0f;
        sad_out[iL] = -1;
    }
    const orbgpu_keypoint kpL = kpsL[iL];
    const int levelL = kpL.octave;
    if (levelL < 0 || levelL >= lv.nlevels) return;
    const float vL = kpL.y, uL = kpL.x;
    const int row = (int)vL;
    if (row < 0 || row >= nRows) return;
    const int rs = row_start[row], re = row_start[row + 1];
    if (rs == re) return;
    const float mb = __fdiv_rn(bf, fx);
    const float minZ = mb, minD = 0.f, maxD = __fdiv_rn(bf, minZ);
    const float minU = __fsub_rn(uL, maxD), maxU = __fsub_rn(uL, minD);
    if (maxU < 0) return;
    // best over the row band: lexicographic (distance, right index), distance < TH_HIGH
    uint64_t best = ~0ull;
    const uint8_t* dL = descL + (size_t)iL * 32;
    for (int b = rs; b < re; b += 32) {
        const int j = b + lane;
        if (j < re) {
            const int iR = row_keys[j];
            const orbgpu_keypoint kpR = kpsR[iR];
            if (kpR.octave >= levelL - 1 && kpR.octave <= levelL + 1 && kpR.x >= minU && kpR.x <= maxU) {
                const int dist = hamming256_ptr(dL, descR + (size_t)iR * 32);
                if (dist < ORBGPU_TH_HIGH) {
                    const uint64_t key = ((uint64_t)dist << 32) | (uint32_t)iR;
                    best = key < best ? key : best;
                }
            }
        }
    }
    best = warp_min_u64(best);
    if (best == ~0ull) return;
    const int bestDist = (int)(best >> 32);
    const int thOrbDist = (ORBGPU_TH_HIGH + ORBGPU_TH_LOW) / 2;
    if (bestDist >= thOrbDist) return;
    const int bestIdxR = (int)(best & 0xFFFFFFFFu);
    // SAD refinement on the unblurred level (src/Frame.cc:951-1020)
    const float uR0 = kpsR[bestIdxR].x;
    const float sf = lv.inv_scale[levelL];
    const float scaleduL = roundf(__fmul_rn(kpL.x, sf));
    const float scaledvL = roundf(__fmul_rn(kpL.y, sf));
    const float scaleduR0 = roundf(__fmul_rn(uR0, sf));
    const int W = 5, L = 5;
    const int lw = lv.w[levelL], lh = lv.h[levelL], lp = lv.pitch[levelL];
    const float iniu = __fsub_rn(__fsub_rn(scaleduR0, (float)L), (float)W);
    const float endu = __fadd_rn(__fadd_rn(__fadd_rn(scaleduR0, (float)L), (float)W), 1.0f);
    if (iniu < 0 || endu >= (float)lw) return;
    const int ly0 = (int)(scaledvL - W), lx0 = (int)(scaleduL - W);
    if (ly0 < 0 || ly0 + 2 * W + 1 > lh || lx0 < 0 || lx0 + 2 * W + 1 > lw) {
        if (lane == 0) atomicOr(status, 1);
        return;
    }
    const uint8_t* left = lv.left[levelL];
    const uint8_t* right = lv.right[levelL];
    // offset t = incR + L on lanes t and t + 11: rows 0-5 and rows 6-10
    int part = 0;
    if (lane < 2 * (2 * L + 1)) {
        const int t = lane < 2 * L + 1 ? lane : lane - (2 * L + 1);
        const int yb = lane < 2 * L + 1 ? 0 : W + 1, ye = lane < 2 * L + 1 ? W + 1 : 2 * W + 1;
        const int incR = t - L;
        const int rx0 = (int)(scaleduR0 + incR - W);
        const int cl = left[(size_t)(ly0 + W) * lp + lx0 + W];
        const int cr = right[(size_t)(ly0 + W) * lp + rx0 + W];
        for (int yy = yb; yy < ye; yy++) {
            const uint8_t* lr = left + (size_t)(ly0 + yy) * lp + lx0;
            const uint8_t* rr = right + (size_t)(ly0 + yy) * lp + rx0;
#pragma unroll
            for (int xx = 0; xx < 2 * W + 1; xx++) part += abs((lr[xx] - cl) - (rr[xx] - cr));
        }
    }
    const int other = __shfl_down_sync(0xffffffffu, part, 2 * L + 1);
    const int sad = lane < 2 * L + 1 ? part + other : 0x7fffffff;
    // first minimum over incR = -L..L (ascending lanes)
    int bestSad = 0x7fffffff, bestinc = 0;
    float dists[2 * 5 + 1];
#pragma unroll
    for (int t = 0; t < 2 * L + 1; t++) {
        const int v = __shfl_sync(0xffffffffu, sad, t);
        dists[t] = (float)v;
        if ((float)v < (float)bestSad) {
            bestSad = v;
            bestinc = t - L;
        }
    }
    if (lane != 0) return;
    if (bestinc == -L || bestinc == L) return;
    const float d1 = dists[L + bestinc - 1], d2 = dists[L + bestinc], d3 = dists[L + bestinc + 1];
    const float deltaR = __fdiv_rn(__fsub_rn(d1, d3), __fmul_rn(2.0f, __fsub_rn(__fadd_rn(d1, d3), __fmul_rn(2.0f, d2))));
    if (deltaR < -1 || deltaR > 1) return;
    float bestuR = __fmul_rn(lv.scale[levelL], __fadd_rn(__fadd_rn(scaleduR0, (float)bestinc), deltaR));
    float disparity = __fsub_rn(uL, bestuR);
    if (disparity >= minD && disparity < maxD) {
        if (disparity <= 0) {
            disparity = 0.01f;
            bestuR = (float)((double)uL - 0.01);
        }
        depth[iL] = __fdiv_rn(bf, disparity);
        uright[iL] = bestuR;
        sad_out[iL] = bestSad;
    }
}

// The median cut of one frame's nL left keypoints by the calling block
// (sort_buf: cap ints, cap a power of two at least nL).  *n_valid (nullable)
// receives the number of accepted matches before the cut.
__device__ __forceinline__ void stereo_median_block(int nL, const int* sad, float* uright, float* depth, int* sort_buf,
                                                    int cap, int* n_valid) {
    __shared__ int s_scan[32];
    int cnt = 0;
    for (int b0 = 0; b0 < nL; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        const int v = (i < nL && sad[i] >= 0) ? 1 : 0;
        int tot;
        const int ex = block_exclusive_scan(v, s_scan, &tot);
        if (v && cnt + ex < cap) sort_buf[cnt + ex] = sad[i];
        cnt += tot;
    }
    __syncthreads();
    if (threadIdx.x == 0 && n_valid) *n_valid = cnt;
    if (cnt == 0 || cnt > cap) return;
    int np2 = 1;
    while (np2 < cnt) np2 <<= 1;
    for (int i = cnt + threadIdx.x; i < np2; i += blockDim.x) sort_buf[i] = 0x7fffffff;
    __syncthreads();
    for (int size = 2; size <= np2; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < np2 / 2; t += blockDim.x) {
                const int lo = 2 * t - (t & (stride - 1));
                const int hi = lo + stride;
                const bool asc = ((lo & size) == 0);
                const int a = sort_buf[lo], b = sort_buf[hi];
                if ((a > b) == asc) {
                    sort_buf[lo] = b;
                    sort_buf[hi] = a;
                }
            }
            __syncthreads();
        }
    const float median = (float)sort_buf[cnt / 2];
    const float thDist = __fmul_rn(1.5f * 1.4f, median);
    for (int i = threadIdx.x; i < nL; i += blockDim.x)
        if (sad[i] >= 0 && !((float)sad[i] < thDist)) {
            uright[i] = -1.0f;
            depth[i] = -1.0f;
        }
}

}  // namespace orbgpu
