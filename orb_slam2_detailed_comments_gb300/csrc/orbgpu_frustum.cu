// orbgpu_frustum.cu -- Frame::isInFrustum (src/Frame.cc:491-578) with
// MapPoint::PredictScale(dist, Frame*) (src/MapPoint.cc:604-619) for the map
// points of many frames in one launch, writing the records the projection
// searches read.
//
// Float semantics follow the compiled reference against the cv stand-in:
// mRcw * P accumulates in double (float products are exact in double) and is
// rounded to float before + mtcw (a float add); cv::norm and Mat::dot
// accumulate in double, the norm is a double sqrt rounded to float and the
// viewing cosine a double division by the float distance rounded to float;
// everything else is float arithmetic in the reference's order, without
// contraction.  The predicted level ceil(logf(ratio) / logf(scale)) is taken
// from per-level thresholds that orbgpu_frustum_frame_init finds with the
// host's logf (the quotient is monotone in ratio), so no device logarithm is
// involved.
#include <cmath>
#include <cstring>

#include "orbgpu_host.h"

namespace orbgpu {

#define FR_THREADS 256
#define FR_BLOCKS_PER_SM 4

__global__ void __launch_bounds__(FR_THREADS) k_is_in_frustum(const orbgpu_frustum_frame* __restrict__ frames,
                                                              int nframes, const int* __restrict__ offsets,
                                                              const orbgpu_mappoint_geometry* __restrict__ mps,
                                                              float cos_limit, orbgpu_mappoint* __restrict__ out,
                                                              int* __restrict__ in_view) {
    const int first = __ldg(offsets), last = __ldg(offsets + nframes);
    if (first < 0) return;
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * FR_THREADS;
    // every lane runs the same number of iterations (warp-wide counting below)
    for (int base = first + blockIdx.x * FR_THREADS + (threadIdx.x & ~31); base < last; base += stride) {
        const int i = base + lane;
        const bool live = i < last;
        int f = 0;
        bool inview = false;
        if (live) {
            // the frame owning map point i: last f with offsets[f] <= i
            int lo = 0, hi = nframes - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (__ldg(offsets + mid) <= i) lo = mid;
                else hi = mid - 1;
            }
            f = lo;
            const orbgpu_frustum_frame& F = frames[f];
            const orbgpu_mappoint_geometry g = mps[i];
            orbgpu_mappoint& o = out[i];
            const double px = g.x, py = g.y, pz = g.z;
            float pc[3];
#pragma unroll
            for (int r = 0; r < 3; r++) {
                double s = __dmul_rn((double)F.Rcw[3 * r], px);
                s = __dadd_rn(s, __dmul_rn((double)F.Rcw[3 * r + 1], py));
                s = __dadd_rn(s, __dmul_rn((double)F.Rcw[3 * r + 2], pz));
                pc[r] = __fadd_rn((float)s, F.tcw[r]);
            }
            do {
                if (pc[2] < 0.0f) break;
                const float invz = __fdiv_rn(1.0f, pc[2]);
                const float u = __fadd_rn(__fmul_rn(__fmul_rn(F.fx, pc[0]), invz), F.cx);
                const float v = __fadd_rn(__fmul_rn(__fmul_rn(F.fy, pc[1]), invz), F.cy);
                if (u < F.min_x || u > F.max_x) break;
                if (v < F.min_y || v > F.max_y) break;
                const float max_d = __fmul_rn(1.2f, g.max_distance);
                const float min_d = __fmul_rn(0.8f, g.min_distance);
                const float po0 = __fsub_rn(g.x, F.Ow[0]), po1 = __fsub_rn(g.y, F.Ow[1]),
                            po2 = __fsub_rn(g.z, F.Ow[2]);
                double ss = __dmul_rn((double)po0, (double)po0);
                ss = __dadd_rn(ss, __dmul_rn((double)po1, (double)po1));
                ss = __dadd_rn(ss, __dmul_rn((double)po2, (double)po2));
                const float dist = (float)__dsqrt_rn(ss);
                if (dist < min_d || dist > max_d) break;
                double dp = __dmul_rn((double)po0, (double)g.nx);
                dp = __dadd_rn(dp, __dmul_rn((double)po1, (double)g.ny));
                dp = __dadd_rn(dp, __dmul_rn((double)po2, (double)g.nz));
                const float view_cos = (float)__ddiv_rn(dp, (double)dist);
                if (view_cos < cos_limit) break;
                const float ratio = __fdiv_rn(g.max_distance, dist);
                int level = 0;
                const int nl = min(F.nlevels, 16);
                for (int n = 0; n < nl - 1; n++) level += ratio > F.level_above[n] ? 1 : 0;
                o.proj_x = u;
                o.proj_y = v;
                o.proj_xr = __fsub_rn(u, __fmul_rn(F.bf, invz));
                o.view_cos = view_cos;
                o.track_scale_level = level;
                inview = true;
            } while (false);
            o.track_in_view = inview ? 1 : 0;
        }
        if (in_view) {
            // one atomic per frame present in the warp
            const unsigned same = __match_any_sync(0xffffffffu, live ? f : -1);
            const unsigned cnt = __ballot_sync(0xffffffffu, inview) & same;
            if (live && lane == __ffs(same) - 1 && cnt) atomicAdd(in_view + f, __popc(cnt));
        }
    }
}

// The largest positive float r with ceil(logf(r) / log_scale) <= n, by
// bisection over the bit patterns of the positive floats (the quotient is
// non-decreasing in r).
float level_threshold(float log_scale, int n) {
    auto at_most_n = [&](uint32_t bits) {
        float r;
        std::memcpy(&r, &bits, 4);
        return std::ceil(std::log(r) / log_scale) <= (float)n;
    };
    uint32_t lo = 0, hi = 0x7f800000u;  // 0 -> -inf (true), +inf -> +inf (false)
    while (hi - lo > 1) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (at_most_n(mid)) lo = mid;
        else hi = mid;
    }
    float r;
    std::memcpy(&r, &lo, 4);
    return r;
}

}  // namespace orbgpu

using namespace orbgpu;

extern "C" int orbgpu_frustum_frame_init(const float* Tcw, float fx, float fy, float cx, float cy, float bf,
                                         float min_x, float max_x, float min_y, float max_y, float scale_factor,
                                         int nlevels, orbgpu_frustum_frame* out) {
    if (!Tcw || !out || nlevels < 1 || nlevels > 16 || !(scale_factor > 1.0f)) {
        orbgpu_set_last_error("orbgpu_frustum_frame_init: bad arguments", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    std::memset(out, 0, sizeof(*out));
    for (int r = 0; r < 3; r++) {
        for (int c = 0; c < 3; c++) out->Rcw[3 * r + c] = Tcw[4 * r + c];
        out->tcw[r] = Tcw[4 * r + 3];
    }
    // mOw = -mRcw.t() * mtcw (src/Frame.cc:454-470): negation, then a product
    // accumulated in double and rounded to float
    for (int i = 0; i < 3; i++) {
        double s = 0.0;
        for (int k = 0; k < 3; k++) s += (double)(-out->Rcw[3 * k + i]) * (double)out->tcw[k];
        out->Ow[i] = (float)s;
    }
    out->fx = fx;
    out->fy = fy;
    out->cx = cx;
    out->cy = cy;
    out->bf = bf;
    out->min_x = min_x;
    out->max_x = max_x;
    out->min_y = min_y;
    out->max_y = max_y;
    out->nlevels = nlevels;
    // mfLogScaleFactor = log(mfScaleFactor), the float overload (src/Frame.cc:134)
    const float log_scale = std::log(scale_factor);
    for (int n = 0; n < nlevels - 1; n++) out->level_above[n] = level_threshold(log_scale, n);
    return ORBGPU_OK;
}

extern "C" int orbgpu_is_in_frustum(const orbgpu_frustum_frame* frames, int nframes, const int* mp_offsets,
                                    const orbgpu_mappoint_geometry* mps, float viewing_cos_limit,
                                    orbgpu_mappoint* mappoints, int* in_view, void* stream) {
    if (nframes < 0 || (nframes > 0 && (!frames || !mp_offsets || !mps || !mappoints))) {
        orbgpu_set_last_error("orbgpu_is_in_frustum: bad arguments", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (nframes == 0) return ORBGPU_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (in_view) ORBGPU_CUDA_TRY(cudaMemsetAsync(in_view, 0, sizeof(int) * (size_t)nframes, st));
    const int blocks = nsm_of_current_device() * FR_BLOCKS_PER_SM;
    k_is_in_frustum<<<blocks, FR_THREADS, 0, st>>>(frames, nframes, mp_offsets, mps, viewing_cos_limit, mappoints,
                                                    in_view);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    return ORBGPU_OK;
}
