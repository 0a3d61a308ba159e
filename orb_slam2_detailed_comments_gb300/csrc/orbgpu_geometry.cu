// orbgpu_geometry.cu -- per-frame geometry on the device:
// Frame::UndistortKeyPoints / ComputeImageBounds (src/Frame.cc:724-819) and
// Frame::isInFrustum (src/Frame.cc:491-578) with MapPoint::PredictScale(dist,
// Frame*) (src/MapPoint.cc:604-619) for the map points of many frames in one
// launch, writing the records the projection searches read.
//
// Undistortion is cv::undistortPoints as Frame calls it (new camera matrix =
// the camera matrix, no rectification), restated from OpenCV 3.2's
// cvUndistortPoints: in double, normalise with 1/fx, 1/fy, five rounds of
// x = (x0 - tangential) / radial, back through the camera matrix, rounded to
// float.  The same routine runs on the host for the image bounds.
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
#include <algorithm>
#include <cmath>
#include <cstring>

#include "orbgpu_host.h"

namespace orbgpu {

#define FR_THREADS 256
#define FR_BLOCKS_PER_SM 4
#define FR_SMEM_FRAMES 128  // frames staged in shared memory (160 bytes each)

// One camera of the undistortion: the camera matrix entries as doubles,
// 1/fx and 1/fy, and k1 k2 p1 p2 k3 (k3 = 0 for four coefficients).
struct UndistortCamera {
    double fx, fy, cx, cy, ifx, ify;
    double k[5];
};

// One point through cv::undistortPoints(src, dst, K, dist, noArray(), K).
// Plain double operators: device code is compiled without FMA contraction
// (-fmad=false) and host code with -ffp-contract=off, so both evaluate the
// same IEEE operations in this order.
__host__ __device__ inline void undistort_point(const UndistortCamera& c, float& u, float& v) {
    const double x0 = ((double)u - c.cx) * c.ifx;
    const double y0 = ((double)v - c.cy) * c.ify;
    double x = x0, y = y0;
    for (int it = 0; it < 5; it++) {
        const double r2 = x * x + y * y;
        const double icdist = 1.0 / (1 + ((c.k[4] * r2 + c.k[1]) * r2 + c.k[0]) * r2);
        const double dx = 2 * c.k[2] * x * y + c.k[3] * (r2 + 2 * x * x);
        const double dy = c.k[2] * (r2 + 2 * y * y) + 2 * c.k[3] * x * y;
        x = (x0 - dx) * icdist;
        y = (y0 - dy) * icdist;
    }
    u = (float)(c.fx * x + 0.0 * y + c.cx);
    v = (float)(0.0 * x + c.fy * y + c.cy);
}

static bool undistort_camera(const float* K4, const float* dist, int ndist, UndistortCamera* c) {
    if (!K4 || !dist || (ndist != 4 && ndist != 5)) return false;
    c->fx = K4[0];
    c->fy = K4[1];
    c->cx = K4[2];
    c->cy = K4[3];
    c->ifx = 1. / c->fx;
    c->ify = 1. / c->fy;
    for (int i = 0; i < 5; i++) c->k[i] = i < ndist ? (double)dist[i] : 0.0;
    return true;
}

// Keypoint records are 7 words (x, y, size, angle, response, octave,
// class_id); one thread per keypoint.
__global__ void __launch_bounds__(FR_THREADS) k_undistort_keypoints(const float* __restrict__ in, int n,
                                                                    UndistortCamera cam, int copy_only,
                                                                    float* __restrict__ out) {
    const int stride = gridDim.x * FR_THREADS;
    for (int i = blockIdx.x * FR_THREADS + threadIdx.x; i < n; i += stride) {
        float w[7];
#pragma unroll
        for (int q = 0; q < 7; q++) w[q] = in[7 * (size_t)i + q];
        if (!copy_only) undistort_point(cam, w[0], w[1]);
#pragma unroll
        for (int q = 0; q < 7; q++) out[7 * (size_t)i + q] = w[q];
    }
}

__global__ void __launch_bounds__(FR_THREADS) k_is_in_frustum(const orbgpu_frustum_frame* frames,
                                                              int nframes, const int* offsets,
                                                              const orbgpu_mappoint_geometry* __restrict__ mps,
                                                              float cos_limit, orbgpu_mappoint* __restrict__ out,
                                                              int* __restrict__ in_view) {
    // the frames and their offsets staged in shared memory (up to
    // FR_SMEM_FRAMES of them; larger batches read them from global memory)
    __shared__ orbgpu_frustum_frame s_frames[FR_SMEM_FRAMES];
    __shared__ int s_off[FR_SMEM_FRAMES + 1];
    const bool staged = nframes <= FR_SMEM_FRAMES;
    if (staged) {
        const int words = nframes * (int)(sizeof(orbgpu_frustum_frame) / 4);
        for (int k = threadIdx.x; k < words; k += blockDim.x)
            reinterpret_cast<float*>(s_frames)[k] = reinterpret_cast<const float*>(frames)[k];
        for (int k = threadIdx.x; k <= nframes; k += blockDim.x) s_off[k] = offsets[k];
        __syncthreads();
        frames = s_frames;
        offsets = s_off;
    }
    const int first = offsets[0], last = offsets[nframes];
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
                if (offsets[mid] <= i) lo = mid;
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

extern "C" int orbgpu_undistort_keypoints(const orbgpu_keypoint* kps, int n, const float* K4, const float* dist,
                                          int ndist, orbgpu_keypoint* out, void* stream) {
    UndistortCamera cam;
    if (n < 0 || (n > 0 && (!kps || !out)) || !undistort_camera(K4, dist, ndist, &cam)) {
        orbgpu_set_last_error("orbgpu_undistort_keypoints: bad arguments", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (n == 0) return ORBGPU_OK;
    // the reference returns mvKeys unchanged when mDistCoef(0) == 0
    const int copy_only = dist[0] == 0.0f ? 1 : 0;
    const int blocks = (int)std::min<long long>(((long long)n + FR_THREADS - 1) / FR_THREADS,
                                                (long long)nsm_of_current_device() * FR_BLOCKS_PER_SM * 2);
    k_undistort_keypoints<<<blocks, FR_THREADS, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float*>(kps), n, cam, copy_only, reinterpret_cast<float*>(out));
    ORBGPU_CUDA_TRY(cudaGetLastError());
    return ORBGPU_OK;
}

extern "C" int orbgpu_compute_image_bounds(int cols, int rows, const float* K4, const float* dist, int ndist,
                                           float* bounds) {
    UndistortCamera cam;
    if (cols < 0 || rows < 0 || !bounds || !undistort_camera(K4, dist, ndist, &cam)) {
        orbgpu_set_last_error("orbgpu_compute_image_bounds: bad arguments", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (dist[0] == 0.0f) {
        bounds[0] = 0.0f;
        bounds[1] = (float)cols;
        bounds[2] = 0.0f;
        bounds[3] = (float)rows;
        return ORBGPU_OK;
    }
    // corners top-left, top-right, bottom-left, bottom-right
    float u[4] = {0.0f, (float)cols, 0.0f, (float)cols}, v[4] = {0.0f, 0.0f, (float)rows, (float)rows};
    for (int c = 0; c < 4; c++) undistort_point(cam, u[c], v[c]);
    bounds[0] = std::min(u[0], u[2]);
    bounds[1] = std::max(u[1], u[3]);
    bounds[2] = std::min(v[0], v[1]);
    bounds[3] = std::max(v[2], v[3]);
    return ORBGPU_OK;
}

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
