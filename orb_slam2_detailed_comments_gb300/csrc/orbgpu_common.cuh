// orbgpu_common.cuh -- shared device helpers of the ORB front-end kernels.
//
// Every floating-point expression that the reference evaluates in float is
// evaluated here with explicitly rounded single-precision intrinsics
// (__fmul_rn, __fadd_rn, __fdiv_rn, ...), so no multiply-add is ever fused
// and results are bit-identical to the reference's uncontracted -std=c++11
// build.  The library is also compiled with -fmad=false.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/orbgpu.h"

#define ORBGPU_MAX_LEVELS 16
#define ORBGPU_EDGE_THRESHOLD 19
#define ORBGPU_HALF_PATCH 15
#define ORBGPU_PATCH_SIZE 31
#define ORBGPU_GRID_COLS 64
#define ORBGPU_GRID_ROWS 48
#define ORBGPU_TH_HIGH 100
#define ORBGPU_TH_LOW 50
#define ORBGPU_HISTO_LENGTH 30
#define ORBGPU_MAX_DIM 4096

namespace orbgpu {

// ---------------------------------------------------------------- rounding
// cvRound: round half to even (lrintf under the default rounding mode).
__device__ __forceinline__ int cv_round(float v) { return __float2int_rn(v); }
// std::round(float): half away from zero.
__device__ __forceinline__ float round_half_away(float v) { return roundf(v); }

// cv::fastAtan2 stand-in (7th-order odd minimax polynomial of atan on [0, 1],
// degrees), evaluated step by step like the host definition.
__device__ __forceinline__ float fast_atan2_deg(float y, float x) {
    const float k180pi = (float)(180 / 3.141592653589793238);
    const float p1 = 0.9997878412794807f * k180pi;
    const float p3 = -0.3258083974640975f * k180pi;
    const float p5 = 0.1555786518463281f * k180pi;
    const float p7 = -0.04432655554792128f * k180pi;
    const float eps = (float)2.220446049250313e-16;
    const float ax = fabsf(x), ay = fabsf(y);
    float a, c, c2;
    if (ax >= ay) {
        c = __fdiv_rn(ay, __fadd_rn(ax, eps));
        c2 = __fmul_rn(c, c);
        a = __fmul_rn(__fadd_rn(__fmul_rn(__fadd_rn(__fmul_rn(__fadd_rn(__fmul_rn(p7, c2), p5), c2), p3), c2), p1), c);
    } else {
        c = __fdiv_rn(ax, __fadd_rn(ay, eps));
        c2 = __fmul_rn(c, c);
        a = __fsub_rn(90.f, __fmul_rn(__fadd_rn(__fmul_rn(__fadd_rn(__fmul_rn(__fadd_rn(__fmul_rn(p7, c2), p5), c2), p3), c2), p1), c));
    }
    if (x < 0) a = __fsub_rn(180.f, a);
    if (y < 0) a = __fsub_rn(360.f, a);
    return a;
}

// ORBmatcher::DescriptorDistance (src/ORBmatcher.cc:2083-2103): popcount of
// the XOR of two 256-bit rows.
__device__ __forceinline__ int hamming256(const uint4 a0, const uint4 a1, const uint4 b0, const uint4 b1) {
    return __popc(a0.x ^ b0.x) + __popc(a0.y ^ b0.y) + __popc(a0.z ^ b0.z) + __popc(a0.w ^ b0.w) +
           __popc(a1.x ^ b1.x) + __popc(a1.y ^ b1.y) + __popc(a1.z ^ b1.z) + __popc(a1.w ^ b1.w);
}

__device__ __forceinline__ int hamming256_ptr(const uint8_t* a, const uint8_t* b) {
    const uint4* pa = reinterpret_cast<const uint4*>(a);
    const uint4* pb = reinterpret_cast<const uint4*>(b);
    return hamming256(pa[0], pa[1], pb[0], pb[1]);
}

// ---------------------------------------------------------------- warp helpers
__device__ __forceinline__ int warp_sum(int v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}
__device__ __forceinline__ int warp_min_i(int v) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// The keypoint indices of the grid cells [x0, x1] x [y0, y1] (cell c =
// ix * rows + iy, lists in CSR form: cell_start / cell_keys) in
// Frame::GetFeaturesInArea's order (cells by ix then iy, each cell's list in
// order), for W-lane segments of a warp (W = 8, 16 or 32), each segment with
// its own window: segment g holds lanes [g W, g W + W).  Cells are stored
// column-major (cell = x * rows + y) and their key lists back to back, so
// the window's keys of grid column x are one range of cell_keys: one lane per
// column instead of one per cell.
// Keys are visited column by column, cell by cell within a column, in list
// order within a cell (GetFeaturesInArea's order); the visitor learns a
// key's cell from the binning.  Every lane of the warp runs the loops to the
// longest segment's bounds (a segment with active == false, or past its own
// bounds, visits with valid == false), so the visitor may use full-warp
// ballots and shuffles.
template <int W, typename Visit>
__device__ __forceinline__ void seg_window_cols(const int* cell_start, const int* cell_keys, int rows, bool active,
                                                int x0, int x1, int y0, int y1, Visit visit) {
    static_assert(W == 8 || W == 16 || W == 32, "segment width");
    const int sl = (threadIdx.x & 31) & (W - 1);
    const int ncol = active && y1 >= y0 ? x1 - x0 + 1 : 0;
    int nmax = ncol;
#pragma unroll
    for (int o = W; o < 32; o <<= 1) nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, o));
    for (int c0 = 0; c0 < nmax; c0 += W) {
        const int cx = c0 + sl;
        int s = 0, n = 0;
        if (cx < ncol) {
            const int base = (x0 + cx) * rows;
            s = cell_start[base + y0];
            n = cell_start[base + y1 + 1] - s;
        }
        int incl = n;
#pragma unroll
        for (int o = 1; o < W; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o, W);
            if (sl >= o) incl += y;
        }
        const int total = __shfl_sync(0xffffffffu, incl, W - 1, W);
        const int excl = incl - n;
        int tmax = total;
#pragma unroll
        for (int o = W; o < 32; o <<= 1) tmax = max(tmax, __shfl_xor_sync(0xffffffffu, tmax, o));
        for (int t0 = 0; t0 < tmax; t0 += W) {
            const int t = t0 + sl;
            // the last lane of the segment whose range starts at or before t holds entry t
            int k = 0;
#pragma unroll
            for (int step = W / 2; step > 0; step >>= 1) {
                const int e = __shfl_sync(0xffffffffu, excl, k + step, W);
                if (e <= t) k += step;
            }
            const int sk = __shfl_sync(0xffffffffu, s, k, W);
            const int ek = __shfl_sync(0xffffffffu, excl, k, W);
            const bool valid = t < total;
            visit(valid ? cell_keys[sk + t - ek] : -1, valid);
        }
    }
}

// The keypoints of the grid cells [x0, x1] x [y0, y1] for one whole warp
// (seg_window_cols with one 32-lane segment); the visitor also gets the
// key's cell (key_cell: the cell of every key from the binning).
template <typename Visit>
__device__ __forceinline__ void warp_window_keys(const int* cell_start, const int* cell_keys, const int* key_cell,
                                                 int rows, int x0, int x1, int y0, int y1, Visit visit) {
    seg_window_cols<32>(cell_start, cell_keys, rows, true, x0, x1, y0, y1, [&](int idx, bool valid) {
        visit(idx, valid ? key_cell[idx] : 0, valid);
    });
}

// Block-wide exclusive scan of one int per thread; returns the block total.
// 'smem' must hold 32 ints.  All threads of the block must call it.
__device__ __forceinline__ int block_exclusive_scan(int v, int* smem, int* total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int s = lane < nw ? smem[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        smem[lane] = s;
    }
    __syncthreads();
    const int warp_prefix = wid > 0 ? smem[wid - 1] : 0;
    const int t = smem[nw - 1];
    __syncthreads();
    if (total) *total = t;
    return warp_prefix + x - v;
}

// ---------------------------------------------------------------- sin / cos
// sin and cos of a float angle in [0, 2*pi] evaluated in double precision
// from the Taylor series after a three-part Cody-Waite reduction by pi/2,
// using only IEEE double + - * (no fused operations), so host and device
// produce the same bits.  Callers that must agree with the host C library's
// cosf/sinf bit for bit correct the rare inputs where the float rounding of
// this value differs with a sorted exception table built on the host.
__host__ __device__ inline void sincos_taylor(float xf, double* s_out, double* c_out) {
    const double x = (double)xf;
    const double two_over_pi = 0x1.45f306dc9c883p-1;
    const double P1 = 0x1.921fb548p+0, P2 = -0x1.de973dc8p-31, P3 = -0x1.9d9cceba3f91fp-62;
#ifdef __CUDA_ARCH__
    const double kd = floor(__dadd_rn(__dmul_rn(x, two_over_pi), 0.5));
    double r = __dsub_rn(x, __dmul_rn(kd, P1));
    r = __dsub_rn(r, __dmul_rn(kd, P2));
    r = __dsub_rn(r, __dmul_rn(kd, P3));
    const double r2 = __dmul_rn(r, r);
#define ORB_DM(a, b) __dmul_rn(a, b)
#define ORB_DA(a, b) __dadd_rn(a, b)
#else
    const double kd = floor(x * two_over_pi + 0.5);
    double r = x - kd * P1;
    r = r - kd * P2;
    r = r - kd * P3;
    const double r2 = r * r;
#define ORB_DM(a, b) ((a) * (b))
#define ORB_DA(a, b) ((a) + (b))
#endif
    // sin r = r * (1 - r2/3! + r2^2/5! - ...), cos r = 1 - r2/2! + ...
    const double s_c[12] = {-0x1.5555555555555p-3, 0x1.1111111111111p-7, -0x1.a01a01a01a01ap-13,
                            0x1.71de3a556c734p-19, -0x1.ae64567f544e4p-26, 0x1.6124613a86d09p-33,
                            -0x1.ae7f3e733b81fp-41, 0x1.952c77030ad4ap-49, -0x1.2f49b46814157p-57,
                            0x1.71b8ef6dcf572p-66, -0x1.761b41316381ap-75, 0x1.3f3ccdd165fa9p-84};
    const double c_c[12] = {-0x1.0000000000000p-1, 0x1.5555555555555p-5, -0x1.6c16c16c16c17p-10,
                            0x1.a01a01a01a01ap-16, -0x1.27e4fb7789f5cp-22, 0x1.1eed8eff8d898p-29,
                            -0x1.93974a8c07c9dp-37, 0x1.ae7f3e733b81fp-45, -0x1.6827863b97d97p-53,
                            0x1.e542ba4020225p-62, -0x1.0ce396db7f853p-70, 0x1.f2cf01972f578p-80};
    double ps = s_c[11], pc = c_c[11];
    for (int i = 10; i >= 0; i--) {
        ps = ORB_DA(ORB_DM(ps, r2), s_c[i]);
        pc = ORB_DA(ORB_DM(pc, r2), c_c[i]);
    }
    const double sr = ORB_DA(r, ORB_DM(ORB_DM(r, r2), ps));
    const double cr = ORB_DA(1.0, ORB_DM(r2, pc));
#undef ORB_DM
#undef ORB_DA
    const int k = ((int)kd) & 3;
    double s, c;
    if (k == 0) { s = sr; c = cr; }
    else if (k == 1) { s = cr; c = -sr; }
    else if (k == 2) { s = -sr; c = -cr; }
    else { s = -cr; c = sr; }
    *s_out = s;
    *c_out = c;
}

}  // namespace orbgpu

// Internal error reporting of the library.
#define ORBGPU_CUDA_TRY(expr)                                           \
    do {                                                                \
        cudaError_t _e = (expr);                                        \
        if (_e != cudaSuccess) {                                        \
            orbgpu_set_last_error(cudaGetErrorString(_e), __FILE__, __LINE__); \
            return _e == cudaErrorMemoryAllocation ? ORBGPU_ERR_OOM : ORBGPU_ERR_CUDA; \
        }                                                               \
    } while (0)

void orbgpu_set_last_error(const char* msg, const char* file, int line);

namespace orbgpu {
// cudaMalloc of the library's working buffers, except while a test has asked
// (orbgpu_debug_fail_allocations) for allocations to fail: then it returns
// cudaErrorMemoryAllocation without allocating.
cudaError_t dev_malloc(void** p, size_t bytes);
template <typename T> inline cudaError_t dev_malloc(T** p, size_t bytes) { return dev_malloc((void**)p, bytes); }
}  // namespace orbgpu
