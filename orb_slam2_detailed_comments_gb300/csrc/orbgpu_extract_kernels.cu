// orbgpu_extract_kernels.cu -- the ORB extraction stages (see the .cuh).
#include <algorithm>

#include "orbgpu_async.cuh"
#include "orbgpu_extract_kernels.cuh"
#include "orb_pattern.h"
#include "orbgpu_host.h"

namespace orbgpu {

__constant__ int c_gauss_taps[7];
__constant__ int c_umax[ORBGPU_HALF_PATCH + 1];
__constant__ signed char c_pattern[256 * 4];

// Exception table of the descriptor rotation: sorted float bit patterns x for
// which the host C library's cosf(x)/sinf(x) differ from the rounded
// sincos_taylor(x) value, with the library's results.
__device__ const uint32_t* g_cos_exc_key = nullptr;
__device__ const float* g_cos_exc_val = nullptr;
__device__ int g_cos_exc_n = 0;
__device__ const uint32_t* g_sin_exc_key = nullptr;
__device__ const float* g_sin_exc_val = nullptr;
__device__ int g_sin_exc_n = 0;
// bucket index (input bits >> ORBGPU_EXC_SHIFT) -> first table entry, one
// array per table, nbuckets + 1 entries each; inside bucket b, sub-bucket s
// (the next ORBGPU_EXC_SUB_BITS input bits) starts sub[b * 64 + s] entries
// after the bucket's first
#define ORBGPU_EXC_SHIFT 12
#define ORBGPU_EXC_SUB_BITS 6
__device__ const int* g_cos_exc_bucket = nullptr;
__device__ const int* g_sin_exc_bucket = nullptr;
__device__ const uint16_t* g_cos_exc_sub = nullptr;
__device__ const uint16_t* g_sin_exc_sub = nullptr;
__device__ int g_exc_nbuckets = 0;

__device__ __forceinline__ int reflect101(int p, int len) {
    if (len == 1) return 0;
    while (p < 0 || p >= len) p = p < 0 ? -p : 2 * len - 2 - p;
    return p;
}

// Entry and index of block b within a launch over a RangeMap.
__device__ __forceinline__ void map_item(const RangeMap& rm, int b, int& desc, int& index) {
    int lo = 0, hi = rm.n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (rm.prefix[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    desc = rm.desc0 + lo * rm.desc_stride;
    index = b - rm.prefix[lo];
}

// ---------------------------------------------------------------- FAST
// The 16 pixels of the radius-3 Bresenham circle in cyclic order, as
// offsets from the centre for a row stride 'rw': (dx, dy) = (0,3) (1,3)
// (2,2) (3,1) (3,0) (3,-1) (2,-2) (1,-3) (0,-3) (-1,-3) (-2,-2) (-3,-1)
// (-3,0) (-3,1) (-2,2) (-1,3).
__host__ __device__ __forceinline__ void load_circle(const uint8_t* cp, int rw, int p[16]) {
    p[0] = cp[3 * rw];
    p[1] = cp[3 * rw + 1];
    p[2] = cp[2 * rw + 2];
    p[3] = cp[rw + 3];
    p[4] = cp[3];
    p[5] = cp[-rw + 3];
    p[6] = cp[-2 * rw + 2];
    p[7] = cp[-3 * rw + 1];
    p[8] = cp[-3 * rw];
    p[9] = cp[-3 * rw - 1];
    p[10] = cp[-2 * rw - 2];
    p[11] = cp[-rw - 3];
    p[12] = cp[-3];
    p[13] = cp[rw - 3];
    p[14] = cp[2 * rw - 2];
    p[15] = cp[3 * rw - 1];
}

__host__ __device__ __forceinline__ bool has_run9(uint32_t m) {
    uint32_t m32 = m | (m << 16);
    uint32_t r = m32 & (m32 >> 1);
    r &= r >> 2;
    r &= r >> 4;
    r &= m32 >> 8;
    return (r & 0xFFFFu) != 0;
}

// Max over the 16 cyclic nine-element windows of the window minimum of a
// (by doubling: windows of 2, 4, 8, then 9).  Only min/max of the values
// themselves: the darker- and brighter-centre cases are evaluated on two
// arrays (v - p and p - v) instead of negating inside a max.
__host__ __device__ __forceinline__ int best_window_min9(const int a[16]) {
    int m2[16], m4[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const int x = a[k], y = a[(k + 1) & 15];
        m2[k] = x < y ? x : y;
    }
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const int x = m2[k], y = m2[(k + 2) & 15];
        m4[k] = x < y ? x : y;
    }
    int best = 0;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const int x = m4[k], y = m4[(k + 4) & 15], z = a[(k + 8) & 15];
        int m = x < y ? x : y;
        m = m < z ? m : z;
        best = best > m ? best : m;
    }
    return best;
}

// Necessary condition for a FAST corner at threshold t: two compass points
// (dy = +3, dx = +3, dy = -3, dx = -3) four apart on the circle are both
// brighter than v + t or both darker than v - t.
__device__ __forceinline__ bool compass_test(const uint8_t* cp, int rw, int t) {
    const int v = cp[0];
    const int p0 = cp[3 * rw], p4 = cp[3], p8 = cp[-3 * rw], p12 = cp[-3];
    const int hi = v + t, lo = v - t;
    const bool b0 = p0 > hi, b4 = p4 > hi, b8 = p8 > hi, b12 = p12 > hi;
    const bool d0 = p0 < lo, d4 = p4 < lo, d8 = p8 < lo, d12 = p12 < lo;
    return ((b0 & b4) | (b4 & b8) | (b8 & b12) | (b12 & b0)) | ((d0 & d4) | (d4 & d8) | (d8 & d12) | (d12 & d0));
}

// Largest arc threshold (max over the 16 nine-pixel arcs of the smallest
// absolute difference of consistent sign) if the pixel is a FAST corner at
// threshold t, else 0.
__host__ __device__ __forceinline__ int arc_strength(const uint8_t* roi, int rw, int r, int c, int t) {
    const uint8_t* cp = roi + r * rw + c;
    const int v = cp[0];
    const int p0 = cp[3 * rw], p4 = cp[3], p8 = cp[-3 * rw], p12 = cp[-3];
    const int hi = v + t, lo = v - t;
    const bool b0 = p0 > hi, b4 = p4 > hi, b8 = p8 > hi, b12 = p12 > hi;
    const bool d0 = p0 < lo, d4 = p4 < lo, d8 = p8 < lo, d12 = p12 < lo;
    const bool maybe_b = (b0 & b4) | (b4 & b8) | (b8 & b12) | (b12 & b0);
    const bool maybe_d = (d0 & d4) | (d4 & d8) | (d8 & d12) | (d12 & d0);
    if (!maybe_b && !maybe_d) return 0;
    int pc[16], dark[16], bright[16];
    load_circle(cp, rw, pc);
    uint32_t bm = 0, dm = 0;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const int p = pc[k];
        dark[k] = v - p;    // circle darker than the centre
        bright[k] = p - v;  // circle brighter than the centre
        bm |= (uint32_t)(p > hi) << k;
        dm |= (uint32_t)(p < lo) << k;
    }
    if (!has_run9(bm) && !has_run9(dm)) return 0;
    const int a = best_window_min9(dark), b = best_window_min9(bright);
    return a > b ? a : b;
}

// ---------------------------------------------------------------- resize, blur + FAST strength
// Both kernels tile a level in strips of 120 columns x TH rows, RS_WPB strips
// (one warp each) per block, so they share one block count per level.
#define RS_COLS 120       // level columns per strip
#define RS_WPB 2          // strips (warps) per block
#define RS_CAND (30 * 28) // FAST candidates of one 7-row block at most

// Level l (l >= 1) from level l-1: cv::resize INTER_LINEAR in 11-bit fixed
// point.  Lane k (k < 30) of the strip's warp produces columns
// [x0 + 4k, x0 + 4k + 4) of the strip's rows.  The horizontal pass is one
// dp2a per pixel on the two source bytes that a prmt picks from the lane's
// source words, which are loaded two rows ahead; a source row shared by two
// consecutive output rows is loaded and interpolated once.  Weights come in pairs
// summing to 2047..2049 (checked when the tables are built), so the
// vertical sum 4 (h0 b0 + h1 b1) + 2^23 stays below 2^32 and its byte 3 is
// (h0 b0 + h1 b1 + 2^21) >> 22.
template <int TH>
__global__ void __launch_bounds__(32 * RS_WPB) k_level_resize(const LevelDesc* descs, RangeMap rm) {
    __shared__ int4 s_rows[RS_WPB][TH + 1];  // output row i: source rows r0, r1, 4 b0 | 4 b1 << 16
    WorkItem it;
    map_item(rm, blockIdx.x, it.desc, it.index);
    const LevelDesc& d = descs[it.desc];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = d.w, h = d.h;
    const int tiles_x = (w + RS_COLS - 1) / RS_COLS;
    const int tile = it.index * RS_WPB + warp;
    if (tile >= tiles_x * ((h + TH - 1) / TH)) return;
    const int x0 = (tile % tiles_x) * RS_COLS, y0 = (tile / tiles_x) * TH;
    const int X = x0 + 4 * lane;
    const bool writer = lane < RS_COLS / 4 && X < w;
    int4* rows = s_rows[warp];
    for (int i = lane; i <= TH; i += 32) {
        const int y = min(y0 + i, h - 1);
        const int sy = d.yofs[y];
        rows[i] = make_int4(min(max(sy, 0), d.sh - 1), min(max(sy + 1, 0), d.sh - 1),
                            (4 * (int)d.ybeta[2 * y]) | ((4 * (int)d.ybeta[2 * y + 1]) << 16), 0);
    }
    // per pixel the packed weights (a0 | a1 << 16) and the byte selector of
    // (sx, sx1) among the 8 source bytes from bmin; columns past the level
    // width repeat the last one (their bytes land in the row padding)
    uint32_t coef[4], sel[4];
    int sxs[4], sx1s[4], bmin = 1 << 30, bmax = -1;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int x = min(X + j, w - 1);
        sxs[j] = d.xofs[x];
        sx1s[j] = min(sxs[j] + 1, d.sw - 1);
        coef[j] = (uint32_t)(uint16_t)d.xalpha[2 * x] | ((uint32_t)(uint16_t)d.xalpha[2 * x + 1] << 16);
        bmin = min(bmin, sxs[j]);
        bmax = max(bmax, sx1s[j]);
    }
    const bool fastcols = bmax - bmin <= 7;
    const int sbase = bmin & ~3;
    const uint32_t sshift = 8u * (uint32_t)(bmin & 3);
    const int nwords = writer && fastcols ? (bmax - sbase) / 4 + 1 : 0;
#pragma unroll
    for (int j = 0; j < 4; j++) sel[j] = (uint32_t)(sxs[j] - bmin) | ((uint32_t)(sx1s[j] - bmin) << 4);
    __syncwarp();

    // the level descriptor's fields as locals: the byte stores below could
    // otherwise alias them and force reloads
    const uint8_t* const src = d.src;
    const int spitch = d.spitch;
    auto source_words = [&](int s, uint32_t& w0, uint32_t& w1, uint32_t& w2) {
        const uint8_t* p = src + (size_t)s * spitch + sbase;
        w0 = nwords > 0 ? *reinterpret_cast<const uint32_t*>(p) : 0u;
        w1 = nwords > 1 ? *reinterpret_cast<const uint32_t*>(p + 4) : 0u;
        w2 = nwords > 2 ? *reinterpret_cast<const uint32_t*>(p + 8) : 0u;
    };
    auto hinterp = [&](int s, uint32_t w0, uint32_t w1, uint32_t w2, uint32_t* hv) {
        if (fastcols) {
            const uint32_t W0 = __funnelshift_r(w0, w1, sshift), W1 = __funnelshift_r(w1, w2, sshift);
#pragma unroll
            for (int j = 0; j < 4; j++) hv[j] = __dp2a_lo(coef[j], __byte_perm(W0, W1, sel[j]), 0u);
        } else {
            // source columns more than 7 apart (scale factors above about 1.6)
            const uint8_t* row = src + (size_t)s * spitch;
#pragma unroll
            for (int j = 0; j < 4; j++)
                hv[j] = (uint32_t)row[sxs[j]] * (coef[j] & 0xFFFFu) + (uint32_t)row[sx1s[j]] * (coef[j] >> 16);
        }
    };

    const int nrows = min(TH, h - y0);
    // source words of output rows i (set i & 1) and i + 1, loaded two rows ahead
    uint32_t pw[2][6];
    {
        const int4 e0 = rows[0], e1 = rows[min(1, TH)];
        source_words(e0.x, pw[0][0], pw[0][1], pw[0][2]);
        source_words(e0.y, pw[0][3], pw[0][4], pw[0][5]);
        source_words(e1.x, pw[1][0], pw[1][1], pw[1][2]);
        source_words(e1.y, pw[1][3], pw[1][4], pw[1][5]);
    }
    uint8_t* out = d.dst + (size_t)y0 * d.pitch + X;
    // an output row's first source row is usually the previous output row's
    // second (scale 1.2): its horizontal pass is reused, and its words are
    // not loaded (the test is the same for every lane of the warp)
    uint32_t hlast[4] = {0u, 0u, 0u, 0u};
    int rlast = -1;  // source row of hlast
    auto row_step = [&](int i, uint32_t* cur) {
        const int4 e = rows[i];
        uint32_t ha[4], hb[4];
        if (e.x == rlast) {
#pragma unroll
            for (int j = 0; j < 4; j++) ha[j] = hlast[j];
        } else {
            hinterp(e.x, cur[0], cur[1], cur[2], ha);
        }
        hinterp(e.y, cur[3], cur[4], cur[5], hb);
        rlast = e.y;
#pragma unroll
        for (int j = 0; j < 4; j++) hlast[j] = hb[j];
        const int4 e1 = rows[min(i + 1, TH)], e2 = rows[min(i + 2, TH)];
        if (e2.x != e1.y) source_words(e2.x, cur[0], cur[1], cur[2]);
        source_words(e2.y, cur[3], cur[4], cur[5]);
        const uint32_t B0 = (uint32_t)e.z & 0xFFFFu, B1 = (uint32_t)e.z >> 16;
        uint32_t v[4];
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = ha[j] * B0 + hb[j] * B1 + (1u << 23);
        if (writer)
            *reinterpret_cast<uint32_t*>(out + (size_t)i * d.pitch) =
                __byte_perm(__byte_perm(v[0], v[1], 0x0073), __byte_perm(v[2], v[3], 0x0073), 0x5410);
    };
    for (int i = 0; i < nrows; i += 2) {
        row_step(i, pw[0]);
        if (i + 1 < nrows) row_step(i + 1, pw[1]);
    }
}

// The 7x7 Gaussian (8-bit fixed point, REFLECT_101) of every pixel of level l
// and the FAST compass pre-test of every pixel of the cells' detection
// region.  Lane k holds the four pixels of columns [x0 - 4 + 4k, x0 + 4k) of a
// row as one 32-bit word: lanes 1..30 own the strip's columns, lanes 0 and 31
// the 4-column halos (reflected outside the level).  The warp walks the
// TH + 6 rows [y0 - 3, y0 + TH + 3) top to bottom with the last seven rows in
// registers:
//  * horizontal sums by two dp4a per pixel from the lane's word and its
//    neighbours' (shuffles), the vertical pass over seven rows of sums;
//  * FAST at the lower threshold t: the compass-point pre-test (two circle
//    points among 0, 4, 8, 12 that are adjacent on the circle both brighter
//    than v + t or both darker than v - t; every nine-pixel arc contains such
//    a pair) in 16-bit lanes gives the level's candidate bit map: the lanes of
//    a pair (odd, even) own the 8 columns of one byte (x0 is a multiple of 8),
//    so each row costs one shuffle and one byte store per pair; k_fast_cells
//    scores the candidates.
// Only rows and columns [19, dim - 19) are tested: every cell's detection
// region lies inside them (cells start at EDGE_THRESHOLD - 3 + 3 and end 3
// before maxBorder = dim - EDGE_THRESHOLD + 3), and k_fast_cells reads
// nothing else.
// The warps of a block share nothing: no block-level synchronisation.
template <int TH>
struct StripShared {
    int rows[TH + 7];  // input row i: reflected level row
};

// Even (bytes 0, 2) and odd (bytes 1, 3) pixels of a word in 16-bit lanes.
__device__ __forceinline__ uint32_t rs_even(uint32_t w) { return w & 0x00FF00FFu; }
__device__ __forceinline__ uint32_t rs_odd(uint32_t w) { return __byte_perm(w, 0u, 0x4341); }

// Compass pre-test of the two pixels in the 16-bit lanes of c (centres) and
// p0, p4, p8, p12 (circle points), K = (0x8000 - t - 1) in both lanes: every
// lane sum stays within [0x7E01, 0x80FE], so no borrow crosses lanes and bit
// 15 of a lane is set exactly when p - c > t (or c - p > t).  Returns bit 15 /
// bit 31 set for candidates.
__device__ __forceinline__ uint32_t rs_compass(uint32_t c, uint32_t p0, uint32_t p4, uint32_t p8, uint32_t p12,
                                               uint32_t K) {
    const uint32_t b0 = p0 + K - c, b4 = p4 + K - c, b8 = p8 + K - c, b12 = p12 + K - c;
    const uint32_t d0 = c + K - p0, d4 = c + K - p4, d8 = c + K - p8, d12 = c + K - p12;
    // adjacent pairs (0,4) (4,8) (8,12) (12,0) == (0 | 8) & (4 | 12)
    return (((b0 | b8) & (b4 | b12)) | ((d0 | d8) & (d4 | d12))) & 0x80008000u;
}

template <int TH>
__global__ void __launch_bounds__(32 * RS_WPB, 12) k_level_strip(const LevelDesc* descs, RangeMap rm) {
    static_assert((TH + 6) % 7 == 0, "TH + 6 rows must be whole blocks of 7");
    constexpr int NB = (TH + 6) / 7;
    __shared__ __align__(16) StripShared<TH> sh_all[RS_WPB];
    WorkItem it;
    map_item(rm, blockIdx.x, it.desc, it.index);
    const LevelDesc& d = descs[it.desc];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = d.w, h = d.h, pitch = d.pitch;
    const int tiles_x = (w + RS_COLS - 1) / RS_COLS;
    const int tile = it.index * RS_WPB + warp;
    if (tile >= tiles_x * ((h + TH - 1) / TH)) return;
    StripShared<TH>& S = sh_all[warp];
    const int x0 = (tile % tiles_x) * RS_COLS, y0 = (tile / tiles_x) * TH;
    const int X = x0 - 4 + 4 * lane;
    const bool writer = lane >= 1 && lane <= 30 && X < w;
    // the lane's pixels inside the detection region's columns
    uint32_t colmask = 0;
#pragma unroll
    for (int j = 0; j < 4; j++)
        if (writer && X + j >= ORBGPU_EDGE_THRESHOLD && X + j < w - ORBGPU_EDGE_THRESHOLD) colmask |= 1u << j;
    const int t = min(min(max(d.ini_th, 0), 255), min(max(d.min_th, 0), 255));
    const uint32_t K = (0x8000u - (uint32_t)t - 1u) * 0x00010001u;
    for (int i = lane; i < TH + 7; i += 32) S.rows[i] = reflect101(y0 - 3 + min(i, TH + 5), h);
    // the lane's columns, reflected at the level edges
    int xr[4];
#pragma unroll
    for (int j = 0; j < 4; j++) xr[j] = reflect101(X + j, w);
    const bool interior = X >= 0 && X + 3 < w;
    __syncwarp();
    const uint32_t TA = (uint32_t)c_gauss_taps[0] | ((uint32_t)c_gauss_taps[1] << 8) |
                        ((uint32_t)c_gauss_taps[2] << 16) | ((uint32_t)c_gauss_taps[3] << 24);
    const uint32_t TB = (uint32_t)c_gauss_taps[4] | ((uint32_t)c_gauss_taps[5] << 8) | ((uint32_t)c_gauss_taps[6] << 16);
    // tap pairs of the vertical pass (bytes 0, 1 for dp2a)
    const uint32_t T01 = (uint32_t)c_gauss_taps[0] | ((uint32_t)c_gauss_taps[1] << 8);
    const uint32_t T23 = (uint32_t)c_gauss_taps[2] | ((uint32_t)c_gauss_taps[3] << 8);
    const uint32_t T45 = (uint32_t)c_gauss_taps[4] | ((uint32_t)c_gauss_taps[5] << 8);
    const uint32_t T6 = (uint32_t)c_gauss_taps[6];
    // the level descriptor's fields as locals: the stores below could
    // otherwise alias them and force reloads
    const uint8_t* const lvl = d.dst;
    uint8_t* const blur = d.blur;
    // candidate bytes: the odd writer lane of a pair stores columns X .. X + 7
    const bool cwriter = writer && (lane & 1);
    uint8_t* const cbits = d.cbits + (cwriter ? X >> 3 : 0);
    const int cstride = d.cbits_stride;
    auto level_word = [&](int rr) -> uint32_t {
        const uint8_t* row = lvl + (size_t)rr * pitch;
        if (interior) return *reinterpret_cast<const uint32_t*>(row + X);
        return (uint32_t)row[xr[0]] | ((uint32_t)row[xr[1]] << 8) | ((uint32_t)row[xr[2]] << 16) |
               ((uint32_t)row[xr[3]] << 24);
    };

    uint32_t cw[7], pr[7][4], hprev[4] = {0, 0, 0, 0};
    // level rows in flight: q[u] holds input row 7 blk + u, loaded one block
    // (seven rows) ahead
    uint32_t q[7];
#pragma unroll
    for (int u = 0; u < 7; u++) q[u] = level_word(S.rows[u]);
    for (int blk = 0; blk < NB; blk++) {
#pragma unroll
        for (int u = 0; u < 7; u++) {
            const int i = 7 * blk + u;
            const uint32_t c = q[u];
            if (blk + 1 < NB) q[u] = level_word(S.rows[i + 7]);
            const uint32_t l = __shfl_up_sync(0xffffffffu, c, 1), r = __shfl_down_sync(0xffffffffu, c, 1);
            cw[u] = c;
            // horizontal Gaussian sums of the lane's 4 pixels (columns X + j - 3 .. X + j + 3; at most
            // 255 * 257 = 65535), paired with the previous row's in 16-bit halves
            uint32_t hcur[4];
            hcur[0] = __dp4a(__funnelshift_r(l, c, 8), TA, __dp4a(__funnelshift_r(c, r, 8), TB, 0u));
            hcur[1] = __dp4a(__funnelshift_r(l, c, 16), TA, __dp4a(__funnelshift_r(c, r, 16), TB, 0u));
            hcur[2] = __dp4a(__funnelshift_r(l, c, 24), TA, __dp4a(__funnelshift_r(c, r, 24), TB, 0u));
            hcur[3] = __dp4a(c, TA, __dp4a(r, TB, 0u));
#pragma unroll
            for (int j = 0; j < 4; j++) {
                pr[u][j] = __byte_perm(hprev[j], hcur[j], 0x5410);  // rows i - 1 | i << 16
                hprev[j] = hcur[j];
            }
            if (blk > 0 || u == 6) {
                const int y = y0 + i - 6;  // output row: input rows i - 6 .. i
                if (y < h) {
                    // vertical pass over rows i - 6 .. i as three row pairs and row i;
                    // (acc + 2^15) >> 16 clamped to 255 == byte 2 of min(acc + 2^15, 2^24 - 1)
                    uint32_t acc[4];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        uint32_t s = __dp2a_lo(pr[(u + 2) % 7][j], T01, (1u << 15) + T6 * hcur[j]);
                        s = __dp2a_lo(pr[(u + 4) % 7][j], T23, s);
                        s = __dp2a_lo(pr[(u + 6) % 7][j], T45, s);
                        acc[j] = min(s, 0xFFFFFFu);
                    }
                    const uint32_t blurw =
                        __byte_perm(__byte_perm(acc[0], acc[1], 0x0062), __byte_perm(acc[2], acc[3], 0x0062), 0x5410);
                    if (writer) *reinterpret_cast<uint32_t*>(blur + (size_t)y * pitch + X) = blurw;
                    if (y >= ORBGPU_EDGE_THRESHOLD && y < h - ORBGPU_EDGE_THRESHOLD) {
                        const int cc = (u + 4) % 7, up = (u + 1) % 7;
                        const uint32_t cm = cw[cc];
                        const uint32_t lm = __shfl_up_sync(0xffffffffu, cm, 1), rm_ = __shfl_down_sync(0xffffffffu, cm, 1);
                        const uint32_t p4 = __funnelshift_r(cm, rm_, 24), p12 = __funnelshift_r(lm, cm, 8);
                        const uint32_t E = rs_compass(rs_even(cm), rs_even(cw[u]), rs_even(p4), rs_even(cw[up]),
                                                      rs_even(p12), K);
                        const uint32_t O =
                            rs_compass(rs_odd(cm), rs_odd(cw[u]), rs_odd(p4), rs_odd(cw[up]), rs_odd(p12), K);
                        const uint32_t m = (E >> 15) | (O >> 14);  // pixels 0, 1 at bits 0, 1; 2, 3 at bits 16, 17
                        const uint32_t nib = (m | (m >> 14)) & colmask & 0xFu;
                        const uint32_t nib_next = __shfl_down_sync(0xffffffffu, nib, 1);
                        if (cwriter) cbits[(size_t)y * cstride] = (uint8_t)(nib | (nib_next << 4));
                    }
                }
            }
        }
    }
}

#define FAST_MAX_ROI 72
#define FAST_MAX_DET (FAST_MAX_ROI - 6)

// Largest arc threshold of the pixel at cp (row pitch rw, a shared-memory
// tile): max over the sixteen nine-pixel arcs of the arc's smallest
// difference, for the darker-centre (v - p) and brighter-centre (p - v)
// differences clipped at 0, which travel together in the 16-bit halves of one
// word.  Above t exactly when the pixel is a FAST corner at threshold t.
__device__ __forceinline__ int tile_arc_strength(const uint8_t* cp, int rw) {
    const uint32_t v = cp[0];
    const uint32_t p[16] = {cp[3 * rw],  cp[3 * rw + 1],  cp[2 * rw + 2],  cp[rw + 3],  cp[3],      cp[-rw + 3],
                            cp[-2 * rw + 2], cp[-3 * rw + 1], cp[-3 * rw], cp[-3 * rw - 1], cp[-2 * rw - 2],
                            cp[-rw - 3], cp[-3],          cp[rw - 3],      cp[2 * rw - 2], cp[3 * rw - 1]};
    uint32_t a[16], m2[16], m4[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        const uint32_t x = p[k] | (v << 16), y = v | (p[k] << 16);
        a[k] = __vmaxu2(x, y) - x;  // (v - p)+ | (p - v)+ << 16
    }
#pragma unroll
    for (int k = 0; k < 16; k++) m2[k] = __vminu2(a[k], a[(k + 1) & 15]);
#pragma unroll
    for (int k = 0; k < 16; k++) m4[k] = __vminu2(m2[k], m2[(k + 2) & 15]);
    uint32_t best = 0;
#pragma unroll
    for (int k = 0; k < 16; k++) best = __vmaxu2(best, __vminu2(__vminu2(m4[k], m4[(k + 4) & 15]), a[(k + 8) & 15]));
    return (int)max(best & 0xFFFFu, best >> 16);
}

// FAST-9 segment test of the pixel at cp (row pitch rw, a shared-memory
// tile) at the threshold of K = (0x8000 - t - 1) in both 16-bit lanes: nine
// contiguous circle points brighter than v + t or darker than v - t.  Circle
// points k and k + 8 share a word; as in the compass test no borrow crosses
// the lanes and bit 15 / 31 of P + K - C is p - v > t (of C + K - P,
// v - p > t).  Equivalent to tile_arc_strength(cp, rw) > t.
__device__ __forceinline__ bool tile_is_corner(const uint8_t* cp, int rw, uint32_t K) {
    const uint32_t v = cp[0];
    const uint32_t C = v * 0x00010001u;
    const uint32_t P[8] = {(uint32_t)cp[3 * rw] | ((uint32_t)cp[-3 * rw] << 16),
                           (uint32_t)cp[3 * rw + 1] | ((uint32_t)cp[-3 * rw - 1] << 16),
                           (uint32_t)cp[2 * rw + 2] | ((uint32_t)cp[-2 * rw - 2] << 16),
                           (uint32_t)cp[rw + 3] | ((uint32_t)cp[-rw - 3] << 16),
                           (uint32_t)cp[3] | ((uint32_t)cp[-3] << 16),
                           (uint32_t)cp[-rw + 3] | ((uint32_t)cp[rw - 3] << 16),
                           (uint32_t)cp[-2 * rw + 2] | ((uint32_t)cp[2 * rw - 2] << 16),
                           (uint32_t)cp[-3 * rw + 1] | ((uint32_t)cp[3 * rw - 1] << 16)};
    uint32_t br = 0, dk = 0;  // bit k: point k (k < 8) at bit k, point k + 8 at bit 16 + k
#pragma unroll
    for (int k = 0; k < 8; k++) {
        br |= ((P[k] + K - C) & 0x80008000u) >> (15 - k);
        dk |= ((C + K - P[k]) & 0x80008000u) >> (15 - k);
    }
    br = (br & 0xFFu) | ((br >> 8) & 0xFF00u);
    dk = (dk & 0xFFu) | ((dk >> 8) & 0xFF00u);
    return has_run9(br) || has_run9(dk);
}

// The cell loop of ComputeKeyPointsOctTree (src/ORBextractor.cc:1069-1142).
// A persistent kernel: each warp takes chunks of 1, 2 or 4 consecutive
// cells of the launch (work item u = a cell of one (frame, level); two
// unless the launch has too few cells to give every warp several), the
// chunks dealt round-robin over the warps, and per cell
//   1. lane 0 copies the cell's ROI (the detection region and its 3-pixel
//      ring) into shared memory with one tensor copy (box cell_box_w x
//      (hCell + 6) from column iniX rounded down to 16), issued as soon as
//      the previous cell's scoring is done with the tile (the tensor map is
//      fenced when the level changes); meanwhile the warp clears the
//      strength window and lists the region's candidates from the strips'
//      bit map (one region row per lane, the words loaded a cell ahead, bits
//      funnel-shifted to the region's first column);
//   2. the FAST-9 segment test at the lower threshold keeps the candidates
//      that are corners (about one in eight), and the corners' arc strengths
//      (score + 1) from the tile go to the window;
//   3. suppression: FAST's per-ROI 3x3 suppression keeps pixel p at
//      threshold th when its score beats every neighbour's (a neighbour that
//      is not a corner at th, or lies outside the ROI's detection region,
//      scores 0).  On the arc strength m that is m > th' and m > m(q) for the
//      8 neighbours q (0 outside the region), with th' = max(th, 1) unless
//      the region is a single pixel: a neighbour at or below th is below m
//      already, and a pixel of score 0 (m = 1) loses to any neighbour.  The
//      neighbour test does not depend on th, so one pass over the corners
//      yields the survivors at iniThFAST and at minThFAST; the latter are
//      used when the former are none;
//   4. the survivors are written in the detector's row-major order (ranked
//      by row and column).
// CPB (warps per block, 1 / 2 / 4) is chosen by the autotuner.  A copy that
// does not arrive within the bounded wait sets status bit 128 and ends the
// warp once the copies in flight are drained.
struct FastCellGeom {
    const LevelDesc* d;
    int cell, iniX, iniY, rw, rh;
    bool ok;   // the cell is scanned
    bool bad;  // the cell exceeds the launch's shared memory (status bit 1)
};
template <int CPB>
__global__ void __launch_bounds__(32 * CPB) k_fast_cells(const LevelDesc* descs, RangeMap rm, int total, int chunk,
                                                          int* status, FastCellsSmem sm) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // per warp (sm.warp_bytes, 128-byte aligned): the ROI tile, the strength
    // window (sm.rows of ws bytes), the candidate list (sm.cand_cap keys),
    // which the minThFAST survivors overwrite from its start as the
    // suppression pass reads it, and the iniThFAST survivors (sm.min_cap keys)
    extern __shared__ __align__(128) uint8_t s_dyn[];
    __shared__ uint64_t s_bar[CPB];
    const int ws = sm.win_stride;
    const uint32_t dyn0 = smem_u32(s_dyn);
    uint8_t* const tile = s_dyn + (((dyn0 + 127u) & ~127u) - dyn0) + (size_t)warp * sm.warp_bytes;
    uint8_t* const mstr = tile + sm.tile_bytes;
    uint16_t* const cand = reinterpret_cast<uint16_t*>(mstr + sm.rows * ws);
    uint16_t* const smin = cand;
    uint16_t* const sini = cand + sm.cand_cap;
    uint64_t* const bar = &s_bar[warp];
    if (lane == 0) {
        mbar_init(bar, 1);
        mbar_init_fence();
    }
    __syncwarp();
    // work: chunks of 'chunk' (1, 2 or 4) consecutive cells (one level,
    // mostly: the tensor map is fenced once per chunk), chunk c to warp c mod
    // nw, so that the textured parts of an image spread over the warps
    const int nw = gridDim.x * CPB, gw = blockIdx.x * CPB + warp;
    auto next_cell = [&](int u) {  // the warp's cell after u
        return ((u + 1) & (chunk - 1)) != 0 ? u + 1 : u + 1 + (nw - 1) * chunk;
    };
    const int minB = ORBGPU_EDGE_THRESHOLD - 3;
    int ent = -1, ent_lo = 0, ent_hi = 0;  // the entry of the last cell: items [ent_lo, ent_hi)
    auto geom = [&](int u, FastCellGeom& G) {
        if (u < ent_lo || u >= ent_hi) {  // the last entry starting at or before u (prefix has n + 1 entries)
            int lo = ent < 0 ? 0 : ent, hi = rm.n - 1;
            if (u < ent_lo) lo = 0;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (rm.prefix[mid] <= u) lo = mid;
                else hi = mid - 1;
            }
            ent = lo;
            ent_lo = rm.prefix[lo];
            ent_hi = rm.prefix[lo + 1];
        }
        const int c = u - ent_lo;
        const LevelDesc& d = descs[rm.desc0 + ent * rm.desc_stride];
        G.d = &d;
        G.cell = c;
        const int i = c / d.nCols, j = c - i * d.nCols;
        G.iniY = minB + i * d.hCell;
        G.iniX = minB + j * d.wCell;
        int maxY = G.iniY + d.hCell + 6, maxX = G.iniX + d.wCell + 6;
        const bool skip = (G.iniY >= d.maxBorderY - 3) || (G.iniX >= d.maxBorderX - 6);
        if (maxY > d.maxBorderY) maxY = d.maxBorderY;
        if (maxX > d.maxBorderX) maxX = d.maxBorderX;
        G.rw = maxX - G.iniX;
        G.rh = maxY - G.iniY;
        const int bw = d.cell_box_w, bh = d.hCell + 6;
        G.ok = !skip && G.rw >= 7 && G.rh >= 7;
        G.bad = G.ok && (G.rw > FAST_MAX_ROI || G.rh > FAST_MAX_ROI || G.rh - 4 > sm.rows || G.rw + 2 > sm.win_stride ||
                         (G.rw - 6) * (G.rh - 6) > sm.cand_cap || bw * bh > sm.tile_bytes ||
                         (G.iniX & 15) + G.rw > bw || G.rh > bh);
        G.ok = G.ok && !G.bad;
    };
    const void* fenced = nullptr;  // lane 0: the tensor map it last acquired
    auto prefetch = [&](const FastCellGeom& G) {
        if (lane == 0 && G.ok) {
            const LevelDesc& d = *G.d;
            if (d.tm_cell != fenced) {
                tensormap_acquire(d.tm_cell);
                fenced = d.tm_cell;
            }
            mbar_expect_tx(bar, (uint32_t)(d.cell_box_w * (d.hCell + 6)));
            tma_load_2d(tile, d.tm_cell, G.iniX & ~15, G.iniY, bar);
        }
    };
    // the bit-map words of region row 'lane' of a cell (rows 32 and up are
    // read when the cell is processed: regions that high are rare); the
    // map's rows are 8-byte aligned and a row's last words run into the
    // next row, which exists (region rows end 19 rows above h)
    auto load_bits = [&](const FastCellGeom& G, uint32_t (&w)[4]) {
        w[0] = w[1] = w[2] = w[3] = 0u;
        if (G.ok && lane < G.rh - 6) {
            const LevelDesc& d = *G.d;
            const uint32_t* wr =
                reinterpret_cast<const uint32_t*>(d.cbits + (size_t)(G.iniY + 3 + lane) * d.cbits_stride) +
                ((G.iniX + 3) >> 5);
            w[0] = wr[0];
            w[1] = wr[1];
            w[2] = wr[2];
            if (G.rw - 6 > 64) w[3] = wr[3];
        }
    };
    uint32_t par = 0;  // the phase parity the tile's barrier waits for next
    FastCellGeom cur, nxt;
    uint32_t wcur[4], wnxt[4];
    const int u0 = gw * chunk;
    if (u0 < total) {
        geom(u0, cur);
        prefetch(cur);
        load_bits(cur, wcur);
    }
    for (int u = u0; u < total; u = next_cell(u)) {
        const int un = next_cell(u);
        const bool more = un < total;
        if (more) {
            geom(un, nxt);
            load_bits(nxt, wnxt);  // in flight while this cell is processed
        }
        const LevelDesc& d = *cur.d;
        const int cell = cur.cell;
        if (!cur.ok) {
            if (lane == 0) {
                d.cell_count[cell] = 0;
                if (cur.bad) atomicOr(status, 1);
            }
            if (more) prefetch(nxt);
        } else {
            const int dw = cur.rw - 6, dh = cur.rh - 6, bw = d.cell_box_w;
            const int gx0 = cur.iniX + 3, gy0 = cur.iniY + 3;  // level coordinates of region pixel (0, 0)
            // the strength window: byte b of a row <-> region column b - 4,
            // rows 0 and dh + 1 and everything outside the region stay zero
            {
                uint4* m16 = reinterpret_cast<uint4*>(mstr);
                for (int q = lane; q < (dh + 2) * (ws / 16); q += 32) m16[q] = make_uint4(0u, 0u, 0u, 0u);
            }
            // the region's candidates, one row per lane (bits of columns gx0
            // .. gx0 + dw - 1, funnel-shifted from the map's words)
            int ncand;
            {
                const int k0 = gx0 >> 5, sh = gx0 & 31;
                uint32_t m[3][3];  // [row slot][32-column group]
                int cnt = 0;
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    const int r = lane + 32 * q;
                    m[q][0] = m[q][1] = m[q][2] = 0u;
                    if (r < dh) {
                        uint32_t w0 = wcur[0], w1 = wcur[1], w2 = wcur[2], w3 = wcur[3];
                        if (q > 0) {
                            const uint32_t* wr =
                                reinterpret_cast<const uint32_t*>(d.cbits + (size_t)(gy0 + r) * d.cbits_stride) + k0;
                            w0 = wr[0];
                            w1 = wr[1];
                            w2 = wr[2];
                            w3 = dw > 64 ? wr[3] : 0u;
                        }
                        m[q][0] = __funnelshift_r(w0, w1, sh);
                        m[q][1] = __funnelshift_r(w1, w2, sh);
                        m[q][2] = __funnelshift_r(w2, w3, sh);
#pragma unroll
                        for (int g = 0; g < 3; g++) {
                            const int valid = min(max(dw - 32 * g, 0), 32);
                            if (valid < 32) m[q][g] &= (1u << valid) - 1u;
                            cnt += __popc(m[q][g]);
                        }
                    }
                }
                int incl = cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int n = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += n;
                }
                ncand = __shfl_sync(0xffffffffu, incl, 31);
                int pos = incl - cnt;
#pragma unroll
                for (int q = 0; q < 3; q++)
#pragma unroll
                    for (int g = 0; g < 3; g++)
                        for (uint32_t bits = m[q][g]; bits; bits &= bits - 1)
                            cand[pos++] = (uint16_t)(((lane + 32 * q) << 8) | (32 * g + __ffs(bits) - 1));
            }
            __syncwarp();  // the cleared window and the candidate list are the warp's
            if (!__all_sync(0xffffffffu, mbar_wait(bar, par))) {
                mbar_wait(bar, par);  // the copy gets one more bounded wait before the warp leaves
                if (lane == 0) {
                    atomicOr(status, 128);
                    d.cell_count[cell] = 0;
                }
                return;
            }
            par ^= 1u;
            // the candidates that are corners at the lower threshold, by the
            // segment test, compacted in place (a corner's slot is never
            // above its candidate's: the list is read before it is written),
            // then their arc strengths into the window
            const int tl = min(min(max(d.ini_th, 0), 255), min(max(d.min_th, 0), 255));
            const uint32_t K = (0x8000u - (uint32_t)tl - 1u) * 0x00010001u;
            const uint8_t* const org = tile + 3 * bw + (cur.iniX & 15) + 3;  // region pixel (0, 0)
            const unsigned below = (1u << lane) - 1u;
            int ncorner = 0;
            for (int q0 = 0; q0 < ncand; q0 += 32) {
                const int q = q0 + lane;
                int key = 0;
                bool corner = false;
                if (q < ncand) {
                    key = cand[q];
                    corner = tile_is_corner(org + (key >> 8) * bw + (key & 255), bw, K);
                }
                const unsigned bc = __ballot_sync(0xffffffffu, corner);
                if (corner) cand[ncorner + __popc(bc & below)] = (uint16_t)key;
                ncorner += __popc(bc);
            }
            __syncwarp();
            for (int q = lane; q < ncorner; q += 32) {
                const int key = cand[q];
                const int r = key >> 8, c = key & 255;
                mstr[(r + 1) * ws + c + 4] = (uint8_t)tile_arc_strength(org + r * bw + c, bw);
            }
            __syncwarp();  // the tile is read: the next cell's copy may land
            if (more) prefetch(nxt);
            const int single = dw * dh == 1;
            int ini_th = min(max(d.ini_th, 0), 255), min_th = min(max(d.min_th, 0), 255);
            if (!single) {
                ini_th = max(ini_th, 1);
                min_th = max(min_th, 1);
            }
            const int cell_cap = d.cell_cap;
            uint32_t* const out = d.slots + (size_t)cell * cell_cap;
            // the survivors at both thresholds, as row-major keys (row << 8 | column)
            int total_ini = 0, total_min = 0;
            {
                for (int q0 = 0; q0 < ncorner; q0 += 32) {
                    const int q = q0 + lane;
                    bool oi = false, om = false;
                    int key = 0;
                    if (q < ncorner) {
                        key = cand[q];
                        const int r = key >> 8, c = key & 255;
                        const uint8_t* p = mstr + (r + 1) * ws + c + 4;
                        const int m = p[0];
                        int nb = max(max(p[-1], p[1]), max(max(p[-ws - 1], p[-ws]), p[-ws + 1]));
                        nb = max(nb, max(max(p[ws - 1], p[ws]), p[ws + 1]));
                        if (m > nb) {
                            oi = m > ini_th;
                            om = m > min_th;
                        }
                    }
                    const unsigned bi = __ballot_sync(0xffffffffu, oi), bm = __ballot_sync(0xffffffffu, om);
                    if (oi) {
                        const int pos = total_ini + __popc(bi & below);
                        if (pos < sm.min_cap) sini[pos] = (uint16_t)key;
                    }
                    if (om) {
                        const int pos = total_min + __popc(bm & below);
                        if (pos < sm.min_cap) smin[pos] = (uint16_t)key;
                    }
                    total_ini += __popc(bi);
                    total_min += __popc(bm);
                }
            }
            __syncwarp();
            // iniThFAST's survivors if there are any, else minThFAST's, in the
            // detector's row-major order: a survivor's output row is the
            // number of smaller keys (keys are distinct)
            const bool use_ini = total_ini > 0;
            const uint16_t* L = use_ini ? sini : smin;
            const int tot = use_ini ? total_ini : total_min;
            const int n = min(tot, sm.min_cap);
            for (int q = lane; q < n; q += 32) {
                const int key = L[q];
                int rank = 0;
                for (int t = 0; t < n; t++) rank += (int)L[t] < key;
                if (rank < cell_cap) {
                    const int r = key >> 8, c = key & 255;
                    out[rank] = (uint32_t)(gx0 + c) | ((uint32_t)(gy0 + r) << 12) |
                                ((uint32_t)(mstr[(r + 1) * ws + c + 4] - 1) << 24);
                }
            }
            if (lane == 0) {
                if (tot > cell_cap || tot > sm.min_cap) atomicOr(status, 2);
                d.cell_count[cell] = min(n, cell_cap);
            }
        }
        __syncwarp();  // this cell's window and lists are read
        cur = nxt;
#pragma unroll
        for (int q = 0; q < 4; q++) wcur[q] = wnxt[q];
    }
}

// Arc strength of every interior pixel of an image (pixels closer than 3 to
// the border get 0), for the stage tests of the detector.
__global__ void k_fast_strength_map(const uint8_t* img, int pitch, int w, int h, int t, uint8_t* out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= w || y >= h) return;
    int m = 0;
    if (x >= 3 && x < w - 3 && y >= 3 && y < h - 3) m = arc_strength(img + (size_t)y * pitch, pitch, 0, x, t);
    out[(size_t)y * w + x] = (uint8_t)m;
}

// ---------------------------------------------------------------- DistributeOctTree
// List order of the reference's std::list<ExtractorNode>: after the initial
// nodes are appended, nodes are only ever pushed to the front, so the list
// is "children by creation number descending, then the initial nodes".  A
// split step therefore rebuilds the list as: the children created in this
// step in reverse creation order, followed by the nodes that were not split,
// in their previous order.  Node arrays are indexed by list position.

__device__ __forceinline__ int quadrant_of(uint32_t p, const DNode& n) {
    const float x = (float)((int)(p & 0xFFF) - (ORBGPU_EDGE_THRESHOLD - 3));
    const float y = (float)((int)((p >> 12) & 0xFFF) - (ORBGPU_EDGE_THRESHOLD - 3));
    const int halfX = (int)ceilf(__fdiv_rn((float)(n.x1 - n.x0), 2.f));
    const int halfY = (int)ceilf(__fdiv_rn((float)(n.y1 - n.y0), 2.f));
    const int xm = n.x0 + halfX, ym = n.y0 + halfY;
    if (x < (float)xm) return y < (float)ym ? 0 : 2;
    return y < (float)ym ? 1 : 3;
}

__device__ __forceinline__ DNode child_rect(const DNode& n, int q) {
    const int halfX = (int)ceilf(__fdiv_rn((float)(n.x1 - n.x0), 2.f));
    const int halfY = (int)ceilf(__fdiv_rn((float)(n.y1 - n.y0), 2.f));
    const int xm = n.x0 + halfX, ym = n.y0 + halfY;
    DNode c;
    c.x0 = (int16_t)((q & 1) ? xm : n.x0);
    c.x1 = (int16_t)((q & 1) ? n.x1 : xm);
    c.y0 = (int16_t)((q & 2) ? ym : n.y0);
    c.y1 = (int16_t)((q & 2) ? n.y1 : ym);
    return c;
}

// The working arrays of one level's DistributeOctTree: the keys (candidate,
// node, quadrant) and the nodes (two node lists, quadrant counts, child
// positions, three scratch ints, best key), each in shared memory when the
// launch's budget holds it, else in the level's global buffers.
struct DistArrays {
    uint32_t* cand;
    int* node_of;
    uint8_t* quad;
    DNode *a, *b;
    int4 *cnt4, *childpos;
    int *aux0, *aux1, *aux2;
    uint32_t* best;
};
#define DIST_KEY_BYTES 9  // per key: cand, node_of, quad
// Shared-memory offsets of the node arrays for nc nodes: a and b, then
// (16-byte aligned) cnt4 and childpos, then aux0-2 and best; the total is a
// multiple of 16.
__host__ __device__ inline size_t dist_nodes_ab(size_t nc) { return (2 * nc * sizeof(DNode) + 15) & ~(size_t)15; }
__host__ __device__ inline size_t dist_node_bytes(size_t nc) {
    return (dist_nodes_ab(nc) + 2 * nc * sizeof(int4) + 4 * nc * sizeof(int) + 15) & ~(size_t)15;
}

// Applies one split step.  split_rank[n] >= 0 is node n's rank in creation
// order (nsplit nodes split), -1 for nodes kept.  order[rank] = node.
// Returns (through smem) the new alive count and the number of children with
// more than one key.
__device__ void split_step(const LevelDesc& d, const DistArrays& m, DNode*& A, DNode*& B, int& alive, int K,
                           int nsplit, int& next_id, int& n_big, int* s_scan, int* s_vars) {
    int* split_rank = m.aux0;
    int* order = m.aux1;
    int* base = m.aux2;
    // 1. quadrant counts for keys of split nodes
    for (int n = threadIdx.x; n < alive; n += blockDim.x) m.cnt4[n] = make_int4(0, 0, 0, 0);
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const int n = m.node_of[k];
        if (split_rank[n] < 0) continue;
        const int q = quadrant_of(m.cand[k], A[n]);
        m.quad[k] = (uint8_t)q;
        atomicAdd(&((int*)&m.cnt4[n])[q], 1);
    }
    __syncthreads();
    // 2. children per split node, in creation order -> creation base
    int E = 0;
    const int U_count = alive - nsplit;
    for (int b0 = 0; b0 < nsplit; b0 += blockDim.x) {
        const int rk = b0 + threadIdx.x;
        int c = 0;
        if (rk < nsplit) {
            const int4 q = m.cnt4[order[rk]];
            c = (q.x > 0) + (q.y > 0) + (q.z > 0) + (q.w > 0);
        }
        int tot;
        const int ex = block_exclusive_scan(c, s_scan, &tot);
        if (rk < nsplit) base[rk] = E + ex;
        E += tot;
    }
    __syncthreads();
    if (E + U_count > d.node_cap) {  // node arrays too small: report and stop
        if (threadIdx.x == 0) s_vars[15] = 1;
        __syncthreads();
        n_big = 0;
        return;
    }
    // 3. unsplit nodes keep their order after the E children
    int U = 0;
    for (int b0 = 0; b0 < alive; b0 += blockDim.x) {
        const int n = b0 + threadIdx.x;
        const int u = (n < alive && split_rank[n] < 0) ? 1 : 0;
        int tot;
        const int ex = block_exclusive_scan(u, s_scan, &tot);
        if (u) {
            B[E + U + ex] = A[n];
            m.childpos[n] = make_int4(E + U + ex, 0, 0, 0);
        }
        U += tot;
    }
    // 4. children
    int big = 0;
    for (int rk = threadIdx.x; rk < nsplit; rk += blockDim.x) {
        const int n = order[rk];
        const int4 q4 = m.cnt4[n];
        const int cq[4] = {q4.x, q4.y, q4.z, q4.w};
        int pos4[4] = {-1, -1, -1, -1};
        int r = 0;
        for (int q = 0; q < 4; q++) {
            if (cq[q] == 0) continue;
            const int e = base[rk] + r++;
            const int pos = E - 1 - e;
            DNode c = child_rect(A[n], q);
            c.cnt = cq[q];
            c.id = next_id + e;
            c.flags = cq[q] == 1 ? 1 : 0;
            B[pos] = c;
            pos4[q] = pos;
            big += cq[q] > 1;
        }
        m.childpos[n] = make_int4(pos4[0], pos4[1], pos4[2], pos4[3]);
    }
    __syncthreads();
    // 5. keys follow their nodes
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const int n = m.node_of[k];
        const int4 cp = m.childpos[n];
        if (split_rank[n] < 0) m.node_of[k] = cp.x;
        else {
            const int q = m.quad[k];
            m.node_of[k] = q == 0 ? cp.x : (q == 1 ? cp.y : (q == 2 ? cp.z : cp.w));
        }
    }
    // block sum of 'big'
    int tot_big;
    block_exclusive_scan(big, s_scan, &tot_big);
    DNode* t = A;
    A = B;
    B = t;
    next_id += E;
    alive = E + U;
    n_big = tot_big;
    __syncthreads();
}

__global__ void __launch_bounds__(512) k_distribute(const LevelDesc* descs, int* status, int sort_cap,
                                                     int node_smem_cap, int key_smem_cap) {
    const LevelDesc& d = descs[blockIdx.x];
    __shared__ int s_scan[32];
    __shared__ int s_vars[16];
    __shared__ int s_root_cnt[64];
    __shared__ int s_root_pos[64];
    // dynamic: the final phase's sort keys (sort_cap), then node arrays for
    // node_smem_cap nodes (if > 0), then key arrays for key_smem_cap keys
    extern __shared__ __align__(16) unsigned long long s_sort[];
    uint8_t* sp = reinterpret_cast<uint8_t*>(s_sort + sort_cap);
    DistArrays m;
    if (node_smem_cap >= d.node_cap) {
        const size_t nc = (size_t)node_smem_cap;
        m.a = reinterpret_cast<DNode*>(sp);
        m.b = m.a + nc;
        m.cnt4 = reinterpret_cast<int4*>(sp + dist_nodes_ab(nc));
        m.childpos = m.cnt4 + nc;
        m.aux0 = reinterpret_cast<int*>(m.childpos + nc);
        m.aux1 = m.aux0 + nc;
        m.aux2 = m.aux1 + nc;
        m.best = reinterpret_cast<uint32_t*>(m.aux2 + nc);
    } else {
        m.a = (DNode*)d.nodes_a;
        m.b = (DNode*)d.nodes_b;
        m.cnt4 = d.cnt4;
        m.childpos = d.childpos;
        m.aux0 = d.aux0;
        m.aux1 = d.aux1;
        m.aux2 = d.aux2;
        m.best = d.best;
    }
    sp += dist_node_bytes((size_t)node_smem_cap);
    const int ncells = d.nCols * d.nRows;
    // 1. candidates in the reference's emission order: cell rows, cell
    //    columns, then the detector's row-major order inside each cell (the
    //    count first: it decides where the key arrays live)
    int K = 0;
    for (int b0 = 0; b0 < ncells; b0 += blockDim.x) {
        const int c = b0 + threadIdx.x;
        int tot;
        block_exclusive_scan(c < ncells ? d.cell_count[c] : 0, s_scan, &tot);
        K += tot;
    }
    if (K <= key_smem_cap) {
        m.cand = reinterpret_cast<uint32_t*>(sp);
        m.node_of = reinterpret_cast<int*>(m.cand + key_smem_cap);
        m.quad = reinterpret_cast<uint8_t*>(m.node_of + key_smem_cap);
    } else {
        m.cand = d.cand;
        m.node_of = d.node_of;
        m.quad = d.quad;
    }
    K = 0;
    for (int b0 = 0; b0 < ncells; b0 += blockDim.x) {
        const int c = b0 + threadIdx.x;
        const int cnt = c < ncells ? d.cell_count[c] : 0;
        int tot;
        const int ex = block_exclusive_scan(cnt, s_scan, &tot);
        for (int k = 0; k < cnt; k++) m.cand[K + ex + k] = d.slots[(size_t)c * d.cell_cap + k];
        K += tot;
    }
    __syncthreads();
    if (K == 0 || d.nIni <= 0) {
        if (threadIdx.x == 0) *d.kept_count = 0;
        return;
    }
    DNode* A = m.a;
    DNode* B = m.b;
    const int minB = ORBGPU_EDGE_THRESHOLD - 3;
    const int Wd = d.maxBorderX - minB, Hd = d.maxBorderY - minB;
    const int nIni = d.nIni;
    const float hX = __fdiv_rn((float)Wd, (float)nIni);
    // 2. initial nodes
    if (threadIdx.x < 64) s_root_cnt[threadIdx.x] = 0;
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const float x = (float)((int)(m.cand[k] & 0xFFF) - minB);
        int r = (int)__fdiv_rn(x, hX);
        if (r >= nIni) { atomicOr(status, 4); r = nIni - 1; }
        m.node_of[k] = r;
        atomicAdd(&s_root_cnt[r], 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int a = 0;
        for (int r = 0; r < nIni; r++) {
            s_root_pos[r] = -1;
            if (s_root_cnt[r] == 0) continue;
            DNode n;
            n.x0 = (int16_t)(int)__fmul_rn(hX, (float)r);
            n.x1 = (int16_t)(int)__fmul_rn(hX, (float)(r + 1));
            n.y0 = 0;
            n.y1 = (int16_t)Hd;
            n.cnt = s_root_cnt[r];
            n.id = r;
            n.flags = 2 | (s_root_cnt[r] == 1 ? 1 : 0);
            A[a] = n;
            s_root_pos[r] = a++;
        }
        s_vars[0] = a;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x) m.node_of[k] = s_root_pos[m.node_of[k]];
    if (threadIdx.x == 0) s_vars[15] = 0;
    int alive = s_vars[0];
    int next_id = nIni;
    const int N = d.nfeat;
    __syncthreads();
    // 3. full passes (src/ORBextractor.cc:759-904)
    bool final_phase = false;
    for (int guard = 0; guard < 64; guard++) {
        const int prev = alive;
        // every node without bNoMore splits, in list order
        int nsplit = 0;
        for (int b0 = 0; b0 < alive; b0 += blockDim.x) {
            const int n = b0 + threadIdx.x;
            const int s = (n < alive && !(A[n].flags & 1)) ? 1 : 0;
            int tot;
            const int ex = block_exclusive_scan(s, s_scan, &tot);
            if (n < alive) {
                m.aux0[n] = s ? nsplit + ex : -1;
                if (s) m.aux1[nsplit + ex] = n;
            }
            nsplit += tot;
        }
        __syncthreads();
        int n_big = 0;
        split_step(d, m, A, B, alive, K, nsplit, next_id, n_big, s_scan, s_vars);
        if (s_vars[15]) break;
        if (alive >= N || alive == prev) break;
        if (alive + n_big * 3 > N) { final_phase = true; break; }
        if (guard == 63) atomicOr(status, 8);
    }
    // 4. final phase (src/ORBextractor.cc:908-991): split the largest nodes
    //    first, ties broken by later creation first, until N is reached.
    if (final_phase) {
        for (int guard = 0; guard < 64; guard++) {
            const int prev = alive;
            // nodes with more than one key (all created by the last step)
            int nv = 0;
            for (int b0 = 0; b0 < alive; b0 += blockDim.x) {
                const int n = b0 + threadIdx.x;
                const int s = (n < alive && A[n].cnt > 1) ? 1 : 0;
                int tot;
                const int ex = block_exclusive_scan(s, s_scan, &tot);
                if (s) s_sort[nv + ex] = ((unsigned long long)A[n].cnt << 40) | ((unsigned long long)A[n].id << 16) | (unsigned long long)n;
                nv += tot;
            }
            __syncthreads();
            if (nv == 0) break;
            int np2 = 1;
            while (np2 < nv) np2 <<= 1;
            for (int k = nv + threadIdx.x; k < np2; k += blockDim.x) s_sort[k] = 0ull;
            __syncthreads();
            // bitonic sort, descending
            for (int size = 2; size <= np2; size <<= 1)
                for (int stride = size >> 1; stride > 0; stride >>= 1) {
                    for (int t = threadIdx.x; t < np2 / 2; t += blockDim.x) {
                        const int lo = 2 * t - (t & (stride - 1));
                        const int hi = lo + stride;
                        const bool desc = ((lo & size) == 0);
                        const unsigned long long a = s_sort[lo], b = s_sort[hi];
                        if ((a < b) == desc) {
                            s_sort[lo] = b;
                            s_sort[hi] = a;
                        }
                    }
                    __syncthreads();
                }
            // children count of each candidate node -> how many to split
            for (int n = threadIdx.x; n < alive; n += blockDim.x) m.cnt4[n] = make_int4(0, 0, 0, 0);
            for (int n = threadIdx.x; n < alive; n += blockDim.x) m.aux0[n] = -1;
            __syncthreads();
            for (int j = threadIdx.x; j < nv; j += blockDim.x) m.aux0[(int)(s_sort[j] & 0xFFFF)] = j;
            __syncthreads();
            for (int k = threadIdx.x; k < K; k += blockDim.x) {
                const int n = m.node_of[k];
                if (m.aux0[n] < 0) continue;
                const int q = quadrant_of(m.cand[k], A[n]);
                atomicAdd(&((int*)&m.cnt4[n])[q], 1);
            }
            __syncthreads();
            // prefix of (children - 1) in processing order; first j reaching N
            int acc = 0;
            int J = nv - 1;
            if (threadIdx.x == 0) s_vars[1] = nv - 1;
            __syncthreads();
            for (int b0 = 0; b0 < nv; b0 += blockDim.x) {
                const int j = b0 + threadIdx.x;
                int g = 0;
                if (j < nv) {
                    const int4 q = m.cnt4[(int)(s_sort[j] & 0xFFFF)];
                    g = (q.x > 0) + (q.y > 0) + (q.z > 0) + (q.w > 0) - 1;
                }
                int tot;
                const int ex = block_exclusive_scan(g, s_scan, &tot);
                if (j < nv && alive + acc + ex + g >= N) atomicMin(&s_vars[1], j);
                acc += tot;
            }
            __syncthreads();
            J = s_vars[1];
            const int nsplit = J + 1;
            for (int n = threadIdx.x; n < alive; n += blockDim.x) m.aux0[n] = -1;
            __syncthreads();
            for (int j = threadIdx.x; j < nsplit; j += blockDim.x) {
                const int n = (int)(s_sort[j] & 0xFFFF);
                m.aux0[n] = j;
                m.aux1[j] = n;
            }
            __syncthreads();
            int n_big = 0;
            split_step(d, m, A, B, alive, K, nsplit, next_id, n_big, s_scan, s_vars);
            if (s_vars[15]) break;
            if (alive >= N || alive == prev) break;
            if (guard == 63) atomicOr(status, 8);
        }
    }
    if (s_vars[15]) {
        if (threadIdx.x == 0) {
            atomicOr(status, 32);
            *d.kept_count = 0;
        }
        return;
    }
    // 5. per node the key with the largest response, first in key order
    for (int n = threadIdx.x; n < alive; n += blockDim.x) m.best[n] = 0u;
    __syncthreads();
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        const uint32_t p = m.cand[k];
        const uint32_t key = ((p >> 24) << 20) | (uint32_t)(0xFFFFF - k);
        atomicMax(&m.best[m.node_of[k]], key);
    }
    __syncthreads();
    for (int n = threadIdx.x; n < alive; n += blockDim.x) {
        const int k = 0xFFFFF - (int)(m.best[n] & 0xFFFFF);
        d.kept[n] = m.cand[k];
    }
    if (threadIdx.x == 0) *d.kept_count = alive;
}

// ---------------------------------------------------------------- describe
// The host library's value for input bits xb if the table lists xb, else v.
// The bucket of xb bounds the search to a handful of entries.
__device__ __forceinline__ float lookup_exception(const uint32_t* keys, const float* vals, const int* bucket,
                                                  const uint16_t* sub, uint32_t xb, float v) {
    const uint32_t b = xb >> ORBGPU_EXC_SHIFT;
    if (bucket == nullptr || sub == nullptr || b >= (uint32_t)g_exc_nbuckets) return v;
    constexpr uint32_t NS = 1u << ORBGPU_EXC_SUB_BITS;
    const uint32_t s = (xb >> (ORBGPU_EXC_SHIFT - ORBGPU_EXC_SUB_BITS)) & (NS - 1);
    // the four loads are independent: one round trip for the entry range
    const int base = bucket[b];
    const int lo = base + sub[b * NS + s];
    const int hi = s + 1 < NS ? base + sub[b * NS + s + 1] : bucket[b + 1];
    for (int i = lo; i < hi; i++)
        if (keys[i] == xb) return vals[i];
    return v;
}

// Orientation and descriptor of the kept keypoints, up to 32 keypoints per
// warp task (one per lane) and no block-level synchronisation after the
// prologue.  A task holds TS = 8, 16 or 32 keypoints: the smallest size whose
// tasks fit in one pass of the grid's warps (every block computes the same
// keypoint total), so a small launch spreads its keypoints over more warps
// instead of queueing 64 staging rounds on a few ('task' > 0 fixes TS).
// The task's patches are staged in shared memory by tensor copies in rounds
// of R keypoints through D buffers of the warp, each with its mbarrier; D
// rounds are in flight while one is computed:
//   pass A   the IC_Angle disc of each keypoint from the level plane
//            (DESC_LBOX_*): moments with one lane per patch column;
//   pass B   fastAtan2 and the double-precision rotation of all 32 keypoints
//            at once, one per lane (the FP64 pipe is narrow on this GPU: a
//            full warp per instruction);
//   pass C   the rBRIEF disc from the blurred plane (DESC_BBOX_*): one
//            descriptor byte per lane, two keypoints at a time, the pattern
//            read from shared memory.
// Each block scans the levels' kept counts into shared memory (descriptors
// are frame-major with levels ascending, so a level's offset inside its
// frame is a difference of two prefix entries); keypoint g of the flattened
// list finds its level by binary search.  R (1 / 2 / 4 keypoints per round)
// and D (rounds in flight, 2 / 4; WPB = 24 / (R D) warps per block) are
// chosen by the autotuner.  A copy
// that does not complete within the bounded wait sets status bit 128 and
// ends the warp once the copies in flight are drained.
static_assert(ORBGPU_EDGE_THRESHOLD >= DESC_BBOX_R && ORBGPU_EDGE_THRESHOLD >= ORBGPU_HALF_PATCH,
              "boxes start inside the plane");
static_assert(15 + 2 * ORBGPU_HALF_PATCH + 1 <= DESC_LBOX_W && 15 + DESC_BBOX_H <= DESC_BBOX_W,
              "a box covers its disc from a 16-byte aligned column");
static_assert(DESC_LBOX_W * DESC_LBOX_H <= DESC_SLOT && DESC_BBOX_W * DESC_BBOX_H <= DESC_SLOT &&
                  DESC_SLOT % 128 == 0 && DESC_LBOX_W % 16 == 0 && DESC_BBOX_W % 16 == 0,
              "box slots");
template <int R, int D, int WPB>
__global__ void __launch_bounds__(32 * WPB) k_describe(const LevelDesc* descs, int ndescs, int task,
                                                       orbgpu_keypoint* out_kps, uint8_t* out_desc, int* status) {
    extern __shared__ __align__(128) uint8_t s_dyn[];  // boxes (128-byte aligned) | s_pre[ndescs + 1]
    __shared__ int s_scan[32];
    __shared__ float2 s_pat[16][32];   // lane l's pattern point 16 l + p at [p][l]
    __shared__ uint64_t s_bar[D * WPB];  // per warp: one per buffer
    constexpr unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t dyn0 = smem_u32(s_dyn);
    uint8_t* boxes = s_dyn + (((dyn0 + 127u) & ~127u) - dyn0);
    uint8_t* wbuf = boxes + (size_t)warp * D * R * DESC_SLOT;
    int* s_pre = (int*)(boxes + (size_t)WPB * D * R * DESC_SLOT);
    uint64_t* bar = &s_bar[D * warp];
    if (lane == 0) {
#pragma unroll
        for (int b = 0; b < D; b++) mbar_init(&bar[b], 1);
        mbar_init_fence();
    }
    for (int i = threadIdx.x; i < 512; i += blockDim.x) {
        const int l = i >> 4, p = i & 15;
        s_pat[p][l] = make_float2((float)c_pattern[2 * i], (float)c_pattern[2 * i + 1]);
    }
    int base = 0;
    for (int e0 = 0; e0 < ndescs; e0 += blockDim.x) {
        const int e = e0 + threadIdx.x;
        const int v = e < ndescs ? *descs[e].kept_count : 0;
        int tot;
        const int ex = block_exclusive_scan(v, s_scan, &tot);
        if (e < ndescs) s_pre[e] = base + ex;
        base += tot;
    }
    if (threadIdx.x == 0) s_pre[ndescs] = base;
    __syncthreads();
    const int total = base;
    if (blockIdx.x == 0)
        for (int e = threadIdx.x; e < ndescs; e += blockDim.x) {
            const LevelDesc& d = descs[e];
            if (d.level == 0) *d.frame_total = s_pre[min(ndescs, e + d.nlevels)] - s_pre[e];
        }
    const int u = lane - ORBGPU_HALF_PATCH;  // patch column of this lane in pass A
    const int au = u < 0 ? -u : u;
    // rows of the disc in this lane's column: |v| <= vmax (umax is non-increasing)
    int vmax = -1;
    if (lane < 2 * ORBGPU_HALF_PATCH + 1)
        for (int v = 0; v <= ORBGPU_HALF_PATCH; v++)
            if (c_umax[v] >= au) vmax = v;
    uint32_t par = 0;  // bit b: the phase parity buffer b waits for next
    const long grid_warps = (long)gridDim.x * WPB;
    const int TS = task ? task : total <= 8 * grid_warps ? 8 : total <= 16 * grid_warps ? 16 : 32;
    const int ntasks = (total + TS - 1) / TS;
    for (int t = blockIdx.x * WPB + warp; t < ntasks; t += gridDim.x * WPB) {
        // this lane's keypoint: level, position, output row, validity
        const int g = t * TS + lane;
        int e = 0, x = 0, y = 0, score = 0, o = 0;
        bool valid = false;
        if (lane < TS && g < total) {
            int lo = 0, hi = ndescs - 1;  // last e with s_pre[e] <= g
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_pre[mid] <= g) lo = mid;
                else hi = mid - 1;
            }
            e = lo;
            const LevelDesc& d = descs[e];
            const int k = g - s_pre[e], off = s_pre[e] - s_pre[e - d.level];
            const uint32_t p = d.kept[k];
            x = (int)(p & 0xFFF);
            y = (int)((p >> 12) & 0xFFF);
            score = (int)(p >> 24);
            o = d.out_base + off + k;
            valid = true;
            if (off + k >= d.out_cap) {
                atomicOr(status, 16);
                valid = false;
            } else if (x < ORBGPU_EDGE_THRESHOLD || y < ORBGPU_EDGE_THRESHOLD || x > d.w - ORBGPU_EDGE_THRESHOLD - 1 ||
                       y > d.h - ORBGPU_EDGE_THRESHOLD - 1) {
                // keypoints lie at least EDGE_THRESHOLD pixels inside their
                // level, so both boxes lie inside the plane's rows and start
                // at a column >= 0 (EDGE_THRESHOLD >= DESC_BBOX_R)
                atomicOr(status, 64);
                valid = false;
            }
        }
        const unsigned vmask = __ballot_sync(FULL, valid);
        if (vmask == 0) continue;
        const int nv = __popc(vmask);
        const int rank = __popc(vmask & ((1u << lane) - 1u));  // among the valid lanes
        const int nr = (nv + R - 1) / R;                         // rounds
        const void* tm_l = nullptr;
        const void* tm_b = nullptr;
        if (valid) {
            tm_l = descs[e].tm_level;
            tm_b = descs[e].tm_blur;
            tensormap_acquire(tm_l);
            tensormap_acquire(tm_b);
        }
        // round i of a pass: the valid lanes of ranks [i R, i R + R) copy
        // their box into slot rank - i R of buffer i mod D
        auto issue = [&](int i, bool blurred) {
            const int b = i % D;
            if (lane == 0)
                mbar_expect_tx(&bar[b], (uint32_t)min(R, nv - i * R) *
                                            (blurred ? DESC_BBOX_W * DESC_BBOX_H : DESC_LBOX_W * DESC_LBOX_H));
            __syncwarp();
            if (valid && rank / R == i) {
                uint8_t* dst = wbuf + (b * R + rank % R) * DESC_SLOT;
                if (blurred) tma_load_2d(dst, tm_b, (x - DESC_BBOX_R) & ~15, y - DESC_BBOX_R, &bar[b]);
                else tma_load_2d(dst, tm_l, (x - ORBGPU_HALF_PATCH) & ~15, y - ORBGPU_HALF_PATCH, &bar[b]);
            }
        };
        // bounded wait for round i; on a timeout the rounds still in flight
        // (i .. i + D - 1) get one more bounded wait each before the warp leaves
        auto wait = [&](int i) -> bool {
            const int b = i % D;
            if (__all_sync(FULL, mbar_wait(&bar[b], (par >> b) & 1u))) {
                par ^= 1u << b;
                return true;
            }
            for (int j = i; j < min(nr, i + D); j++) mbar_wait(&bar[j % D], (par >> (j % D)) & 1u);
            if (lane == 0) atomicOr(status, 128);
            return false;
        };
        // pass A: IC_Angle moments (src/ORBextractor.cc:94-141) from the
        // staged discs, integer exact: per column u the sum s and the
        // row-weighted sum sv of the disc's pixels, m_10 = sum u s, m_01 = sum sv
        int my_m01 = 0, my_m10 = 0;
        for (int i = 0; i < min(nr, D); i++) issue(i, false);
        unsigned rest = vmask;
        for (int i = 0; i < nr; i++) {
            if (!wait(i)) return;
            const uint8_t* buf = wbuf + (i % D) * R * DESC_SLOT;
            for (int j = 0; j < R && rest; j++) {
                const int k = __ffs(rest) - 1;
                rest &= rest - 1;
                const int xk = __shfl_sync(FULL, x, k);
                const uint8_t* col = buf + j * DESC_SLOT + ((xk - ORBGPU_HALF_PATCH) & 15) + lane;
                int sum = 0, vsum = 0;
#pragma unroll
                for (int v = -ORBGPU_HALF_PATCH; v <= ORBGPU_HALF_PATCH; v++) {
                    if ((v < 0 ? -v : v) <= vmax) {
                        const int val = col[(v + ORBGPU_HALF_PATCH) * DESC_LBOX_W];
                        sum += val;
                        vsum += v * val;
                    }
                }
                const int m10 = __reduce_add_sync(FULL, u * sum);
                const int m01 = __reduce_add_sync(FULL, vsum);
                if (lane == k) {
                    my_m10 = m10;
                    my_m01 = m01;
                }
            }
            __syncwarp();  // buffer i mod D is read: round i + D may overwrite it
            if (i + D < nr) issue(i + D, false);
        }
        // the first D rounds of pass C travel during pass B
        for (int i = 0; i < min(nr, D); i++) issue(i, true);
        // pass B: angle and rotation, one keypoint per lane
        float angle = 0.f, ca = 0.f, sb = 0.f;
        if (valid) {
            angle = fast_atan2_deg((float)my_m01, (float)my_m10);
            // computeOrbDescriptor on the blurred level (src/ORBextractor.cc:153-204)
            const float factorPI = (float)(3.1415926535897932384626433832795 / 180.f);
            const float ar = __fmul_rn(angle, factorPI);
            double sd, cd;
            sincos_taylor(ar, &sd, &cd);
            ca = __double2float_rn(cd);
            sb = __double2float_rn(sd);
            const uint32_t xb = __float_as_uint(ar);
            if (g_cos_exc_n > 0) ca = lookup_exception(g_cos_exc_key, g_cos_exc_val, g_cos_exc_bucket, g_cos_exc_sub, xb, ca);
            if (g_sin_exc_n > 0) sb = lookup_exception(g_sin_exc_key, g_sin_exc_val, g_sin_exc_bucket, g_sin_exc_sub, xb, sb);
            const LevelDesc& d = descs[e];
            orbgpu_keypoint kp;
            const float sc = d.scale;
            kp.x = d.level == 0 ? (float)x : __fmul_rn((float)x, sc);
            kp.y = d.level == 0 ? (float)y : __fmul_rn((float)y, sc);
            kp.size = (float)(int)__fmul_rn((float)ORBGPU_PATCH_SIZE, sc);
            kp.angle = angle;
            kp.response = (float)score;
            kp.octave = d.level;
            kp.class_id = -1;
            out_kps[o] = kp;
        }
        // pass C: rBRIEF from the staged blurred discs, one descriptor byte
        // per lane, two keypoints at a time
        rest = vmask;
        for (int i = 0; i < nr; i++) {
            if (!wait(i)) return;
            const uint8_t* buf = wbuf + (i % D) * R * DESC_SLOT;
#pragma unroll
            for (int j = 0; j < R; j += 2) {
                if (!rest) break;
                const int ka = __ffs(rest) - 1;
                rest &= rest - 1;
                const int kb = (j + 1 < R && rest) ? __ffs(rest) - 1 : -1;
                if (kb >= 0) rest &= rest - 1;
                const int kb_ = kb < 0 ? ka : kb;
                const int xA = __shfl_sync(FULL, x, ka), xB = __shfl_sync(FULL, x, kb_);
                // the keypoint's pixel inside its box: row DESC_BBOX_R, column
                // DESC_BBOX_R + (x - DESC_BBOX_R) mod 16
                const uint8_t* cA =
                    buf + j * DESC_SLOT + DESC_BBOX_R * DESC_BBOX_W + DESC_BBOX_R + ((xA - DESC_BBOX_R) & 15);
                const uint8_t* cB = buf + (kb < 0 ? j : j + 1) * DESC_SLOT + DESC_BBOX_R * DESC_BBOX_W + DESC_BBOX_R +
                                    ((xB - DESC_BBOX_R) & 15);
                const float aA = __shfl_sync(FULL, ca, ka), bA = __shfl_sync(FULL, sb, ka);
                const float aB = __shfl_sync(FULL, ca, kb_), bB = __shfl_sync(FULL, sb, kb_);
                const int oA = __shfl_sync(FULL, o, ka), oB = __shfl_sync(FULL, o, kb_);
                int valA = 0, valB = 0;
#pragma unroll
                for (int kk = 0; kk < 8; kk++) {
                    int tA[2], tB[2] = {0, 0};
#pragma unroll
                    for (int q = 0; q < 2; q++) {
                        const float2 pt = s_pat[2 * kk + q][lane];
                        {
                            const int ry = cv_round(__fadd_rn(__fmul_rn(pt.x, bA), __fmul_rn(pt.y, aA)));
                            const int rx = cv_round(__fsub_rn(__fmul_rn(pt.x, aA), __fmul_rn(pt.y, bA)));
                            tA[q] = cA[ry * DESC_BBOX_W + rx];
                        }
                        if (kb >= 0) {
                            const int ry = cv_round(__fadd_rn(__fmul_rn(pt.x, bB), __fmul_rn(pt.y, aB)));
                            const int rx = cv_round(__fsub_rn(__fmul_rn(pt.x, aB), __fmul_rn(pt.y, bB)));
                            tB[q] = cB[ry * DESC_BBOX_W + rx];
                        }
                    }
                    valA |= (tA[0] < tA[1]) << kk;
                    valB |= (tB[0] < tB[1]) << kk;
                }
                out_desc[(size_t)oA * 32 + lane] = (uint8_t)valA;
                if (kb >= 0) out_desc[(size_t)oB * 32 + lane] = (uint8_t)valB;
            }
            __syncwarp();
            if (i + D < nr) issue(i + D, true);
        }
    }
}

// ---------------------------------------------------------------- host access
void upload_constants(cudaStream_t st, const int* taps, const int* umax) {
    cudaMemcpyToSymbolAsync(c_gauss_taps, taps, 7 * sizeof(int), 0, cudaMemcpyHostToDevice, st);
    cudaMemcpyToSymbolAsync(c_umax, umax, (ORBGPU_HALF_PATCH + 1) * sizeof(int), 0, cudaMemcpyHostToDevice, st);
    cudaMemcpyToSymbolAsync(c_pattern, kBriefPattern, sizeof(kBriefPattern), 0, cudaMemcpyHostToDevice, st);
}

void set_sincos_exceptions(const uint32_t* ck, const float* cv, int cn, const uint32_t* sk, const float* sv, int sn,
                           const int* cb, const int* sb, const uint16_t* csub, const uint16_t* ssub, int nbuckets) {
    cudaMemcpyToSymbol(g_cos_exc_bucket, &cb, sizeof(cb));
    cudaMemcpyToSymbol(g_sin_exc_bucket, &sb, sizeof(sb));
    cudaMemcpyToSymbol(g_cos_exc_sub, &csub, sizeof(csub));
    cudaMemcpyToSymbol(g_sin_exc_sub, &ssub, sizeof(ssub));
    cudaMemcpyToSymbol(g_exc_nbuckets, &nbuckets, sizeof(nbuckets));
    cudaMemcpyToSymbol(g_cos_exc_key, &ck, sizeof(ck));
    cudaMemcpyToSymbol(g_cos_exc_val, &cv, sizeof(cv));
    cudaMemcpyToSymbol(g_cos_exc_n, &cn, sizeof(cn));
    cudaMemcpyToSymbol(g_sin_exc_key, &sk, sizeof(sk));
    cudaMemcpyToSymbol(g_sin_exc_val, &sv, sizeof(sv));
    cudaMemcpyToSymbol(g_sin_exc_n, &sn, sizeof(sn));
}

template <int TH>
static void launch_resize_only(const LevelDesc* descs, RangeMap rm, int nitems, cudaStream_t st) {
    k_level_resize<TH><<<nitems, 32 * RS_WPB, 0, st>>>(descs, rm);
}
template <int TH>
static void launch_strip_only(const LevelDesc* descs, RangeMap rm, int nitems, cudaStream_t st) {
    k_level_strip<TH><<<nitems, 32 * RS_WPB, 0, st>>>(descs, rm);
}
void launch_level_resize(const LevelDesc* descs, RangeMap rm, int nitems, int rows, cudaStream_t st) {
    if (nitems <= 0) return;
    switch (rows) {
        case 8: launch_resize_only<8>(descs, rm, nitems, st); break;
        case 22: launch_resize_only<22>(descs, rm, nitems, st); break;
        case 64: launch_resize_only<64>(descs, rm, nitems, st); break;
        default: launch_resize_only<36>(descs, rm, nitems, st); break;
    }
}
void launch_level_strip(const LevelDesc* descs, RangeMap rm, int nitems, int rows, cudaStream_t st) {
    if (nitems <= 0) return;
    switch (rows) {
        case 8: launch_strip_only<8>(descs, rm, nitems, st); break;
        case 22: launch_strip_only<22>(descs, rm, nitems, st); break;
        case 64: launch_strip_only<64>(descs, rm, nitems, st); break;
        default: launch_strip_only<36>(descs, rm, nitems, st); break;
    }
}

// Blocks of k_level_resize / k_level_strip for a w x h level (RS_WPB strips
// of 'rows' rows per block).
int resize_blur_tiles(int w, int h, int rows) {
    const int strips = ((w + RS_COLS - 1) / RS_COLS) * ((h + rows - 1) / rows);
    return (strips + RS_WPB - 1) / RS_WPB;
}
// Strip rows of a launch whose level 0 holds 'px' pixels: the tuned value,
// or (unless the policy is off) 8 when the tuned strips of level 0 would not
// fill the device's resident warps one and a half times over (a warp walks
// its strip's rows one after the other, so a short launch is bound by that
// walk, not by the work).
int strip_rows(long px) {
    const int th = tunables().resize_rows;
    if (tunables().strip_rows_small == 0 || th <= 8) return th;
    const long strips = px / ((long)RS_COLS * th);
    const long resident = (long)nsm_of_current_device() * 12 * RS_WPB;  // k_level_strip: 12 blocks per SM
    return 2 * strips < 3 * resident ? 8 : th;
}
void launch_fast(const LevelDesc* descs, RangeMap rm, int ncells, int* status, int max_wcell, int max_hcell,
                 int max_box_bytes, cudaStream_t st) {
    if (ncells <= 0 || max_box_bytes <= 0) return;
    // shared memory for the launch's largest cell: its ROI box, its region
    // rows plus the zero ring, a candidate per region pixel and at most one
    // survivor per 2 x 2 pixels
    FastCellsSmem sm;
    sm.tile_bytes = (max_box_bytes + 127) & ~127;
    sm.rows = std::min(FAST_MAX_DET, std::max(1, max_hcell)) + 2;
    const int mw = std::min(FAST_MAX_DET, std::max(1, max_wcell)), mh = sm.rows - 2;
    sm.cand_cap = mw * mh;
    sm.min_cap = ((mw + 1) / 2) * ((mh + 1) / 2);
    sm.win_stride = (mw + 8 + 15) & ~15;
    sm.warp_bytes = (sm.tile_bytes + sm.rows * sm.win_stride + 2 * sm.cand_cap + 2 * sm.min_cap + 127) & ~127;
    const int cpb = tunables().fast_cells_per_block;
    const size_t smem = (size_t)cpb * sm.warp_bytes + 128;
    // persistent: as many blocks as fit on the device at once, each warp a
    // contiguous run of cells
    const int nsm = nsm_of_current_device();
    auto run = [&](auto kernel) {
        allow_max_dynamic_smem(kernel);
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 32 * cpb, smem) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        const int blocks = std::max(1, std::min((ncells + cpb - 1) / cpb, nsm * per_sm));
        // chunks of two cells when every warp gets several (the tensor map
        // is fenced once per chunk; on the 64-frame step two measured 2.5 %
        // faster than four), single cells when the launch is short of cells:
        // a warp's cells run one after the other
        const long warps = (long)blocks * cpb;
        const int chunk = tunables().fast_chunk ? tunables().fast_chunk : ncells >= 2 * warps ? 2 : 1;
        kernel<<<blocks, 32 * cpb, smem, st>>>(descs, rm, ncells, chunk, status, sm);
    };
    switch (cpb) {
        case 1: run(k_fast_cells<1>); break;
        case 2: run(k_fast_cells<2>); break;
        default: run(k_fast_cells<4>); break;
    }
}
void launch_distribute(const LevelDesc* descs, int ndescs, int sort_cap, int node_cap, int* status,
                       cudaStream_t st) {
    // a 72 KiB budget per block (three 512-thread blocks per SM): the sort
    // keys, the node arrays of the launch's largest level if they fit, and
    // the keys of as many candidates as the rest holds (a level with more
    // keeps them in global memory)
    const size_t budget = 72 * 1024, sort_b = (size_t)sort_cap * sizeof(unsigned long long);
    size_t node_b = dist_node_bytes((size_t)node_cap);
    int node_smem_cap = node_cap;
    if (sort_b + node_b + 16 * 1024 > budget) {
        node_b = 0;
        node_smem_cap = 0;
    }
    const int key_smem_cap = (int)(((budget > sort_b + node_b ? budget - sort_b - node_b : 0) / DIST_KEY_BYTES) & ~15);
    const size_t smem = std::max(budget, sort_b);
    allow_max_dynamic_smem(k_distribute);
    if (ndescs > 0) k_distribute<<<ndescs, 512, smem, st>>>(descs, status, sort_cap, node_smem_cap, key_smem_cap);
}
void launch_describe(const LevelDesc* descs, int ndescs, int max_kept, orbgpu_keypoint* kps, uint8_t* desc, int* status,
                     cudaStream_t st) {
    if (ndescs <= 0 || max_kept <= 0) return;
    const int nsm = nsm_of_current_device();
    const int R = tunables().describe_group, D = R * tunables().describe_depth > 8 ? 2 : tunables().describe_depth;
    // D buffers of R box slots per warp, 24 slots (60 KiB) per block: three
    // blocks per SM.  max_kept (the node capacity) overestimates a level's
    // keypoints about twice; a grid of 32-keypoint tasks' worth of warps, or
    // for a launch that would not fill the SMs that way, 8-keypoint tasks'
    // worth on up to one block per SM (the kernel picks the task size from
    // the grid and the keypoint count); warps stride over the tasks
    const int wpb = 24 / (R * D);
    const size_t smem = (size_t)D * R * wpb * DESC_SLOT + 128 + sizeof(int) * (ndescs + 1);
    const long est = (long)ndescs * max_kept / 2;
    long want = (est + 32 * wpb - 1) / (32 * wpb);
    if (want < nsm) want = std::min((long)nsm, (est + 8 * wpb - 1) / (8 * wpb));
    const int blocks = (int)std::max(1L, std::min(want, (long)nsm * 3));
    auto run = [&](auto kernel) {
        allow_max_dynamic_smem(kernel);
        kernel<<<blocks, 32 * wpb, smem, st>>>(descs, ndescs, tunables().describe_task, kps, desc, status);
    };
    switch (R * 8 + D) {
        case 1 * 8 + 2: run(k_describe<1, 2, 12>); break;
        case 1 * 8 + 4: run(k_describe<1, 4, 6>); break;
        case 2 * 8 + 4: run(k_describe<2, 4, 3>); break;
        case 4 * 8 + 2: run(k_describe<4, 2, 3>); break;
        default: run(k_describe<2, 2, 6>); break;
    }
}

}  // namespace orbgpu

namespace orbgpu {
// The descriptor rotation exactly as k_describe evaluates it (Taylor value
// corrected by the exception table), for the rotation tests.
__global__ void k_sincos_probe(const float* x, int n, float* c, float* s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double sd, cd;
    sincos_taylor(x[i], &sd, &cd);
    float a = __double2float_rn(cd), b = __double2float_rn(sd);
    const uint32_t xb = __float_as_uint(x[i]);
    if (g_cos_exc_n > 0) a = lookup_exception(g_cos_exc_key, g_cos_exc_val, g_cos_exc_bucket, g_cos_exc_sub, xb, a);
    if (g_sin_exc_n > 0) b = lookup_exception(g_sin_exc_key, g_sin_exc_val, g_sin_exc_bucket, g_sin_exc_sub, xb, b);
    c[i] = a;
    s[i] = b;
}
}  // namespace orbgpu

// Device arrays x (n floats) -> the descriptor rotation's cos and sin.
extern "C" int orbgpu_descriptor_sincos(const float* x, int n, float* c, float* s) {
    int rc = orbgpu::ensure_sincos_exceptions();
    if (rc != ORBGPU_OK) return rc;
    if (n <= 0) return ORBGPU_OK;
    orbgpu::k_sincos_probe<<<(n + 255) / 256, 256>>>(x, n, c, s);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    ORBGPU_CUDA_TRY(cudaDeviceSynchronize());
    return ORBGPU_OK;
}

// Device image (pitch bytes per row) -> w*h arc strengths at threshold t.
extern "C" int orbgpu_debug_fast_strength(const uint8_t* img, int pitch, int w, int h, int t, uint8_t* out) {
    dim3 grid((w + 127) / 128, h);
    orbgpu::k_fast_strength_map<<<grid, 128>>>(img, pitch, w, h, t, out);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    ORBGPU_CUDA_TRY(cudaDeviceSynchronize());
    return ORBGPU_OK;
}

