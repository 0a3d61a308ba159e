// orbgpu_mappoint.cu -- MapPoint::ComputeDistinctiveDescriptors for many map
// points in one launch.
//
// The reference (src/MapPoint.cc:365-447) gathers the descriptors of the
// keyframes observing a map point (bad keyframes skipped), fills the N x N
// table of DescriptorDistance values, sorts every row, takes element
// (size_t)(0.5 * (N - 1)) as that descriptor's median distance to the others
// (itself included, at distance 0) and keeps the first descriptor with the
// least median.  Here the lists arrive as CSR: obs_offsets[m + 1] into
// obs_rows, each entry a row of a descriptor pool (the keyframes' descriptor
// matrices, resident in HBM), -1 for an observation of a bad keyframe.
//
// One warp takes 4 consecutive map points.  A map point with at most 8, 16 or
// 32 observations goes to a lane group of that width (4, 2 or 1 map points per
// pass), each lane holding one observation's descriptor; the group's
// descriptors sit in shared memory.  In groups of 8 and 16 every lane computes
// the distances to the next G/2 lanes of its group (cyclically) and receives
// the other half from the lanes before it (distances are symmetric), then
// sorts its row with a bitonic network and reads element k.  In a group of 32
// every lane computes its whole row (up to the list length, in chunks of 8)
// as 16-bit pairs and finds element k by binary lifting over the distance
// range 0..256.  The
// group's minimum of (median, lane) is the reference's first least median.
// Longer lists (more than 32 observations) run one map point per warp: rows
// in chunks of 32 lanes, each row's median from two histogram passes (d >> 4,
// then d & 15 inside the coarse bin) in lane-private shared-memory columns.
#include <algorithm>

#include "orbgpu_host.h"

namespace orbgpu {

#define DD_WARPS 8          // warps per block
#define DD_MPW 4            // map points a warp takes per iteration
#ifndef DD_BLOCKS_PER_SM
#define DD_BLOCKS_PER_SM 4  // resident blocks per SM (64 registers x 256 threads)
#endif

struct DDArgs {
    const uint4* pool;  // pool_rows x 32 bytes
    int pool_rows;
    const int* offsets;  // m + 1
    const int* rows;     // n_obs
    int n_obs;
    int m;
    int* best;   // m
    uint4* out;  // m x 32 bytes, or null
};

struct DDShared {
    uint4 desc[DD_WARPS][2][32];  // one warp's staged descriptors (low, high halves)
    int hist[DD_WARPS][17][32];   // lane-private histogram columns (long lists)
};

#define DD_FULL 0xffffffffu

// Element k of a row of 32 distances held as 16-bit pairs (p[i] = d[2i] |
// d[2i+1] << 16): the smallest v in 0..256 with #{j : d[j] <= v} > k, by
// binary lifting.  Per pair, (0x8000 + v) - d stays within its half (d <= 512,
// v <= 511) and has bit 15 set exactly when d <= v; dp2a adds the two flags.
// Entries of absent or skipped observations hold 512 and never count; the
// pairs of chunks past jmax are all such entries.
__device__ __forceinline__ int dd_row_rank32(const unsigned (&p)[16], int k, int jmax) {
    int lo = 0;
#pragma unroll 1
    for (int step = 256; step >= 1; step >>= 1) {
        const int v = lo + step - 1;
        const unsigned v2 = (unsigned)(0x8000 + v) * 0x10001u;
        unsigned acc = 0;
#pragma unroll
        for (int ic = 0; ic < 16; ic += 4) {
            if (2 * ic >= jmax) break;
#pragma unroll
            for (int i = ic; i < ic + 4; i++) acc = __dp2a_lo((v2 - p[i]) & 0x80008000u, 0x0101u, acc);
        }
        if ((int)(acc >> 15) <= k) lo += step;
    }
    return lo;
}

// Ascending bitonic sorting network over G registers.
template <int G>
__device__ __forceinline__ void dd_sort(int (&d)[G]) {
#pragma unroll
    for (int k = 2; k <= G; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
#pragma unroll
            for (int i = 0; i < G; i++) {
                const int l = i ^ j;
                if (l > i) {
                    const int lo = min(d[i], d[l]), hi = max(d[i], d[l]);
                    d[i] = (i & k) == 0 ? lo : hi;
                    d[l] = (i & k) == 0 ? hi : lo;
                }
            }
        }
    }
}

__device__ __forceinline__ void dd_store(const DDArgs& a, int mp, int row, uint4 d0, uint4 d1) {
    a.best[mp] = row;
    if (a.out) {
        a.out[2 * (size_t)mp] = d0;
        a.out[2 * (size_t)mp + 1] = d1;
    }
}

// The map points of 'mask' (bit g = map point base + g, every list 1..G long)
// in lane groups of width G.  off: lane g (g <= 4) holds obs_offsets[base + g].
template <int G>
__device__ __forceinline__ void dd_group_pass(const DDArgs& a, uint4 (*sd)[32], int lane, int base, int off, unsigned mask) {
    constexpr int NG = 32 / G;
    const int grp = lane / G, l = lane % G;
    const unsigned gmask = G == 32 ? DD_FULL : ((1u << G) - 1u);
    while (mask) {
        // group k takes the k-th map point left in the mask
        int g = -1;
        unsigned mm = mask;
#pragma unroll
        for (int k = 0; k < NG; k++) {
            if (k == grp && mm) g = __ffs(mm) - 1;
            if (mm) mm &= mm - 1;
        }
        mask = mm;
        const int gs = g < 0 ? 0 : g;
        const int o0 = __shfl_sync(DD_FULL, off, gs);
        const int o1 = __shfl_sync(DD_FULL, off, gs + 1);
        const int n = g < 0 ? 0 : o1 - o0;
        int r = -1;
        if (l < n) r = __ldg(a.rows + o0 + l);
        const bool valid = r >= 0 && r < a.pool_rows;
        const bool bad = l < n && (r < -1 || r >= a.pool_rows);
        const unsigned gv = (__ballot_sync(DD_FULL, valid) >> (grp * G)) & gmask;
        const bool gbad = ((__ballot_sync(DD_FULL, bad) >> (grp * G)) & gmask) != 0;
        uint4 d0 = make_uint4(0, 0, 0, 0), d1 = d0;
        if (valid) {
            d0 = __ldg(a.pool + 2 * (size_t)r);
            d1 = __ldg(a.pool + 2 * (size_t)r + 1);
        }
        __syncwarp();
        sd[0][lane] = d0;
        sd[1][lane] = d1;
        __syncwarp();
        const int nv = __popc(gv);
        const int k = (nv - 1) >> 1;
        int median;
        if constexpr (G < 32) {
            // d(l, l + s) for s = 1..G/2 here, d(l, l - s) from lane l - s
            int h[G / 2];
#pragma unroll
            for (int s = 1; s <= G / 2; s++) {
                const int j = grp * G + ((l + s) & (G - 1));
                h[s - 1] = hamming256(d0, d1, sd[0][j], sd[1][j]);
            }
            int d[G];
            d[0] = 0;
#pragma unroll
            for (int s = 1; s <= G / 2; s++) d[s] = (gv >> ((l + s) & (G - 1))) & 1u ? h[s - 1] : 512;
#pragma unroll
            for (int s = 1; s < G / 2; s++) {
                const int v = __shfl_sync(DD_FULL, h[s - 1], (l - s) & (G - 1), G);
                d[G / 2 + s] = (gv >> ((l - s) & (G - 1))) & 1u ? v : 512;
            }
            dd_sort<G>(d);
            median = d[0];
#pragma unroll
            for (int i = 1; i < G / 2; i++) median = i == k ? d[i] : median;
        } else {
            const int jmax = __reduce_max_sync(DD_FULL, n);
            unsigned p[16];
#pragma unroll
            for (int jc = 0; jc < 32; jc += 8) {
#pragma unroll
                for (int i = jc / 2; i < jc / 2 + 4; i++) p[i] = 512u * 0x10001u;
                if (jc < jmax) {
#pragma unroll
                    for (int j = jc; j < jc + 8; j += 2) {
                        const int h0 = hamming256(d0, d1, sd[0][j], sd[1][j]);
                        const int h1 = hamming256(d0, d1, sd[0][j + 1], sd[1][j + 1]);
                        const unsigned e0 = (gv >> j) & 1u ? (unsigned)h0 : 512u;
                        const unsigned e1 = (gv >> (j + 1)) & 1u ? (unsigned)h1 : 512u;
                        p[j / 2] = e0 | (e1 << 16);
                    }
                }
            }
            median = dd_row_rank32(p, k, jmax);
        }
        int key = valid ? (median << 5) | l : 0x7fffffff;
#pragma unroll
        for (int s = G / 2; s >= 1; s >>= 1) key = min(key, __shfl_xor_sync(DD_FULL, key, s));
        if (g >= 0) {
            const int mp = base + g;
            if (gbad) {
                if (l == 0) a.best[mp] = -2;
            } else if (nv == 0) {
                if (l == 0) a.best[mp] = -1;
            } else if (l == (key & 31)) {
                dd_store(a, mp, r, d0, d1);
            }
        }
    }
}

// One map point with more than 32 observations, the whole warp.
__device__ __forceinline__ void dd_long_list(const DDArgs& a, uint4 (*sd)[32], int (*hist)[32], int lane, int mp, int o0, int n) {
    int nv = 0;
    bool bad = false;
    for (int c = 0; c < n; c += 32) {
        const bool in = c + lane < n;
        const int r = in ? __ldg(a.rows + o0 + c + lane) : -1;
        nv += __popc(__ballot_sync(DD_FULL, r >= 0 && r < a.pool_rows));
        bad |= __ballot_sync(DD_FULL, in && (r < -1 || r >= a.pool_rows)) != 0;
    }
    if (bad || nv == 0) {
        if (lane == 0) a.best[mp] = bad ? -2 : -1;
        return;
    }
    const int k = (nv - 1) >> 1;
    const uint4 z = make_uint4(0, 0, 0, 0);
    unsigned long long best = ~0ull;
    for (int rc = 0; rc < n; rc += 32) {
        const int i = rc + lane;
        const int ri = i < n ? __ldg(a.rows + o0 + i) : -1;
        const bool vi = ri >= 0;
        uint4 m0 = z, m1 = z;
        if (vi) {
            m0 = __ldg(a.pool + 2 * (size_t)ri);
            m1 = __ldg(a.pool + 2 * (size_t)ri + 1);
        }
        int coarse = 0, below = 0, median = 0;
        for (int pass = 0; pass < 2; pass++) {
#pragma unroll
            for (int b = 0; b < 17; b++) hist[b][lane] = 0;
            for (int jc = 0; jc < n; jc += 32) {
                const int rj = jc + lane < n ? __ldg(a.rows + o0 + jc + lane) : -1;
                const unsigned vj = __ballot_sync(DD_FULL, rj >= 0);
                uint4 b0 = z, b1 = z;
                if (rj >= 0) {
                    b0 = __ldg(a.pool + 2 * (size_t)rj);
                    b1 = __ldg(a.pool + 2 * (size_t)rj + 1);
                }
                __syncwarp();
                sd[0][lane] = b0;
                sd[1][lane] = b1;
                __syncwarp();
                if (vi) {
                    unsigned todo = vj;
                    while (todo) {
                        const int jj = __ffs(todo) - 1;
                        todo &= todo - 1;
                        const int d = hamming256(m0, m1, sd[0][jj], sd[1][jj]);
                        if (pass == 0) hist[d >> 4][lane]++;
                        else if ((d >> 4) == coarse) hist[d & 15][lane]++;
                    }
                }
            }
            if (vi) {
                // element k lies in the first bin where the running count passes k
                int cum = pass == 0 ? 0 : below;
                const int nb = pass == 0 ? 17 : 16;
                for (int b = 0; b < nb; b++) {
                    const int c = hist[b][lane];
                    if (cum + c > k) {
                        if (pass == 0) {
                            coarse = b;
                            below = cum;
                        } else {
                            median = coarse * 16 + b;
                        }
                        break;
                    }
                    cum += c;
                }
            }
        }
        if (vi) {
            const unsigned long long key = ((unsigned long long)median << 32) | (unsigned)i;
            best = key < best ? key : best;
        }
    }
    best = warp_min_u64(best);
    if (lane == 0) {
        const int r = __ldg(a.rows + o0 + (int)(best & 0xffffffffu));
        dd_store(a, mp, r, __ldg(a.pool + 2 * (size_t)r), __ldg(a.pool + 2 * (size_t)r + 1));
    }
}

__global__ void __launch_bounds__(DD_WARPS * 32, DD_BLOCKS_PER_SM) k_distinctive_descriptors(const __grid_constant__ DDArgs a) {
    __shared__ DDShared sh;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int stride = gridDim.x * DD_WARPS * DD_MPW;
    for (int base = (blockIdx.x * DD_WARPS + w) * DD_MPW; base < a.m; base += stride) {
        int off = 0;
        if (lane <= DD_MPW && base + lane <= a.m) off = __ldg(a.offsets + base + lane);
        unsigned c8 = 0, c16 = 0, c32 = 0, clong = 0;
#pragma unroll
        for (int g = 0; g < DD_MPW; g++) {
            const int o0 = __shfl_sync(DD_FULL, off, g), o1 = __shfl_sync(DD_FULL, off, g + 1);
            if (base + g >= a.m) continue;
            const int n = o1 - o0;
            if (o0 < 0 || n < 0 || o1 > a.n_obs) {
                if (lane == 0) a.best[base + g] = -2;
            } else if (n == 0) {
                if (lane == 0) a.best[base + g] = -1;
            } else if (n <= 8) {
                c8 |= 1u << g;
            } else if (n <= 16) {
                c16 |= 1u << g;
            } else if (n <= 32) {
                c32 |= 1u << g;
            } else {
                clong |= 1u << g;
            }
        }
        if (c8) dd_group_pass<8>(a, sh.desc[w], lane, base, off, c8);
        if (c16) dd_group_pass<16>(a, sh.desc[w], lane, base, off, c16);
        if (c32) dd_group_pass<32>(a, sh.desc[w], lane, base, off, c32);
        while (clong) {
            const int g = __ffs(clong) - 1;
            clong &= clong - 1;
            const int o0 = __shfl_sync(DD_FULL, off, g), o1 = __shfl_sync(DD_FULL, off, g + 1);
            dd_long_list(a, sh.desc[w], sh.hist[w], lane, base + g, o0, o1 - o0);
        }
    }
}

}  // namespace orbgpu

using namespace orbgpu;

extern "C" int orbgpu_distinctive_descriptors(const uint8_t* pool, int pool_rows, const int* obs_offsets,
                                              const int* obs_rows, int n_obs, int m, int* best_rows,
                                              uint8_t* descriptors, void* stream) {
    if (m < 0 || pool_rows < 0 || n_obs < 0 || (m > 0 && (!obs_offsets || !best_rows)) ||
        (pool_rows > 0 && !pool) || (n_obs > 0 && !obs_rows)) {
        orbgpu_set_last_error("orbgpu_distinctive_descriptors: negative size or missing array", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (((uintptr_t)pool & 15) || ((uintptr_t)descriptors & 15)) {
        orbgpu_set_last_error("orbgpu_distinctive_descriptors: pool and descriptors must be 16-byte aligned", __FILE__,
                              __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (m == 0) return ORBGPU_OK;
    DDArgs a;
    a.pool = reinterpret_cast<const uint4*>(pool);
    a.pool_rows = pool_rows;
    a.offsets = obs_offsets;
    a.rows = obs_rows;
    a.n_obs = n_obs;
    a.m = m;
    a.best = best_rows;
    a.out = reinterpret_cast<uint4*>(descriptors);
    const long long per_block = DD_WARPS * DD_MPW;
    const long long want = (m + per_block - 1) / per_block;
    const int blocks = (int)std::min<long long>(want, (long long)nsm_of_current_device() * DD_BLOCKS_PER_SM);
    k_distinctive_descriptors<<<blocks, DD_WARPS * 32, 0, (cudaStream_t)stream>>>(a);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    return ORBGPU_OK;
}
