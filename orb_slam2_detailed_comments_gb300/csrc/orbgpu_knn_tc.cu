// orbgpu_knn_tc.cu -- brute-force k = 2 Hamming kNN on the 5th-generation
// tensor cores (tcgen05).
//
// Each 256-bit descriptor is expanded to 256 FP8 (E4M3) values, +1 for a 0
// bit and -1 for a 1 bit.  For two descriptors the dot product of their
// expansions is 256 - 2 * Hamming, exact in the FP32 accumulator, so
//     Hamming = (256 - dot) / 2.
// The expansions are written in the tensor cores' shared-memory operand
// layout (K-major, no swizzle: 8-row x 16-byte core matrices, 128 bytes
// each, the 16 core matrices of one 8-row group back to back), so a 128-row
// query tile (32 KiB) and a 256-row train tile (64 KiB) are single
// contiguous bulk copies.
//
// One CTA owns 128 queries and a slice of the train rows.  Per train tile:
// one elected thread issues 8 MMAs (M=128, N=256, K=32) into a TMEM
// accumulator (128 lanes x 256 FP32 columns, double-buffered), commits them
// to an mbarrier, and the 16 epilogue warps (4 per TMEM lane quadrant, 64
// columns each) read the accumulator with tcgen05.ld and keep a per-thread
// (distance, index) top-2; train tiles are double-buffered in shared memory.
// All waits are bounded: on timeout the CTA records an error flag, drains,
// frees its TMEM and returns.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "orbgpu_async.cuh"
#include "orbgpu_host.h"

cudaStream_t orbgpu_matcher_stream_internal(orbgpu_matcher* m);
void knn_merge_launch(const int4* partial, int nq, int nslices, int* idx1, int* d1, int* idx2, int* d2,
                      cudaStream_t st);

namespace orbgpu {

#define TC_M 128
#define TC_N 256
#define TC_K 256                      // bytes (= FP8 elements) per row
#define TC_QTILE_BYTES (TC_M * TC_K)  // 32 KiB
#define TC_TTILE_BYTES (TC_N * TC_K)  // 64 KiB
#define TC_EPI_WARPS 16
#define TC_THREADS (32 * (TC_EPI_WARPS + 2))  // + producer warp + MMA warp

// ---------------------------------------------------------------- operand layout
// Byte offset of element (row r, k) inside a tile stored K-major without
// swizzle: core matrix (r / 8, k / 16) is 128 contiguous bytes (8 rows of 16
// bytes); the 16 core matrices along K of one 8-row group are consecutive
// (leading-dimension stride 128 B), 8-row groups are 2048 B apart (stride
// dimension).
__host__ __device__ __forceinline__ uint32_t tc_offset(int r, int k) {
    return (uint32_t)((r >> 3) * 2048 + (k >> 4) * 128 + (r & 7) * 16 + (k & 15));
}

// Expands n descriptors (32 bytes) into tiled FP8 +-1 rows; rows past n are
// +1 everywhere (their distances are discarded by the index bound).  One
// thread per 16 bits: the 16 FP8 values of one core-matrix row, one 16-byte
// store.
__global__ void k_expand_fp8(const uint8_t* __restrict__ desc, int n, int tile_rows, uint8_t* __restrict__ out) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int row = (int)(t >> 4), c = (int)(t & 15);  // bits 16c .. 16c + 15 of the row
    const int tile = row / tile_rows, r = row - tile * tile_rows;
    uint32_t bits = 0;
    if (row < n) bits = (uint32_t)desc[(size_t)row * 32 + 2 * c] | ((uint32_t)desc[(size_t)row * 32 + 2 * c + 1] << 8);
    uint32_t w[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        uint32_t v = 0;
#pragma unroll
        for (int b = 0; b < 4; b++) v |= (((bits >> (4 * q + b)) & 1u) ? 0xB8u : 0x38u) << (8 * b);  // 1 bit -> -1.0
        w[q] = v;
    }
    *reinterpret_cast<uint4*>(out + (size_t)tile * tile_rows * TC_K + tc_offset(r, 16 * c)) = make_uint4(w[0], w[1], w[2], w[3]);
}

// ---------------------------------------------------------------- PTX wrappers
// K-major, no swizzle shared-memory operand descriptor.
__device__ __forceinline__ uint64_t smem_desc(const void* base, uint32_t lbo, uint32_t sbo) {
    const uint64_t a = (uint64_t)((smem_u32(base) >> 4) & 0x3FFF);
    return a | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f8f6f4: D = FP32, A = B = E4M3, both K-major.
__host__ __device__ __forceinline__ uint32_t idesc_e4m3(int M, int N) {
    return (1u << 4)                   // D format F32
           | (0u << 7) | (0u << 10)    // A, B format E4M3
           | ((uint32_t)(N >> 3) << 17)
           | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, int accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive 32-bit columns of this warp's 32 TMEM lanes, without the
// wait (the caller issues tcgen05.wait::ld before reading r).
__device__ __forceinline__ void tc_ld32_raw(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
        "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}

// 32 consecutive FP32 columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
        "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------- probe
// One MMA group of a 128 x 256 tile over K = 256: D[i][j] = sum_k A[i][k] B[j][k]
// written to out (128 x 256 floats), for the layout self-test.
__global__ void __launch_bounds__(128) k_tc_probe(const uint8_t* qa, const uint8_t* tb, float* out, int* status, uint32_t lbo,
                                                  uint32_t sbo) {
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    uint8_t* sA = tc_smem;
    uint8_t* sB = tc_smem + TC_QTILE_BYTES;
    __shared__ __align__(8) uint64_t bar_load, bar_mma;
    __shared__ uint32_t tmem_base;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        mbar_init(&bar_load, 1);
        mbar_init(&bar_mma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(&tmem_base)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    bool ok = true;
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar_load, TC_QTILE_BYTES + TC_TTILE_BYTES);
        bulk_g2s(sA, qa, TC_QTILE_BYTES, &bar_load);
        bulk_g2s(sB, tb, TC_TTILE_BYTES, &bar_load);
        ok = mbar_wait(&bar_load, 0);
        if (ok) {
            tc_fence_after();
            const uint32_t idesc = idesc_e4m3(TC_M, TC_N);
            for (int ks = 0; ks < TC_K / 32; ks++) {
                const uint64_t ad = smem_desc(sA + ks * 256, lbo, sbo);
                const uint64_t bd = smem_desc(sB + ks * 256, lbo, sbo);
                tc_mma(tmem, ad, bd, idesc, ks > 0);
            }
            tc_commit(&bar_mma);
        }
        if (!ok) {
            atomicOr(status, 1);
            mbar_wait(&bar_load, 0);  // give the copies in flight one more bounded wait
        }
    }
    __syncthreads();
    if (!(*status & 1)) {
        const bool done = mbar_wait(&bar_mma, 0);
        if (!done && lane == 0) atomicOr(status, 2);
        tc_fence_after();
        if (done) {
            const int row = warp * 32 + lane;
            for (int c = 0; c < TC_N; c += 32) {
                float v[32];
                tc_ld32(tmem + ((uint32_t)(warp * 32) << 16) + c, v);
                for (int i = 0; i < 32; i++) out[(size_t)row * TC_N + c + i] = v[i];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
}

// ---------------------------------------------------------------- kNN kernel
// qa: query tiles (ceil(nq/128) tiles of 32 KiB), tb: train tiles (ceil(nt/256)
// of 64 KiB).  Grid: (query tiles, slices); each CTA scans train tiles
// [tile0, tile1) of its slice and writes its per-query (best, second) pair.
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_knn_tc(const uint8_t* __restrict__ qa, const uint8_t* __restrict__ tb, int nq, int nt, int tiles_per_slice,
             int4* __restrict__ partial, int* status) {
    extern __shared__ __align__(1024) uint8_t tc_smem[];
    uint8_t* sA = tc_smem;
    uint8_t* sB0 = tc_smem + TC_QTILE_BYTES;
    __shared__ __align__(8) uint64_t bar_a, bar_full[2], bar_empty[2], bar_acc[2], bar_acc_free[2];
    __shared__ uint32_t tmem_base;
    __shared__ int s_abort;
    __shared__ int4 s_part[TC_EPI_WARPS / 4][TC_M];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int qtile = blockIdx.x;
    const int ntiles_t = (nt + TC_N - 1) / TC_N;
    const int t0 = blockIdx.y * tiles_per_slice, t1 = min(ntiles_t, t0 + tiles_per_slice);
    const int producer = TC_EPI_WARPS, issuer = TC_EPI_WARPS + 1;
    if (threadIdx.x == 0) {
        mbar_init(&bar_a, 1);
        for (int i = 0; i < 2; i++) {
            mbar_init(&bar_full[i], 1);
            mbar_init(&bar_empty[i], 1);
            mbar_init(&bar_acc[i], 1);
            mbar_init(&bar_acc_free[i], TC_EPI_WARPS * 32);
        }
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == issuer) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_base)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    const int ntile = max(0, t1 - t0);
    if (warp == producer) {
        if (lane == 0) {
            int issued = 0;
            mbar_expect_tx(&bar_a, TC_QTILE_BYTES);
            bulk_g2s(sA, qa + (size_t)qtile * TC_QTILE_BYTES, TC_QTILE_BYTES, &bar_a);
            for (int i = 0; i < ntile; i++) {
                const int s = i & 1;
                if (i >= 2 && !mbar_wait(&bar_empty[s], ((i >> 1) - 1) & 1)) {
                    atomicOr(status, 4);
                    s_abort = 1;
                    break;
                }
                mbar_expect_tx(&bar_full[s], TC_TTILE_BYTES);
                bulk_g2s(sB0 + s * TC_TTILE_BYTES, tb + (size_t)(t0 + i) * TC_TTILE_BYTES, TC_TTILE_BYTES, &bar_full[s]);
                issued = i + 1;
            }
            // no copy may still be writing shared memory when the CTA ends:
            // wait (bounded) for the last phase issued on every barrier
            bool drained = mbar_wait(&bar_a, 0);
            for (int i = max(0, issued - 2); i < issued; i++) drained &= mbar_wait(&bar_full[i & 1], (i >> 1) & 1);
            if (!drained) atomicOr(status, 32);
        }
    } else if (warp == issuer) {
        if (lane == 0) {
            const uint32_t idesc = idesc_e4m3(TC_M, TC_N);
            bool ok = mbar_wait(&bar_a, 0);
            int issued = 0;
            for (int i = 0; ok && i < ntile; i++) {
                const int s = i & 1;
                ok = mbar_wait(&bar_full[s], (i >> 1) & 1);
                // accumulator buffer s is free once the epilogue drained tile i-2
                if (ok && i >= 2) ok = mbar_wait(&bar_acc_free[s], ((i >> 1) - 1) & 1);
                if (!ok) break;
                tc_fence_after();
                const uint8_t* sB = sB0 + s * TC_TTILE_BYTES;
                const uint32_t d = tmem + (uint32_t)(s * TC_N);
                for (int ks = 0; ks < TC_K / 32; ks++)
                    tc_mma(d, smem_desc(sA + ks * 256, 128, 2048), smem_desc(sB + ks * 256, 128, 2048), idesc, ks > 0);
                tc_commit(&bar_empty[s]);  // train buffer s reusable when these MMAs are done
                tc_commit(&bar_acc[s]);    // accumulator s ready
                issued = i + 1;
            }
            if (!ok) {
                atomicOr(status, 8);
                s_abort = 1;
            }
            // TMEM is freed below: wait (bounded) until the last MMAs issued on
            // both accumulators have completed
            bool drained = true;
            for (int i = max(0, issued - 2); i < issued; i++) drained &= mbar_wait(&bar_acc[i & 1], (i >> 1) & 1);
            if (!drained) atomicOr(status, 64);
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32*(w%4).. and columns 64*(w/4)..
        // Keys pack (distance << 23 | train index), so the lexicographic
        // (distance, index) top-2 is three min/max operations per value.  The
        // dot products are exact integers in [-256, 256]: adding 1.5 * 2^23
        // puts them in the low mantissa bits, and 256 - dot = 2 * Hamming.
        const int quad = warp & 3, part = warp >> 2;
        const int row = quad * 32 + lane;
        uint32_t k1 = 0xFFFFFFFFu, k2 = 0xFFFFFFFFu;
        for (int i = 0; i < ntile; i++) {
            const int s = i & 1;
            // warp-uniform outcome: tcgen05.ld below is a whole-warp instruction
            if (!__all_sync(0xffffffffu, mbar_wait(&bar_acc[s], (i >> 1) & 1))) {
                if (lane == 0) atomicOr(status, 16);
                s_abort = 1;
                break;
            }
            tc_fence_after();
            const int jbase = (t0 + i) * TC_N + part * 64;
            uint32_t r[64];
            const uint32_t ta = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(s * TC_N + part * 64);
            tc_ld32_raw(ta, r);
            tc_ld32_raw(ta + 32, r + 32);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            tc_fence_before();
            mbar_arrive(&bar_acc_free[s]);  // the accumulator is in registers: the next MMAs may overwrite it
            const int valid = nt - jbase;    // columns of this part that are real train rows
            // a value can enter the top 2 only if its dot product reaches the
            // second best's (Hamming <= the second's): groups of 8 whose
            // largest dot falls short are skipped with 8 float max/compares
            float thr = k2 == 0xFFFFFFFFu ? -1.0e30f : (float)(256 - 2 * (int)(k2 >> 23));
#pragma unroll
            for (int c8 = 0; c8 < 64; c8 += 8) {
                float m = __uint_as_float(r[c8]);
#pragma unroll
                for (int k = 1; k < 8; k++) m = fmaxf(m, __uint_as_float(r[c8 + k]));
                if (m >= thr) {
#pragma unroll
                    for (int k = c8; k < c8 + 8; k++) {
                        const uint32_t twice =
                            (uint32_t)(0x4B400000 + 256) - __float_as_uint(__uint_as_float(r[k]) + 12582912.0f);
                        uint32_t key = (twice << 22) | (uint32_t)(jbase + k);
                        key = k < valid ? key : 0xFFFFFFFFu;
                        const uint32_t hi = max(k1, key);
                        k1 = min(k1, key);
                        k2 = min(k2, hi);
                    }
                    thr = k2 == 0xFFFFFFFFu ? -1.0e30f : (float)(256 - 2 * (int)(k2 >> 23));
                }
            }
        }
        s_part[part][row] = make_int4(k1 == 0xFFFFFFFFu ? -1 : (int)(k1 & 0x7FFFFF), (int)(k1 >> 23),
                                      k2 == 0xFFFFFFFFu ? -1 : (int)(k2 & 0x7FFFFF), (int)(k2 >> 23));
    }
    tc_fence_before();
    __syncthreads();
    // merge the 4 column parts of every query row (parts are in increasing
    // column order, so strict comparisons keep the lower index on ties)
    if (threadIdx.x < TC_M) {
        const int row = threadIdx.x;
        const int q = qtile * TC_M + row;
        int b1 = 0x7fffffff, b2 = 0x7fffffff, i1 = -1, i2 = -1;
        for (int p = 0; p < TC_EPI_WARPS / 4; p++) {
            const int4 e = s_part[p][row];
            // candidates of part p: (e.y, e.x) then (e.w, e.z); merge by (dist, index)
            const int cd[2] = {e.y, e.w}, ci[2] = {e.x, e.z};
            for (int u = 0; u < 2; u++) {
                if (ci[u] < 0) continue;
                if (cd[u] < b1 || (cd[u] == b1 && ci[u] < i1)) {
                    b2 = b1; i2 = i1; b1 = cd[u]; i1 = ci[u];
                } else if (cd[u] < b2 || (cd[u] == b2 && ci[u] < i2)) {
                    b2 = cd[u]; i2 = ci[u];
                }
            }
        }
        if (q < nq && !s_abort) partial[(size_t)blockIdx.y * nq + q] = make_int4(i1, b1, i2, b2);
    }
    __syncthreads();
    if (warp == issuer) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

}  // namespace orbgpu

using namespace orbgpu;

// Tensor-core layout self-test: fills a query tile and a train tile with
// +-1 patterns of the given descriptors (host arrays, 128 and 256 rows) and
// returns the 128 x 256 dot products (host) and a status word.
extern "C" int orbgpu_debug_tc_probe(const uint8_t* q128, const uint8_t* t256, float* dots, int* status_out, int lbo,
                                     int sbo) {
    uint8_t *dq = nullptr, *dt = nullptr, *eq = nullptr, *et = nullptr;
    float* dd = nullptr;
    int* st = nullptr;
    ORBGPU_CUDA_TRY(cudaMalloc(&dq, 128 * 32));
    ORBGPU_CUDA_TRY(cudaMalloc(&dt, 256 * 32));
    ORBGPU_CUDA_TRY(cudaMalloc(&eq, TC_QTILE_BYTES));
    ORBGPU_CUDA_TRY(cudaMalloc(&et, TC_TTILE_BYTES));
    ORBGPU_CUDA_TRY(cudaMalloc(&dd, sizeof(float) * 128 * 256));
    ORBGPU_CUDA_TRY(cudaMalloc(&st, sizeof(int)));
    ORBGPU_CUDA_TRY(cudaMemcpy(dq, q128, 128 * 32, cudaMemcpyHostToDevice));
    ORBGPU_CUDA_TRY(cudaMemcpy(dt, t256, 256 * 32, cudaMemcpyHostToDevice));
    ORBGPU_CUDA_TRY(cudaMemset(st, 0, sizeof(int)));
    ORBGPU_CUDA_TRY(cudaMemset(dd, 0, sizeof(float) * 128 * 256));
    k_expand_fp8<<<128 * 16 / 256, 256>>>(dq, 128, TC_M, eq);
    k_expand_fp8<<<256 * 16 / 256, 256>>>(dt, 256, TC_N, et);
    const size_t smem = TC_QTILE_BYTES + TC_TTILE_BYTES;
    ORBGPU_CUDA_TRY(allow_max_dynamic_smem(k_tc_probe));
    k_tc_probe<<<1, 128, smem>>>(eq, et, dd, st, (uint32_t)lbo, (uint32_t)sbo);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    ORBGPU_CUDA_TRY(cudaDeviceSynchronize());
    ORBGPU_CUDA_TRY(cudaMemcpy(dots, dd, sizeof(float) * 128 * 256, cudaMemcpyDeviceToHost));
    ORBGPU_CUDA_TRY(cudaMemcpy(status_out, st, sizeof(int), cudaMemcpyDeviceToHost));
    cudaFree(dq);
    cudaFree(dt);
    cudaFree(eq);
    cudaFree(et);
    cudaFree(dd);
    cudaFree(st);
    return ORBGPU_OK;
}

// The tensor-core kNN (algo 1 of orbgpu_knn2); see orbgpu.h.
int orbgpu_knn2_tc(orbgpu_matcher* m, const uint8_t* query, int nq, const uint8_t* train, int nt, int* idx1, int* d1,
                   int* idx2, int* d2) {
    if (nq <= 0 || nt <= 0) return ORBGPU_ERR_BAD_ARG;  // the caller answers empty sets
    cudaStream_t st = orbgpu_matcher_stream_internal(m);
    int dev, nsm;
    ORBGPU_CUDA_TRY(cudaGetDevice(&dev));
    ORBGPU_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int qt = (nq + TC_M - 1) / TC_M, tt = (nt + TC_N - 1) / TC_N;
    int nslices = std::max(1, std::min(tt, (nsm + qt - 1) / qt * 1));
    // at least ~2 waves of CTAs
    while ((long)qt * nslices < 2L * nsm && nslices < tt) nslices++;
    const int per = (tt + nslices - 1) / nslices;
    nslices = (tt + per - 1) / per;
    uint8_t *eq = nullptr, *et = nullptr;
    int4* partial = nullptr;
    int* status = nullptr;
    ORBGPU_CUDA_TRY(cudaMallocAsync((void**)&eq, (size_t)qt * TC_QTILE_BYTES, st));
    ORBGPU_CUDA_TRY(cudaMallocAsync((void**)&et, (size_t)tt * TC_TTILE_BYTES, st));
    ORBGPU_CUDA_TRY(cudaMallocAsync((void**)&partial, sizeof(int4) * (size_t)nq * nslices, st));
    ORBGPU_CUDA_TRY(cudaMallocAsync((void**)&status, sizeof(int), st));
    ORBGPU_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), st));
    k_expand_fp8<<<qt * TC_M * 16 / 256, 256, 0, st>>>(query, nq, TC_M, eq);
    k_expand_fp8<<<tt * TC_N * 16 / 256, 256, 0, st>>>(train, nt, TC_N, et);
    const size_t smem = TC_QTILE_BYTES + 2 * TC_TTILE_BYTES;
    ORBGPU_CUDA_TRY(allow_max_dynamic_smem(k_knn_tc));
    dim3 grid(qt, nslices);
    k_knn_tc<<<grid, TC_THREADS, smem, st>>>(eq, et, nq, nt, per, partial, status);
    knn_merge_launch(partial, nq, nslices, idx1, d1, idx2, d2, st);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    int hstatus = 0;
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(&hstatus, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    ORBGPU_CUDA_TRY(cudaFreeAsync(eq, st));
    ORBGPU_CUDA_TRY(cudaFreeAsync(et, st));
    ORBGPU_CUDA_TRY(cudaFreeAsync(partial, st));
    ORBGPU_CUDA_TRY(cudaFreeAsync(status, st));
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
    if (hstatus) {
        char msg[96];
        std::snprintf(msg, sizeof(msg), "tensor-core kNN wait timed out (status 0x%x)", hstatus);
        orbgpu_set_last_error(msg, __FILE__, __LINE__);
        return ORBGPU_ERR_TIMEOUT;
    }
    return ORBGPU_OK;
}
