// orbgpu_knn.cu -- brute-force k = 2 Hamming nearest neighbours.
//
// Popcount path: every thread owns one query (its 256 bits in registers) and
// streams tiles of train rows through shared memory; the train set is split
// into slices across blocks so the grid covers the GPU, and a merge kernel
// combines the per-slice (best, second) pairs.  Ties go to the lower train
// index, the rule of a sequential scan over DescriptorDistance
// (src/ORBmatcher.cc:2083-2103).
#include <algorithm>
#include <mutex>

#include "orbgpu_host.h"

cudaStream_t orbgpu_matcher_stream_internal(orbgpu_matcher* m);

namespace orbgpu {

#define KNN_QPB 128
#define KNN_TILE 256

__global__ void __launch_bounds__(KNN_QPB) k_knn_popc(const uint4* __restrict__ q, int nq, const uint4* __restrict__ t,
                                                     int nt, int slice, int4* __restrict__ partial) {
    __shared__ uint4 tile[KNN_TILE * 2];
    const int qi = blockIdx.x * KNN_QPB + threadIdx.x;
    const int t0 = blockIdx.y * slice, t1 = min(nt, t0 + slice);
    uint4 a0 = make_uint4(0, 0, 0, 0), a1 = a0;
    if (qi < nq) {
        a0 = q[2 * (size_t)qi];
        a1 = q[2 * (size_t)qi + 1];
    }
    int b1 = 0x7fffffff, b2 = 0x7fffffff, i1 = -1, i2 = -1;
    for (int base = t0; base < t1; base += KNN_TILE) {
        const int nb = min(KNN_TILE, t1 - base);
        __syncthreads();
        for (int k = threadIdx.x; k < 2 * nb; k += KNN_QPB) tile[k] = t[2 * (size_t)base + k];
        __syncthreads();
        for (int j = 0; j < nb; j++) {
            const int d = hamming256(a0, a1, tile[2 * j], tile[2 * j + 1]);
            if (d < b1) {
                b2 = b1;
                i2 = i1;
                b1 = d;
                i1 = base + j;
            } else if (d < b2) {
                b2 = d;
                i2 = base + j;
            }
        }
    }
    if (qi < nq) partial[(size_t)blockIdx.y * nq + qi] = make_int4(i1, b1, i2, b2);
}

__global__ void k_knn_merge(const int4* __restrict__ partial, int nq, int nslices, int* idx1, int* d1, int* idx2,
                            int* d2) {
    const int qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nq) return;
    // slices are in increasing train order, so strict comparisons keep the
    // lower index on ties
    int b1 = 0x7fffffff, b2 = 0x7fffffff, i1 = -1, i2 = -1;
    for (int s = 0; s < nslices; s++) {
        const int4 p = partial[(size_t)s * nq + qi];
        if (p.x >= 0) {
            if (p.y < b1) {
                b2 = b1; i2 = i1; b1 = p.y; i1 = p.x;
            } else if (p.y < b2) {
                b2 = p.y; i2 = p.x;
            }
        }
        if (p.z >= 0) {
            if (p.w < b1) {
                b2 = b1; i2 = i1; b1 = p.w; i1 = p.z;
            } else if (p.w < b2) {
                b2 = p.w; i2 = p.z;
            }
        }
    }
    idx1[qi] = i1;
    d1[qi] = b1;
    idx2[qi] = i2;
    d2[qi] = b2;
}

// Lowe's ratio test in the reference's form (src/ORBmatcher.cc:647:
// bestDist < (float)bestDist2 * nnratio); no second neighbour rejects.
__global__ void k_knn_accept(const int* d1, const int* d2, int n, float ratio, uint8_t* accept) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int b = d1[i], s = d2[i];
    accept[i] = (s != 0x7fffffff && (float)b < __fmul_rn((float)s, ratio)) ? 1 : 0;
}

}  // namespace orbgpu

using namespace orbgpu;

extern "C" int orbgpu_knn2_accept(const int* d1, const int* d2, int n, float ratio, uint8_t* accept, void* stream) {
    if (n < 0 || (n > 0 && (!d1 || !d2 || !accept))) return ORBGPU_ERR_BAD_ARG;
    if (n == 0) return ORBGPU_OK;
    cudaStream_t st = (cudaStream_t)stream;
    k_knn_accept<<<(n + 255) / 256, 256, 0, st>>>(d1, d2, n, ratio, accept);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
    return ORBGPU_OK;
}

void knn_merge_launch(const int4* partial, int nq, int nslices, int* idx1, int* d1, int* idx2, int* d2,
                      cudaStream_t st) {
    k_knn_merge<<<(nq + 255) / 256, 256, 0, st>>>(partial, nq, nslices, idx1, d1, idx2, d2);
}

int orbgpu_knn2_tc(orbgpu_matcher* m, const uint8_t* query, int nq, const uint8_t* train, int nt, int* idx1, int* d1,
                   int* idx2, int* d2);

extern "C" int orbgpu_knn2(orbgpu_matcher* m, const uint8_t* query, int nq, const uint8_t* train, int nt, int* idx1,
                           int* d1, int* idx2, int* d2, int algo) {
    if (!m || nq < 0 || nt < 0 || (nq > 0 && (!query || !idx1 || !d1 || !idx2 || !d2)) || (nt > 0 && !train) ||
        (algo != 0 && algo != 1 && algo != -1))
        return ORBGPU_ERR_BAD_ARG;
    if (nq == 0) return ORBGPU_OK;
    if (algo == -1)  // automatic: the tensor cores from the tuned problem size on
        algo = (long long)nq * nt >= tunables().knn_tc_min_pairs ? 1 : 0;
    if (nt >= (1 << 23)) algo = 0;  // the tensor-core epilogue packs train indices in 23 bits
    if (algo == 1 && nt > 0) return orbgpu_knn2_tc(m, query, nq, train, nt, idx1, d1, idx2, d2);
    cudaStream_t st = orbgpu_matcher_stream_internal(m);
    int dev, nsm;
    ORBGPU_CUDA_TRY(cudaGetDevice(&dev));
    ORBGPU_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int qblocks = (nq + KNN_QPB - 1) / KNN_QPB;
    // enough slices for ~8 resident blocks per SM, each slice a whole number of tiles
    int nslices = std::max(1, std::min((nt + KNN_TILE - 1) / KNN_TILE, (8 * nsm + qblocks - 1) / qblocks));
    int slice = (nt + nslices - 1) / nslices;
    slice = ((slice + KNN_TILE - 1) / KNN_TILE) * KNN_TILE;
    nslices = std::max(1, (nt + slice - 1) / std::max(1, slice));
    int4* partial = nullptr;
    ORBGPU_CUDA_TRY(cudaMallocAsync((void**)&partial, sizeof(int4) * (size_t)nq * nslices, st));
    dim3 grid(qblocks, nslices);
    k_knn_popc<<<grid, KNN_QPB, 0, st>>>((const uint4*)query, nq, (const uint4*)train, nt, slice, partial);
    k_knn_merge<<<(nq + 255) / 256, 256, 0, st>>>(partial, nq, nslices, idx1, d1, idx2, d2);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    ORBGPU_CUDA_TRY(cudaFreeAsync(partial, st));
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
    return ORBGPU_OK;
}

// ---------------------------------------------------------------- allocation-free variant
// orbgpu_knn2_noalloc keeps its per-slice (best, second) pairs in this
// file-scope device array instead of memory it allocates.  Each GPU that
// loads the library holds the array (16 MiB) until the process exits.
#define ORBGPU_KNN_NOALLOC_MAX_PARTIAL (1 << 20)
static __device__ __align__(256) int4 g_knn_noalloc_partial[ORBGPU_KNN_NOALLOC_MAX_PARTIAL];

namespace {
std::mutex g_noalloc_mutex;
// device address of the array, per device ordinal, looked up once; a
// cudaDeviceReset ends the context that address belongs to, so it must not be
// followed by further calls in the same process
int4* g_noalloc_partial[256] = {};
}  // namespace

extern "C" int orbgpu_knn2_noalloc(const uint8_t* query, int nq, const uint8_t* train, int nt, int* idx1, int* d1,
                                   int* idx2, int* d2, void* stream) {
    if (nq < 0 || nt < 0 || (nq > 0 && (!query || !idx1 || !d1 || !idx2 || !d2)) || (nt > 0 && !train)) {
        orbgpu_set_last_error("invalid kNN arguments", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (nq > ORBGPU_KNN_NOALLOC_MAX_PARTIAL) {
        orbgpu_set_last_error("orbgpu_knn2_noalloc: more than 1048576 query rows (its fixed scratch holds one "
                              "(best, second) pair per query per train slice)", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (nq == 0) return ORBGPU_OK;
    int dev = 0, nsm = 0;
    ORBGPU_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) {
        orbgpu_set_last_error("orbgpu_knn2_noalloc: device ordinal beyond 255", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    int4* partial = nullptr;
    {
        // first call on a device: look up the array's device address with
        // that device current (the host-side symbol is not a device address)
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_partial[dev]) {
            void* p = nullptr;
            ORBGPU_CUDA_TRY(cudaGetSymbolAddress(&p, g_knn_noalloc_partial));
            g_noalloc_partial[dev] = (int4*)p;
        }
        partial = g_noalloc_partial[dev];
    }
    ORBGPU_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t st = (cudaStream_t)stream;
    const int qblocks = (nq + KNN_QPB - 1) / KNN_QPB;
    int nslices = std::max(1, std::min((nt + KNN_TILE - 1) / KNN_TILE, (8 * nsm + qblocks - 1) / qblocks));
    nslices = std::max(1, std::min(nslices, ORBGPU_KNN_NOALLOC_MAX_PARTIAL / nq));
    int slice = (nt + nslices - 1) / nslices;
    slice = ((slice + KNN_TILE - 1) / KNN_TILE) * KNN_TILE;
    nslices = std::max(1, (nt + slice - 1) / std::max(1, slice));
    // every partial entry read by the merge is written by the popcount
    // kernel of the same call, so nothing is cleared between calls
    dim3 grid(qblocks, nslices);
    k_knn_popc<<<grid, KNN_QPB, 0, st>>>((const uint4*)query, nq, (const uint4*)train, nt, slice, partial);
    k_knn_merge<<<(nq + 255) / 256, 256, 0, st>>>(partial, nq, nslices, idx1, d1, idx2, d2);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    return ORBGPU_OK;
}
