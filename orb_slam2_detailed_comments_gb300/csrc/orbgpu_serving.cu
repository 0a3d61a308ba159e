// orbgpu_serving.cu -- the per-stream state of the serving loop on the device.
//
// The serving loop (orb_slam2_detailed_comments_gb300/serving.py) runs
// TrackWithMotionModel's search, SearchByProjection(CurrentFrame, LastFrame,
// th, bMono) (src/Tracking.cc:1321-1353, src/ORBmatcher.cc:1710-1879), for a
// batch of frames from many camera streams, each against its own stream's
// previous frame.  The previous frames live in a state store: per stream slot
// 'cap' rows of keypoints, map points (orbgpu_frame_mappoint) and
// descriptors.  Three launches per batch, all asynchronous on the caller's
// stream:
//   k_state_gather   the LastFrame rows of every batch frame, back to back
//                    (the batched search's last_kps / last_mps / last_desc);
//   k_state_update   the batch's keypoints and descriptors become the
//                    streams' new rows, and each keypoint's map point is its
//                    ray from the frame's pose met with the plane Z = depth of
//                    the stream's scene model (the synthetic streams view a
//                    textured plane; this stands in for stereo depth or
//                    triangulated points), in double, independent of the batch;
//   k_retry_select   the 2 * th retry of TrackWithMotionModel (src/Tracking.cc:
//                    1347-1353): a frame whose first search found fewer than
//                    20 matches takes the second search's result.
#include <algorithm>

#include "orbgpu_common.cuh"
#include "orbgpu_ext.h"
#include "orbgpu_host.h"

namespace orbgpu {

__global__ void k_state_gather(const orbgpu_keypoint* __restrict__ skps, const orbgpu_frame_mappoint* __restrict__ smps,
                               const uint4* __restrict__ sdesc, int cap, const int* __restrict__ slots,
                               const int* __restrict__ offsets, int nframes, orbgpu_keypoint* __restrict__ lkps,
                               orbgpu_frame_mappoint* __restrict__ lmps, uint4* __restrict__ ldesc) {
    const int f = blockIdx.y;
    if (f >= nframes) return;
    const int o0 = offsets[f], n = offsets[f + 1] - o0;
    const size_t src0 = (size_t)slots[f] * cap;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n && k < cap; k += gridDim.x * blockDim.x) {
        lkps[o0 + k] = skps[src0 + k];
        lmps[o0 + k] = smps[src0 + k];
        ldesc[2 * (size_t)(o0 + k)] = sdesc[2 * (src0 + k)];
        ldesc[2 * (size_t)(o0 + k) + 1] = sdesc[2 * (src0 + k) + 1];
    }
}

// rays[f]: M (row-major 3 x 3, R^T K^-1 of the frame's pose) then the camera
// centre C (3), doubles; depth[f]: the plane Z of the frame's stream.
__global__ void k_state_update(const orbgpu_keypoint* __restrict__ kps, const uint4* __restrict__ desc,
                               const int* __restrict__ counts, int cap, const int* __restrict__ slots,
                               const double* __restrict__ rays, const double* __restrict__ depth, int nframes,
                               int flags, orbgpu_keypoint* __restrict__ skps, orbgpu_frame_mappoint* __restrict__ smps,
                               uint4* __restrict__ sdesc) {
    const int f = blockIdx.y;
    if (f >= nframes) return;
    const int n = min(counts[f], cap);
    const size_t src0 = (size_t)f * cap, dst0 = (size_t)slots[f] * cap;
    const double* M = rays + 12 * f;
    const double* C = M + 9;
    const double Z = depth[f];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const orbgpu_keypoint kp = kps[src0 + k];
        const double x = (double)kp.x, y = (double)kp.y;
        // ray direction M (x, y, 1) and its meeting with Z = depth, each
        // product rounded separately (no contraction: the library is built
        // with -fmad=false)
        const double dx = __dadd_rn(__dadd_rn(__dmul_rn(M[0], x), __dmul_rn(M[1], y)), M[2]);
        const double dy = __dadd_rn(__dadd_rn(__dmul_rn(M[3], x), __dmul_rn(M[4], y)), M[5]);
        const double dz = __dadd_rn(__dadd_rn(__dmul_rn(M[6], x), __dmul_rn(M[7], y)), M[8]);
        const double lam = __ddiv_rn(__dsub_rn(Z, C[2]), dz);
        orbgpu_frame_mappoint mp;
        mp.x = (float)__dadd_rn(C[0], __dmul_rn(lam, dx));
        mp.y = (float)__dadd_rn(C[1], __dmul_rn(lam, dy));
        mp.z = (float)__dadd_rn(C[2], __dmul_rn(lam, dz));
        mp.flags = flags;
        skps[dst0 + k] = kp;
        smps[dst0 + k] = mp;
        sdesc[2 * (dst0 + k)] = desc[2 * (src0 + k)];
        sdesc[2 * (dst0 + k) + 1] = desc[2 * (src0 + k) + 1];
    }
}

// One block per frame: every thread reads the frame's first count before
// thread 0 replaces it.
__global__ void k_retry_select(int* __restrict__ match, int* __restrict__ nm, const int* __restrict__ match2,
                               const int* __restrict__ nm2, int cap, int nframes, int min_matches) {
    const int f = blockIdx.x;
    if (f >= nframes) return;
    const bool retry = nm[f] < min_matches;
    __syncthreads();
    if (!retry) return;
    for (int k = threadIdx.x; k < cap; k += blockDim.x) match[(size_t)f * cap + k] = match2[(size_t)f * cap + k];
    if (threadIdx.x == 0) nm[f] = nm2[f];
}

}  // namespace orbgpu

using namespace orbgpu;

struct orbgpu_stream_state {
    int max_streams = 0, cap = 0;
    orbgpu_keypoint* kps = nullptr;
    orbgpu_frame_mappoint* mps = nullptr;
    uint8_t* desc = nullptr;
};

extern "C" int orbgpu_stream_state_create(int max_streams, int cap, orbgpu_stream_state** out) {
    if (!out || max_streams < 1 || cap < 1) {
        orbgpu_set_last_error("invalid stream state size", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    orbgpu_stream_state* s = new orbgpu_stream_state();
    s->max_streams = max_streams;
    s->cap = cap;
    const size_t rows = (size_t)max_streams * cap;
    if (dev_malloc(&s->kps, sizeof(orbgpu_keypoint) * rows) != cudaSuccess ||
        dev_malloc(&s->mps, sizeof(orbgpu_frame_mappoint) * rows) != cudaSuccess ||
        dev_malloc(&s->desc, 32 * rows) != cudaSuccess) {
        orbgpu_stream_state_destroy(s);
        orbgpu_set_last_error("stream state allocation failed", __FILE__, __LINE__);
        return ORBGPU_ERR_OOM;
    }
    *out = s;
    return ORBGPU_OK;
}

extern "C" int orbgpu_stream_state_destroy(orbgpu_stream_state* s) {
    if (!s) return ORBGPU_OK;
    // gathers and updates run on the callers' streams: all of them are done
    // before the store is freed
    cudaDeviceSynchronize();
    cudaFree(s->kps);
    cudaFree(s->mps);
    cudaFree(s->desc);
    delete s;
    return ORBGPU_OK;
}

extern "C" int orbgpu_stream_state_gather(orbgpu_stream_state* s, int nframes, const int* slots, const int* offsets,
                                          int max_rows, orbgpu_keypoint* last_kps, orbgpu_frame_mappoint* last_mps,
                                          uint8_t* last_desc, void* stream) {
    if (!s || nframes < 0 || (nframes > 0 && (!slots || !offsets || !last_kps || !last_mps || !last_desc)) ||
        max_rows < 0) {
        orbgpu_set_last_error("invalid stream state gather", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (nframes == 0 || max_rows == 0) return ORBGPU_OK;
    const int rows = std::min(max_rows, s->cap);
    dim3 g((rows + 255) / 256, nframes);
    k_state_gather<<<g, 256, 0, (cudaStream_t)stream>>>(s->kps, s->mps, (const uint4*)s->desc, s->cap, slots, offsets,
                                                        nframes, last_kps, last_mps, (uint4*)last_desc);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    return ORBGPU_OK;
}

extern "C" int orbgpu_stream_state_update(orbgpu_stream_state* s, int nframes, const int* slots,
                                          const orbgpu_keypoint* kps, const uint8_t* desc, const int* counts, int cap,
                                          const double* rays, const double* depth, int flags, void* stream) {
    if (!s || nframes < 0 || cap != s->cap ||
        (nframes > 0 && (!slots || !kps || !desc || !counts || !rays || !depth))) {
        orbgpu_set_last_error("invalid stream state update", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (nframes == 0) return ORBGPU_OK;
    dim3 g((cap + 255) / 256, nframes);
    k_state_update<<<g, 256, 0, (cudaStream_t)stream>>>(kps, (const uint4*)desc, counts, cap, slots, rays, depth,
                                                        nframes, flags, s->kps, s->mps, (uint4*)s->desc);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    return ORBGPU_OK;
}

extern "C" int orbgpu_serving_retry_select(int* match, int* nmatches, const int* match2, const int* nmatches2,
                                           int cap, int nframes, int min_matches, void* stream) {
    if (nframes < 0 || cap < 0 || (nframes > 0 && (!match || !nmatches || !match2 || !nmatches2))) {
        orbgpu_set_last_error("invalid retry selection", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (nframes == 0 || cap == 0) return ORBGPU_OK;
    k_retry_select<<<nframes, 256, 0, (cudaStream_t)stream>>>(match, nmatches, match2, nmatches2, cap, nframes,
                                                             min_matches);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    return ORBGPU_OK;
}

extern "C" int orbgpu_stream_state_slot(const orbgpu_stream_state* s, int slot, const orbgpu_keypoint** kps,
                                        const orbgpu_frame_mappoint** mps, const uint8_t** desc) {
    if (!s || slot < 0 || slot >= s->max_streams) {
        orbgpu_set_last_error("invalid stream state slot", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    const size_t r0 = (size_t)slot * s->cap;
    if (kps) *kps = s->kps + r0;
    if (mps) *mps = s->mps + r0;
    if (desc) *desc = s->desc + 32 * r0;
    return ORBGPU_OK;
}
