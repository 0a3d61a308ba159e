/* orbgpu_ext.h -- entry points of liborbgpu.so beyond the reference's
 * interfaces: the batched projection search that follows
 * orbgpu_batch_extract, batch instrumentation, and the stage accessors and
 * kernels that the stage tests drive.  None of these has a counterpart in
 * ORB-SLAM2; the reference-facing entry points are in orbgpu.h.
 * Return codes are orbgpu_status values. */
#ifndef ORBGPU_EXT_H
#define ORBGPU_EXT_H

#include <stddef.h>
#include <stdint.h>

#include "orbgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ batched projection search */
/* SearchByProjection(Frame&, vector<MapPoint*>, th) (src/ORBmatcher.cc:72-183)
 * for every frame of the last orbgpu_batch_extract call, in one pass.
 * kps / desc / counts: that call's device outputs.  mappoints /
 * mp_descriptors: all frames' map points back to back (device memory or
 * page-locked host memory, read in place), frame f
 * owning [mp_offsets[f], mp_offsets[f + 1]) (host array of nframes + 1).
 * match_out: device, nframes * per_frame_capacity ints (map point index
 * within the frame, -1 none, -3 past the frame's keypoints); nmatches:
 * device, nframes ints.  Returns after the results are complete. */
int orbgpu_batch_search_by_projection(orbgpu_batch* b, const orbgpu_keypoint* kps, const uint8_t* desc,
                                      const int* counts, const orbgpu_mappoint* mappoints,
                                      const uint8_t* mp_descriptors, const int* mp_offsets, float th, float nnratio,
                                      int* match_out, int* nmatches);
/* Kernel launches of the last orbgpu_batch_search_by_projection call of the
 * calling thread (5 when every frame is resolved in shared memory, 17 with
 * the global-memory rounds). */
int orbgpu_batch_search_launch_count(void);
/* Fixed-point rounds the slowest frame of the last shared-memory resolution
 * of orbgpu_batch_search_by_projection took on the calling thread. */
int orbgpu_batch_search_rounds(void);
/* Resolution of the batched search on the calling thread: 0 (default) one
 * block per frame in shared memory when every frame fits, else the
 * global-memory rounds; 1 always the global-memory rounds.  Both give the
 * same results. */
int orbgpu_batch_search_mode(int mode);

/* SearchByProjection(Frame& CurrentFrame, const Frame& LastFrame, th, bMono)
 * (src/ORBmatcher.cc:1710-1879) for every frame of the last
 * orbgpu_batch_extract call: CurrentFrame f is the batch's frame f (its
 * mvpMapPoints empty beforehand, as TrackWithMotionModel leaves them), and
 * LastFrame f owns rows [last_offsets[f], last_offsets[f + 1]) of last_kps /
 * last_mps / last_desc (device; last_offsets and motions are host arrays of
 * nframes + 1 and nframes).  check_ori is the matcher's checkOri.
 * match_out: device, nframes * per_frame_capacity ints (LastFrame row within
 * the frame whose map point now fills the keypoint, -1 none, -4 reset by the
 * rotation check, -3 past the frame's keypoints); nmatches: device, nframes
 * ints (the reference's return value).  Per-frame capacity below 4096. */
int orbgpu_batch_search_by_projection_frame(orbgpu_batch* b, const orbgpu_keypoint* kps, const uint8_t* desc,
                                            const int* counts, const orbgpu_keypoint* last_kps,
                                            const orbgpu_frame_mappoint* last_mps, const uint8_t* last_desc,
                                            const int* last_offsets, const orbgpu_frame_motion* motions, float th,
                                            int mono, int check_ori, int* match_out, int* nmatches);

/* Frame::ComputeStereoMatches (src/Frame.cc:831-1082) for npairs (left,
 * right) frame pairs of the batch's last extraction in one pass, reading the
 * pyramids the extraction left in the batch's arena.  left_frame[p] /
 * right_frame[p]: frame indices of that extraction (same image size); bf[p]
 * (mbf) and fx[p] (K(0,0)): the pair's camera (host arrays).  kps / desc /
 * counts: the extraction's outputs (device; frame f's rows at f *
 * per_frame_capacity).  uright / depth: device, npairs * per_frame_capacity
 * floats; pair p's left keypoint i at p * per_frame_capacity + i (rows past
 * the left frame's count are not written).  Returns after the stream
 * finished. */
int orbgpu_batch_compute_stereo_matches(orbgpu_batch* b, const orbgpu_keypoint* kps, const uint8_t* desc,
                                        const int* counts, int npairs, const int* left_frame, const int* right_frame,
                                        const float* bf, const float* fx, float* uright, float* depth);

/* ------------------------------------------------------------ serving state */
/* The serving loop's per-stream LastFrame state (no reference counterpart:
 * the reference keeps one Tracking object, with its mLastFrame, per camera).
 * A store holds max_streams slots of 'cap' rows each: keypoints, map points
 * (orbgpu_frame_mappoint) and descriptors of the stream's previous frame.
 * All calls are asynchronous on 'stream' (a cudaStream_t); arrays are device
 * memory. */
typedef struct orbgpu_stream_state orbgpu_stream_state;
int orbgpu_stream_state_create(int max_streams, int cap, orbgpu_stream_state** out);
/* Waits for all device work (the calls run on the callers' streams), then
 * frees the store. */
int orbgpu_stream_state_destroy(orbgpu_stream_state* s);
/* LastFrame rows of a batch: frame f's previous frame is slot slots[f]; its
 * offsets[f + 1] - offsets[f] rows (at most max_rows) are copied to
 * last_kps / last_mps / last_desc from row offsets[f] -- the inputs of
 * orbgpu_batch_search_by_projection_frame. */
int orbgpu_stream_state_gather(orbgpu_stream_state* s, int nframes, const int* slots, const int* offsets,
                               int max_rows, orbgpu_keypoint* last_kps, orbgpu_frame_mappoint* last_mps,
                               uint8_t* last_desc, void* stream);
/* The batch's frames become their streams' previous frames: frame f's
 * counts[f] keypoints (rows f * cap of kps / desc, the batch's outputs) are
 * copied to slot slots[f], each with the map point where its ray meets the
 * plane Z = depth[f]: rays[12 f ..] = R^T K^-1 (row-major 3 x 3) and the camera
 * centre -R^T t of the frame's pose, doubles; flags = ORBGPU_MP_* of every
 * new map point. */
int orbgpu_stream_state_update(orbgpu_stream_state* s, int nframes, const int* slots, const orbgpu_keypoint* kps,
                               const uint8_t* desc, const int* counts, int cap, const double* rays,
                               const double* depth, int flags, void* stream);
/* Device pointers of slot 'slot''s rows (cap each; any output may be NULL). */
int orbgpu_stream_state_slot(const orbgpu_stream_state* s, int slot, const orbgpu_keypoint** kps,
                             const orbgpu_frame_mappoint** mps, const uint8_t** desc);
/* TrackWithMotionModel's retry (src/Tracking.cc:1347-1353): frames whose
 * first search found fewer than min_matches take the second search's result
 * (match2 / nmatches2, run with 2 th); match / nmatches are updated in place
 * (frame f's rows at f * cap). */
int orbgpu_serving_retry_select(int* match, int* nmatches, const int* match2, const int* nmatches2, int cap,
                                int nframes, int min_matches, void* stream);

/* ------------------------------------------------------------ batch instrumentation */
/* Device milliseconds of the five stages of the last orbgpu_batch_extract
 * (gather, resize + blur, FAST, octree, orientation + descriptor); n >= 5. */
int orbgpu_batch_stage_times(orbgpu_batch* b, float* ms, int n);
/* Kernel launches of one orbgpu_batch_extract of the last frame list. */
int orbgpu_batch_launch_count(const orbgpu_batch* b);
/* The batch's CUDA stream (cudaStream_t). */
void* orbgpu_batch_stream(const orbgpu_batch* b);

/* ------------------------------------------------------------ stage accessors (tests) */
/* Device pointer of blurred level 'level' of the last extraction (same
 * geometry as orbgpu_extractor_pyramid_level). */
int orbgpu_extractor_blurred_level(const orbgpu_extractor* ex, int level, const uint8_t** dev_ptr);
/* Per-level internals of the last extraction, copied to the host dst
 * (cap bytes): what = 0 cell counts (ncells ints), 1 cell slots (ncells *
 * cell_cap uint32: x | y << 12 | score << 24, level coordinates), 2
 * distributed keypoints (node_cap uint32), 3 geometry (8 ints: nCols,
 * nRows, wCell, hCell, cell_cap, nIni, node_cap, keypoints kept). */
int orbgpu_extractor_debug_level(const orbgpu_extractor* ex, int level, int what, void* dst, size_t cap);
/* Synchronous device-to-host copy (device-wide synchronize first). */
int orbgpu_copy_to_host(void* dst, const void* src, size_t bytes);
/* Arc strength (FAST score + 1, 0 = no corner) of every pixel of a device
 * image at threshold t, into out (w * h bytes, device). */
int orbgpu_debug_fast_strength(const uint8_t* img, int pitch, int w, int h, int t, uint8_t* out);
/* The descriptor rotation's cos / sin of n device floats (device outputs). */
int orbgpu_descriptor_sincos(const float* x, int n, float* c, float* s);
/* One 128 x 256 x 256 FP8 tensor-core MMA group of +-1 expansions of host
 * descriptors (128 and 256 rows) with the given operand strides; dots:
 * host 128 x 256 floats. */
int orbgpu_debug_tc_probe(const uint8_t* q128, const uint8_t* t256, float* dots, int* status_out, int lbo, int sbo);

/* ------------------------------------------------------------ autotuner parameters */
/* Launch shapes the autotuner chooses (orb_slam2_detailed_comments_gb300.autotune):
 *   "resize_rows"          strip rows of the resize and blur / FAST pre-test kernels: 8, 22, 36, 64
 *   "fast_cells_per_block" warps per block of the FAST cell kernel: 1, 2, 4
 *   "describe_group"       keypoints per staging round of the descriptor kernel: 1, 2, 4
 *   "describe_depth"       staging rounds in flight per warp of the descriptor kernel: 2, 4
 *                          (with describe_group 4, 2 is used)
 *   "knn_tc_min_pairs"     query x train size from which orbgpu_knn2(algo -1) uses tcgen05
 * and three policies for launches too small to fill the device (one frame, a
 * few frames), which the autotuner leaves alone:
 *   "describe_task"        keypoints per descriptor warp task: 0 (by the launch's keypoint
 *                          count, the default), 8, 16, 32
 *   "fast_chunk"           consecutive cells per FAST cell warp chunk: 0 (by the launch's
 *                          cell count, the default), 1, 2, 4
 *   "strip_rows_small"     strip rows of resize and blur launches whose level-0 strips would
 *                          not fill the device: 8 (the default), or 0 for resize_rows always
 * Process-wide; a change makes extractors and batches re-plan (and re-capture
 * their graphs) on their next call.  Results do not depend on these values. */
int orbgpu_tune_set(const char* name, long long value);
int orbgpu_tune_get(const char* name, long long* value);

/* ------------------------------------------------------------ failure injection (tests) */
/* The library's next 'count' working-buffer allocations (extractor plans,
 * batch arenas and scratch, stream state stores) fail as if the device had
 * no memory left: the call that needed one returns ORBGPU_ERR_OOM and leaves
 * its handle usable.  0 turns the injection off. */
int orbgpu_debug_fail_allocations(int count);

/* ------------------------------------------------------------ rotation table */
/* Builds the descriptor-rotation exception table (path NULL = next to the
 * library) with 'threads' host threads. */
int orbgpu_build_sincos_table(const char* path, int threads);
/* Where the library looks for that table. */
const char* orbgpu_sincos_table_path(void);

#ifdef __cplusplus
}
#endif

#endif /* ORBGPU_EXT_H */
