// orbgpu_extract_kernels.cuh -- the ORB extraction stages as CUDA kernels.
//
// Each kernel walks a list of work items, so the same kernels serve one frame
// (the drop-in path) and a ragged batch of frames of different sizes.
//
//   k_level_resize       level l from level l-1 (cv::resize INTER_LINEAR,
//                        11-bit fixed point).
//   k_level_strip        the 7x7 sigma-2 blur of level l (REFLECT_101) and the
//                        FAST compass pre-test of every pixel of the cells'
//                        detection region (a candidate bit map): one warp per
//                        120-column strip, rows walked with a 7-row register
//                        window.
//   k_fast_cells         one 30-px cell at a time per warp (persistent, in
//                        chunks of 1 or 2 cells): the cell's ROI staged in
//                        shared memory by a tensor copy, the segment test and
//                        arc strength of the cell's candidates, per-ROI
//                        non-max suppression at iniThFAST and minThFAST in
//                        one pass (the latter used when the former keeps
//                        nothing), ordered compaction.
//   k_distribute         one (frame, level) per block: DistributeOctTree as a
//                        sequence of parallel split steps over node creation
//                        numbers, its arrays in shared memory when they fit.
//   k_describe           8, 16 or 32 keypoints per warp task, their patches
//                        staged in shared memory by tensor copies in rounds
//                        of 1 to 4: IC_Angle, fastAtan2, rBRIEF.
#pragma once

#include "orbgpu_common.cuh"

namespace orbgpu {

// Patch boxes of the descriptor kernel's tensor copies (bytes x rows): the
// IC_Angle disc of radius HALF_PATCH_SIZE from a 16-byte aligned column of
// the level plane, and the rBRIEF samples (rotated pattern points lie within
// 18.4 pixels of the keypoint) from a 16-byte aligned column of the blurred
// plane.  Each box has its own 128-byte aligned slot in shared memory, large
// enough for either box.
#define ORBGPU_TMAP_BYTES 128
#define DESC_LBOX_W 48
#define DESC_LBOX_H (2 * ORBGPU_HALF_PATCH + 1)
#define DESC_BBOX_R 19
#define DESC_BBOX_W 64
#define DESC_BBOX_H (2 * DESC_BBOX_R + 1)
#define DESC_SLOT 2560  // 64 x 39 = 2496 bytes (the larger box), rounded up to 128

// Per-(frame, level) description shared by all stages.
struct LevelDesc {
    // pyramid
    const uint8_t* src;  // level l-1 (unused at level 0)
    int sw, sh, spitch;
    uint8_t* dst;  // level l (unblurred)
    uint8_t* blur; // level l blurred (same pitch)
    int w, h, pitch;
    const int* xofs;      // resize tables of this level: source column per output column
    const short* xalpha;  // 2 weights per output column
    const int* yofs;      // source row per output row (unclamped)
    const short* ybeta;   // 2 weights per output row
    // FAST cells
    int nCols, nRows, wCell, hCell;
    int maxBorderX, maxBorderY;
    int cell_cap;
    uint32_t* slots;  // nCols*nRows*cell_cap packed (x | y << 12 | score << 24), level coordinates
    int* cell_count;  // nCols*nRows
    int ini_th, min_th;
    // FAST candidates (pixels that passed the compass pre-test), one bit per
    // pixel: bit x & 7 of byte x >> 3 of row y, written by k_level_strip for
    // the detection rows and columns [19, dim - 19), read by k_fast_cells
    uint8_t* cbits;
    int cbits_stride;  // bytes per row: pitch / 8
    // tensor map of the level plane for k_fast_cells' copy of a cell's ROI:
    // box cell_box_w x (hCell + 6) bytes from a 16-byte aligned column
    const void* tm_cell;
    int cell_box_w;
    // distribute
    int nfeat;
    int nIni;
    int cand_cap;     // nCols*nRows*cell_cap
    int node_cap;
    uint32_t* cand;   // cand_cap
    int* node_of;     // cand_cap
    uint8_t* quad;    // cand_cap
    void* nodes_a;    // node_cap DNode
    void* nodes_b;    // node_cap DNode
    int4* cnt4;       // node_cap
    int4* childpos;   // node_cap
    int* aux0;        // node_cap (split rank / order)
    int* aux1;        // node_cap
    int* aux2;        // node_cap
    uint32_t* best;   // node_cap
    uint32_t* kept;   // node_cap: distributed keypoints, packed like slots
    int* kept_count;  // one int
    // describe
    int level;
    int frame;
    float scale;          // mvScaleFactor[level]
    int* level_counts;    // the frame's kept_count of every level (nlevels ints)
    int nlevels;
    int out_base;         // first output row of the frame
    int out_cap;          // output rows available to the frame
    int* frame_total;     // the frame's keypoint count
    // tensor maps (CUtensorMap, in the frame's arena) of the level plane and
    // the blurred plane for the descriptor kernel's patch copies
    const void* tm_level;
    const void* tm_blur;
};

// Launch shapes chosen by the autotuner (orbgpu_tune_set): strip rows of the
// resize and blur / FAST pre-test kernels, warps per block of the FAST cell
// kernel, keypoints per staging round and rounds in flight of the descriptor
// kernel, and the query x train size from which orbgpu_knn2's automatic
// choice uses the tensor cores.  Three launch policies for launches too
// small to fill the device (one frame, a few frames): keypoints per
// descriptor task (0: by the launch's keypoint count, else 8 / 16 / 32),
// cells per FAST chunk (0: by the launch's cell count, else 1 / 2 / 4) and
// the strip rows of such launches (8, or 0 for resize_rows always).
// Changing one bumps the generation, so cached frame plans and captured
// graphs are rebuilt.
struct Tunables {
    int resize_rows = 36;
    int fast_cells_per_block = 4;
    int describe_group = 1;
    int describe_depth = 2;
    int describe_task = 0;
    int fast_chunk = 0;
    int strip_rows_small = 8;
    long long knn_tc_min_pairs = 1LL << 28;
};
const Tunables& tunables();
int tune_generation();

struct DNode {
    int16_t x0, x1, y0, y1;
    int32_t cnt;
    int32_t id;
    int32_t flags;  // 1 = bNoMore, 2 = initial node
};

// One tile of k_level_resize_blur / one cell of k_fast_cells.
struct WorkItem {
    int desc;
    int index;
};

// The work of one launch over a list of n entries (frames, or (frame,
// level) pairs): entry e owns blocks [prefix[e], prefix[e+1]) and uses level
// descriptor desc0 + e * desc_stride.  Blocks find their entry by binary
// search, so the host uploads n + 1 ints per launch instead of a block list.
struct RangeMap {
    const int* prefix;
    int n;
    int desc0;
    int desc_stride;
};

void upload_constants(cudaStream_t st, const int* taps, const int* umax);
void set_sincos_exceptions(const uint32_t* ck, const float* cv, int cn, const uint32_t* sk, const float* sv, int sn,
                           const int* cb, const int* sb, const uint16_t* csub, const uint16_t* ssub, int nbuckets);
// Level l's resize (l >= 1) and its blur / FAST pre-test strips, in strips of
// 'rows' rows; callers run the resize chain on one stream and the strips on
// another (the strip of level l after the resize of level l).
void launch_level_resize(const LevelDesc* descs, RangeMap rm, int nitems, int rows, cudaStream_t st);
void launch_level_strip(const LevelDesc* descs, RangeMap rm, int nitems, int rows, cudaStream_t st);
// Shared memory layout of k_fast_cells for one launch (per warp).
struct FastCellsSmem {
    int tile_bytes;  // the largest ROI box of the launch, 128-byte multiple
    int rows;        // strength window rows: the largest detection region + 2
    int win_stride;  // strength window row bytes: the largest region width + 8, 16-byte multiple
    int cand_cap;    // candidates: the largest detection region's pixels
    int min_cap;     // survivors kept per threshold
    // tile_bytes + rows * win_stride + 2 * cand_cap + 2 * min_cap (the
    // candidate list, which the minThFAST survivors reuse, and the iniThFAST
    // survivors), 128-byte multiple
    int warp_bytes;
};
// The cell box width of a level (16-byte multiple covering the ROI from a
// 16-byte aligned column).
inline int fast_cell_box_w(int wcell) { return (15 + wcell + 6 + 15) & ~15; }
// The FAST cells of a launch: rm maps work item u (0 <= u < ncells) to a
// (frame, level) entry and a cell of it (the prefix counts cells);
// max_wcell / max_hcell / max_box_bytes: the largest cell and ROI box of the
// launch (they size its shared memory).
void launch_fast(const LevelDesc* descs, RangeMap rm, int ncells, int* status, int max_wcell, int max_hcell,
                 int max_box_bytes, cudaStream_t st);
int resize_blur_tiles(int w, int h, int rows);
int strip_rows(long level0_pixels);
// DistributeOctTree of every (frame, level); node_cap: the largest level's
// node capacity (its arrays go to shared memory when they fit).
void launch_distribute(const LevelDesc* descs, int ndescs, int sort_cap, int node_cap, int* status,
                       cudaStream_t st);
void launch_describe(const LevelDesc* descs, int ndescs, int max_kept, orbgpu_keypoint* kps, uint8_t* desc, int* status,
                     cudaStream_t st);

}  // namespace orbgpu
