// orbgpu_host.h -- host-side structures shared by the extractor, the batch
// pipeline and the matchers.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "orbgpu_extract_kernels.cuh"
#include "orbgpu_ext.h"

namespace orbgpu {

// Scale tables, per-level budgets, the IC_Angle row bounds and the Gaussian
// taps of one ORBextractor configuration (src/ORBextractor.cc:469-571).
struct ExtractorTables {
    int nlevels = 0;
    std::vector<float> scale, inv_scale, sigma2, inv_sigma2;
    std::vector<int> nfeat;
    int umax[ORBGPU_HALF_PATCH + 1];
    int taps[7];
};

// Geometry of one pyramid level of one image.
struct LevelGeom {
    int w, h, pitch;
    int maxBorderX, maxBorderY;
    int nCols, nRows, wCell, hCell, ncells;
    int nIni;
    int cell_cap, cand_cap, node_cap;
    int nfeat;
};

struct LevelOffsets {
    size_t pyr, blur, xofs, xalpha, yofs, ybeta, cbits, slots, cell_count, cand, node_of, quad, nodes_a,
        nodes_b, cnt4, childpos, aux0, aux1, aux2, best, kept;
};

// Byte offsets of one frame's buffers inside a device arena.
struct FrameLayout {
    std::vector<LevelOffsets> lv;
    size_t level_counts = 0, frame_total = 0;
    // three tensor maps per level (128 bytes each, level-major): the
    // descriptor kernel's level and blurred patch boxes, the FAST cell
    // kernel's ROI box
    size_t patch_maps = 0;
    size_t bytes = 0;
    size_t plan(const std::vector<LevelGeom>& g, size_t base);
};

ExtractorTables make_tables(int nfeatures, float scale_factor, int nlevels);
// Returns false if a weight pair is negative or sums above 2049 (the
// resize kernel's 32-bit vertical sum relies on both; the rounding of
// (1 - f) * 2048 and f * 2048 keeps every pair within [2047, 2049]).
bool resize_tables(int sw, int sh, int dw, int dh, int* xofs, short* xalpha, int* yofs, short* ybeta);
int level_geometry(const ExtractorTables& t, int w, int h, std::vector<LevelGeom>& g);
void fill_descs(const std::vector<LevelGeom>& g, const ExtractorTables& t, const FrameLayout& lay, uint8_t* arena,
                int frame, int ini_th, int min_th, int out_base, int out_cap, LevelDesc* out);

// Encodes the tensor maps of one frame (the layout's patch_maps block: 3 x
// 128 bytes per level) for the arena slot at 'arena' into 'out'; the caller
// copies them to arena + lay.patch_maps.
int encode_patch_maps(const std::vector<LevelGeom>& g, const FrameLayout& lay, uint8_t* arena,
                      std::vector<uint8_t>& out);

int ensure_sincos_exceptions();
int ensure_constants();
std::string default_sincos_table_path();
// Builds the table of descriptor-angle inputs whose host cosf/sinf differ
// from the rounded sincos_taylor value, and writes it to 'path'.
int build_sincos_table(const char* path, int threads);

// The reference's bForward / bBackward decision of SearchByProjection(Frame&,
// const Frame&) (src/ORBmatcher.cc:1724-1741): 1 forward, 2 backward, 0 neither.
int motion_level_mode(const orbgpu_frame_motion& mo, int mono);

// Raises a kernel's dynamic shared memory limit, once per kernel and device,
// to the most the device allows a block (less the kernel's static shared
// memory).  The limit is a function attribute shared by every thread and
// stream of the process: set per launch to the launch's own size, one thread
// could lower it below what another thread's launch in flight or captured
// graph needs.  The limit only caps requests: a launch still gets the size it
// asks for.
cudaError_t allow_max_dynamic_smem(const void* kernel);
template <typename K>
inline cudaError_t allow_max_dynamic_smem(K* kernel) {
    return allow_max_dynamic_smem(reinterpret_cast<const void*>(kernel));
}

// SM count of the current device, cached per device ordinal.
inline int nsm_of_current_device() {
    static int cache[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 132;
    if (cache[dev] == 0) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = n > 0 ? n : 132;
    }
    return cache[dev];
}

}  // namespace orbgpu
