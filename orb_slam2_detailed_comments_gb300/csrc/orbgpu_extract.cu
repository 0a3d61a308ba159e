// orbgpu_extract.cu -- host side of the extractor: level geometry, device
// buffers, work lists and the C ABI of include/orbgpu.h for extraction.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "orbgpu_extract_kernels.cuh"
#include "orbgpu_host.h"

namespace {
thread_local std::string g_last_error;
}

void orbgpu_set_last_error(const char* msg, const char* file, int line) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "%s (%s:%d)", msg, file, line);
    g_last_error = buf;
}

extern "C" const char* orbgpu_last_error(void) { return g_last_error.c_str(); }
extern "C" int orbgpu_version(void) { return 1; }

cudaError_t orbgpu::allow_max_dynamic_smem(const void* kernel) {
    static std::mutex mu;
    static std::set<std::pair<int, const void*>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (done.count({dev, kernel})) return cudaSuccess;
    int optin = 0;
    cudaFuncAttributes fa;
    if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess ||
        (e = cudaFuncGetAttributes(&fa, kernel)) != cudaSuccess)
        return e;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    if (e == cudaSuccess) done.insert({dev, kernel});
    return e;
}

static std::atomic<int> g_fail_allocs{0};
cudaError_t orbgpu::dev_malloc(void** p, size_t bytes) {
    int n = g_fail_allocs.load();
    while (n > 0)
        if (g_fail_allocs.compare_exchange_weak(n, n - 1)) return cudaErrorMemoryAllocation;
    return cudaMalloc(p, bytes);
}

// Test hook; see orbgpu_ext.h.
extern "C" int orbgpu_debug_fail_allocations(int count) {
    if (count < 0) return ORBGPU_ERR_BAD_ARG;
    g_fail_allocs.store(count);
    return ORBGPU_OK;
}

namespace orbgpu {
static Tunables g_tunables;
static std::atomic<int> g_tune_gen{0};
const Tunables& tunables() { return g_tunables; }
int tune_generation() { return g_tune_gen.load(); }
}  // namespace orbgpu

// Autotuner parameters; see orbgpu_ext.h.
extern "C" int orbgpu_tune_set(const char* name, long long value) {
    if (!name) return ORBGPU_ERR_BAD_ARG;
    orbgpu::Tunables& t = orbgpu::g_tunables;
    const std::string n(name);
    if (n == "resize_rows" && (value == 8 || value == 22 || value == 36 || value == 64)) t.resize_rows = (int)value;
    else if (n == "fast_cells_per_block" && (value == 1 || value == 2 || value == 4))
        t.fast_cells_per_block = (int)value;
    else if (n == "describe_group" && (value == 1 || value == 2 || value == 4))
        t.describe_group = (int)value;
    else if (n == "describe_depth" && (value == 2 || value == 4)) t.describe_depth = (int)value;
    else if (n == "describe_task" && (value == 0 || value == 8 || value == 16 || value == 32))
        t.describe_task = (int)value;
    else if (n == "fast_chunk" && (value == 0 || value == 1 || value == 2 || value == 4)) t.fast_chunk = (int)value;
    else if (n == "strip_rows_small" && (value == 0 || value == 8)) t.strip_rows_small = (int)value;
    else if (n == "knn_tc_min_pairs" && value >= 0) t.knn_tc_min_pairs = value;
    else {
        orbgpu_set_last_error("unknown tuning parameter or value", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    orbgpu::g_tune_gen++;
    return ORBGPU_OK;
}

extern "C" int orbgpu_tune_get(const char* name, long long* value) {
    if (!name || !value) return ORBGPU_ERR_BAD_ARG;
    const orbgpu::Tunables& t = orbgpu::g_tunables;
    const std::string n(name);
    if (n == "resize_rows") *value = t.resize_rows;
    else if (n == "fast_cells_per_block") *value = t.fast_cells_per_block;
    else if (n == "describe_group") *value = t.describe_group;
    else if (n == "describe_depth") *value = t.describe_depth;
    else if (n == "describe_task") *value = t.describe_task;
    else if (n == "fast_chunk") *value = t.fast_chunk;
    else if (n == "strip_rows_small") *value = t.strip_rows_small;
    else if (n == "knn_tc_min_pairs") *value = t.knn_tc_min_pairs;
    else return ORBGPU_ERR_BAD_ARG;
    return ORBGPU_OK;
}

namespace orbgpu {

// ---------------------------------------------------------------- tables
// ORBextractor::ORBextractor, src/ORBextractor.cc:469-571.
ExtractorTables make_tables(int nfeatures, float scale_factor, int nlevels) {
    ExtractorTables t;
    t.nlevels = nlevels;
    const double sf = (double)scale_factor;  // scaleFactor is a double member
    t.scale.assign(nlevels, 1.0f);
    t.sigma2.assign(nlevels, 1.0f);
    for (int i = 1; i < nlevels; i++) {
        t.scale[i] = (float)(t.scale[i - 1] * sf);
        t.sigma2[i] = t.scale[i] * t.scale[i];
    }
    t.inv_scale.resize(nlevels);
    t.inv_sigma2.resize(nlevels);
    for (int i = 0; i < nlevels; i++) {
        t.inv_scale[i] = 1.0f / t.scale[i];
        t.inv_sigma2[i] = 1.0f / t.sigma2[i];
    }
    t.nfeat.assign(nlevels, 0);
    const float factor = (float)(1.0f / sf);
    float per_scale = nfeatures * (1 - factor) / (1 - (float)std::pow((double)factor, (double)nlevels));
    int sum = 0;
    for (int l = 0; l < nlevels - 1; l++) {
        t.nfeat[l] = (int)std::lrint(per_scale);
        sum += t.nfeat[l];
        per_scale *= factor;
    }
    t.nfeat[nlevels - 1] = std::max(nfeatures - sum, 0);
    const int hp = ORBGPU_HALF_PATCH;
    const int vmax = (int)std::floor(hp * std::sqrt(2.f) / 2 + 1);
    const int vmin = (int)std::ceil(hp * std::sqrt(2.f) / 2);
    const double hp2 = hp * hp;
    for (int v = 0; v <= vmax; ++v) t.umax[v] = (int)std::lrint(std::sqrt(hp2 - v * v));
    for (int v = hp, v0 = 0; v >= vmin; --v) {
        while (t.umax[v0] == t.umax[v0 + 1]) ++v0;
        t.umax[v] = v0;
        ++v0;
    }
    // getGaussianKernel(7, 2, CV_32F) in 8-bit fixed point
    {
        float cf[7];
        double s = 0;
        for (int i = 0; i < 7; i++) {
            const double x = i - 3.0;
            cf[i] = (float)std::exp(-0.125 * x * x);
            s += cf[i];
        }
        s = 1. / s;
        for (int i = 0; i < 7; i++) cf[i] = (float)(cf[i] * s);
        for (int i = 0; i < 7; i++) t.taps[i] = (int)std::lrint(cf[i] * 256.f);
    }
    return t;
}

static inline short sat_short_round(float v) {
    long r = std::lrint(v);
    return (short)std::min(32767L, std::max(-32768L, r));
}
static inline int floor_f(float v) {
    int i = (int)v;
    return i - (i > v);
}

// cv::resize INTER_LINEAR coefficient tables (the fixed-point path).
bool resize_tables(int sw, int sh, int dw, int dh, int* xofs, short* xalpha, int* yofs, short* ybeta) {
    const double scale_x = 1. / ((double)dw / sw), scale_y = 1. / ((double)dh / sh);
    int xmax = dw;
    for (int dx = 0; dx < dw; dx++) {
        float fx = (float)((dx + 0.5) * scale_x - 0.5);
        int sx = floor_f(fx);
        fx -= sx;
        if (sx < 0) { fx = 0.f; sx = 0; }
        if (sx + 1 >= sw) {
            if (dx < xmax) xmax = dx;
            if (sx >= sw - 1) { fx = 0.f; sx = sw - 1; }
        }
        xofs[dx] = sx;
        xalpha[2 * dx] = sat_short_round((1.f - fx) * 2048);
        xalpha[2 * dx + 1] = sat_short_round(fx * 2048);
    }
    // past xmax the horizontal pass uses the left sample alone (weight 2048)
    for (int dx = xmax; dx < dw; dx++) {
        xalpha[2 * dx] = 2048;
        xalpha[2 * dx + 1] = 0;
    }
    for (int dy = 0; dy < dh; dy++) {
        float fy = (float)((dy + 0.5) * scale_y - 0.5);
        int sy = floor_f(fy);
        fy -= sy;
        yofs[dy] = sy;
        ybeta[2 * dy] = sat_short_round((1.f - fy) * 2048);
        ybeta[2 * dy + 1] = sat_short_round(fy * 2048);
    }
    auto fits = [](const short* wt, int n) {
        for (int i = 0; i < n; i++)
            if (wt[2 * i] < 0 || wt[2 * i + 1] < 0 || wt[2 * i] + wt[2 * i + 1] > 2049) return false;
        return true;
    };
    return fits(xalpha, dw) && fits(ybeta, dh);
}

// Level geometry of one image (src/ORBextractor.cc:1037-1063, 1661-1663).
int level_geometry(const ExtractorTables& t, int w, int h, std::vector<LevelGeom>& g) {
    g.resize(t.nlevels);
    for (int l = 0; l < t.nlevels; l++) {
        LevelGeom& L = g[l];
        L.w = (int)std::lrint((float)w * t.inv_scale[l]);
        L.h = (int)std::lrint((float)h * t.inv_scale[l]);
        if (L.w < 1 || L.h < 1) return ORBGPU_ERR_BAD_ARG;
        L.pitch = (L.w + 63) & ~63;
        const int minB = ORBGPU_EDGE_THRESHOLD - 3;
        L.maxBorderX = L.w - ORBGPU_EDGE_THRESHOLD + 3;
        L.maxBorderY = L.h - ORBGPU_EDGE_THRESHOLD + 3;
        const float width = (float)(L.maxBorderX - minB), height = (float)(L.maxBorderY - minB);
        L.nCols = (int)(width / 30.f);
        L.nRows = (int)(height / 30.f);
        if (L.nCols <= 0 || L.nRows <= 0 || width <= 0 || height <= 0) {
            // no cell fits: the level yields no keypoints
            L.nCols = L.nRows = 0;
            L.wCell = L.hCell = 0;
            L.nIni = 0;
            L.cell_cap = 0;
        } else {
            L.wCell = (int)std::ceil(width / L.nCols);
            L.hCell = (int)std::ceil(height / L.nRows);
            L.nIni = (int)std::round(static_cast<float>(L.maxBorderX - minB) / (float)(L.maxBorderY - minB));
            // DistributeOctTree would index an empty vector (aspect below 0.5)
            if (L.nIni < 1 || L.nIni > 64) return ORBGPU_ERR_BAD_ARG;
            L.cell_cap = ((L.wCell + 1) / 2) * ((L.hCell + 1) / 2);
            if (L.wCell + 6 > 72 || L.hCell + 6 > 72) return ORBGPU_ERR_BAD_ARG;
        }
        L.ncells = L.nCols * L.nRows;
        L.cand_cap = L.ncells * L.cell_cap;
        L.nfeat = t.nfeat[l];
        L.node_cap = std::max(L.nfeat + 8, 4 * L.nIni + 8);
        L.node_cap = (L.node_cap + 31) & ~31;
        if (L.node_cap > 60000) return ORBGPU_ERR_BAD_ARG;
    }
    return ORBGPU_OK;
}

// ---------------------------------------------------------------- arena
size_t FrameLayout::plan(const std::vector<LevelGeom>& g, size_t base) {
    size_t off = base;
    auto take = [&](size_t bytes) {
        off = (off + 255) & ~(size_t)255;
        size_t r = off;
        off += bytes;
        return r;
    };
    lv.resize(g.size());
    for (size_t l = 0; l < g.size(); l++) {
        const LevelGeom& L = g[l];
        LevelOffsets& o = lv[l];
        o.pyr = take((size_t)L.pitch * L.h);
        o.blur = take((size_t)L.pitch * L.h);
        o.xofs = take(sizeof(int) * L.w);
        o.xalpha = take(sizeof(short) * 2 * L.w);
        o.yofs = take(sizeof(int) * L.h);
        o.ybeta = take(sizeof(short) * 2 * L.h);
        o.cbits = take((size_t)(L.pitch / 8) * L.h);
        o.slots = take(sizeof(uint32_t) * std::max(1, L.cand_cap));
        o.cell_count = take(sizeof(int) * std::max(1, L.ncells));
        o.cand = take(sizeof(uint32_t) * std::max(1, L.cand_cap));
        o.node_of = take(sizeof(int) * std::max(1, L.cand_cap));
        o.quad = take(std::max(1, L.cand_cap));
        o.nodes_a = take(sizeof(DNode) * L.node_cap);
        o.nodes_b = take(sizeof(DNode) * L.node_cap);
        o.cnt4 = take(sizeof(int4) * L.node_cap);
        o.childpos = take(sizeof(int4) * L.node_cap);
        o.aux0 = take(sizeof(int) * L.node_cap);
        o.aux1 = take(sizeof(int) * L.node_cap);
        o.aux2 = take(sizeof(int) * L.node_cap);
        o.best = take(sizeof(uint32_t) * L.node_cap);
        o.kept = take(sizeof(uint32_t) * L.node_cap);
    }
    level_counts = take(sizeof(int) * 16);
    frame_total = take(sizeof(int) * 4);
    patch_maps = take((size_t)3 * ORBGPU_TMAP_BYTES * g.size());
    bytes = off - base;
    return off;
}

void fill_descs(const std::vector<LevelGeom>& g, const ExtractorTables& t, const FrameLayout& lay, uint8_t* arena,
                int frame, int ini_th, int min_th, int out_base, int out_cap, LevelDesc* out) {
    for (size_t l = 0; l < g.size(); l++) {
        const LevelGeom& L = g[l];
        const LevelOffsets& o = lay.lv[l];
        LevelDesc& d = out[l];
        std::memset(&d, 0, sizeof(d));
        if (l > 0) {
            const LevelGeom& P = g[l - 1];
            d.src = arena + lay.lv[l - 1].pyr;
            d.sw = P.w;
            d.sh = P.h;
            d.spitch = P.pitch;
        }
        d.dst = arena + o.pyr;
        d.blur = arena + o.blur;
        d.w = L.w;
        d.h = L.h;
        d.pitch = L.pitch;
        d.xofs = (const int*)(arena + o.xofs);
        d.xalpha = (const short*)(arena + o.xalpha);
        d.yofs = (const int*)(arena + o.yofs);
        d.ybeta = (const short*)(arena + o.ybeta);
        d.nCols = L.nCols;
        d.nRows = L.nRows;
        d.wCell = L.wCell;
        d.hCell = L.hCell;
        d.maxBorderX = L.maxBorderX;
        d.maxBorderY = L.maxBorderY;
        d.cell_cap = L.cell_cap;
        d.slots = (uint32_t*)(arena + o.slots);
        d.cell_count = (int*)(arena + o.cell_count);
        d.ini_th = ini_th;
        d.min_th = min_th;
        d.cbits = arena + o.cbits;
        d.cbits_stride = L.pitch / 8;
        d.cell_box_w = fast_cell_box_w(L.wCell);
        d.nfeat = L.nfeat;
        d.nIni = L.nIni;
        d.cand_cap = L.cand_cap;
        d.node_cap = L.node_cap;
        d.cand = (uint32_t*)(arena + o.cand);
        d.node_of = (int*)(arena + o.node_of);
        d.quad = arena + o.quad;
        d.nodes_a = arena + o.nodes_a;
        d.nodes_b = arena + o.nodes_b;
        d.cnt4 = (int4*)(arena + o.cnt4);
        d.childpos = (int4*)(arena + o.childpos);
        d.aux0 = (int*)(arena + o.aux0);
        d.aux1 = (int*)(arena + o.aux1);
        d.aux2 = (int*)(arena + o.aux2);
        d.best = (uint32_t*)(arena + o.best);
        d.kept = (uint32_t*)(arena + o.kept);
        d.level_counts = (int*)(arena + lay.level_counts);
        d.kept_count = d.level_counts + l;
        d.level = (int)l;
        d.frame = frame;
        d.scale = t.scale[l];
        d.nlevels = (int)g.size();
        d.out_base = out_base;
        d.out_cap = out_cap;
        d.frame_total = (int*)(arena + lay.frame_total);
        d.tm_level = arena + lay.patch_maps + (size_t)(3 * l) * ORBGPU_TMAP_BYTES;
        d.tm_blur = arena + lay.patch_maps + (size_t)(3 * l + 1) * ORBGPU_TMAP_BYTES;
        d.tm_cell = arena + lay.patch_maps + (size_t)(3 * l + 2) * ORBGPU_TMAP_BYTES;
    }
}

// ---------------------------------------------------------------- patch tensor maps
// k_describe copies each keypoint's patches into shared memory with 2-D
// tensor copies: a DESC_LBOX_W x DESC_LBOX_H box of the level plane
// (IC_Angle) and a DESC_BBOX_W x DESC_BBOX_H box of the blurred plane
// (rBRIEF); k_fast_cells copies each cell's ROI, a fast_cell_box_w(wCell) x
// (hCell + 6) box of the level plane.  The maps span pitch x h bytes of the
// slot's planes (the pitch is a multiple of 64 and the planes start 256-byte
// aligned, as the tensor copy requires); box bytes past the pitch or the last
// row read as zero and are never used.
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, []() {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

int encode_patch_maps(const std::vector<LevelGeom>& g, const FrameLayout& lay, uint8_t* arena,
                      std::vector<uint8_t>& out) {
    static_assert(sizeof(CUtensorMap) == ORBGPU_TMAP_BYTES, "tensor map size");
    auto encode = tensor_map_encoder();
    if (!encode) {
        orbgpu_set_last_error("cuTensorMapEncodeTiled is not available", __FILE__, __LINE__);
        return ORBGPU_ERR_CUDA;
    }
    out.assign((size_t)3 * ORBGPU_TMAP_BYTES * g.size(), 0);
    for (size_t l = 0; l < g.size(); l++) {
        const LevelGeom& L = g[l];
        for (int k = 0; k < 3; k++) {
            // a level lower than the blurred box holds no describable
            // keypoint (they lie EDGE_THRESHOLD >= DESC_BBOX_R rows inside),
            // a level without cells no FAST corner: no maps
            if (k < 2 ? L.h < DESC_BBOX_H : L.ncells == 0) continue;
            uint8_t* base = arena + (k == 1 ? lay.lv[l].blur : lay.lv[l].pyr);
            const cuuint64_t dims[2] = {(cuuint64_t)L.pitch, (cuuint64_t)L.h};
            const cuuint64_t strides[1] = {(cuuint64_t)L.pitch};
            const cuuint32_t box[2] = {k == 0   ? (cuuint32_t)DESC_LBOX_W
                                       : k == 1 ? (cuuint32_t)DESC_BBOX_W
                                                : (cuuint32_t)fast_cell_box_w(L.wCell),
                                       k == 0   ? (cuuint32_t)DESC_LBOX_H
                                       : k == 1 ? (cuuint32_t)DESC_BBOX_H
                                                : (cuuint32_t)(L.hCell + 6)};
            const cuuint32_t estr[2] = {1, 1};
            if (((uintptr_t)base & 15) || (L.pitch & 15) || box[0] > 256 || box[1] > 256) {
                orbgpu_set_last_error("plane or box not valid for tensor copies", __FILE__, __LINE__);
                return ORBGPU_ERR_CUDA;
            }
            CUtensorMap* m = (CUtensorMap*)(out.data() + (size_t)(3 * l + k) * ORBGPU_TMAP_BYTES);
            const CUresult r = encode(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, base, dims, strides, box, estr,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) {
                char msg[96];
                std::snprintf(msg, sizeof(msg), "cuTensorMapEncodeTiled failed (%d)", (int)r);
                orbgpu_set_last_error(msg, __FILE__, __LINE__);
                return ORBGPU_ERR_CUDA;
            }
        }
    }
    return ORBGPU_OK;
}

// ---------------------------------------------------------------- sin/cos exceptions
// The descriptor angle's cos/sin must equal the host C library's
// cosf/sinf (what std::cos(float) / std::sin(float) call in
// computeOrbDescriptor, src/ORBextractor.cc:157).  The device evaluates
// sincos_taylor and corrects the inputs listed in an exception table built
// here from the host library.  The table covers every float in
// [0, 360 * pi/180] and is cached on disk next to the library.
static std::once_flag g_exc_once;
static int g_exc_status = ORBGPU_OK;
static uint32_t* g_exc_dev = nullptr;

int load_sincos_exceptions(const char* path) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return ORBGPU_ERR_BAD_ARG;
    int32_t hdr[4];
    if (std::fread(hdr, sizeof(int32_t), 4, f) != 4 || hdr[0] != 0x4f524258) {
        std::fclose(f);
        return ORBGPU_ERR_BAD_ARG;
    }
    const int cn = hdr[1], sn = hdr[2];
    std::vector<uint32_t> buf((size_t)2 * (cn + sn));
    if (std::fread(buf.data(), sizeof(uint32_t), buf.size(), f) != buf.size()) {
        std::fclose(f);
        return ORBGPU_ERR_BAD_ARG;
    }
    std::fclose(f);
    // bucket offsets: first entry of every 4096-wide range of input bits
    const uint32_t hi_bits = 0x40C90FDCu;  // just above 360 * pi / 180 as a float
    const int nb = (int)(hi_bits >> 12) + 1;
    std::vector<uint32_t> bk((size_t)2 * (nb + 1));
    auto fill_buckets = [&](const uint32_t* keys, int n, uint32_t* out) {
        int j = 0;
        for (int b = 0; b <= nb; b++) {
            while (j < n && (keys[j] >> 12) < (uint32_t)b) j++;
            out[b] = (uint32_t)j;
        }
    };
    fill_buckets(buf.data(), cn, bk.data());
    fill_buckets(buf.data() + 2 * cn, sn, bk.data() + nb + 1);
    // sub-bucket offsets: inside bucket b, the entries whose next 6 input
    // bits are below s (64 uint16 per bucket; a bucket holds at most 4096)
    std::vector<uint16_t> sub((size_t)2 * nb * 64, 0);
    auto fill_sub = [&](const uint32_t* keys, int n, uint16_t* out) {
        for (int i = 0; i < n; i++) {
            const uint32_t b = keys[i] >> 12;
            if (b < (uint32_t)nb) out[(size_t)b * 64 + ((keys[i] >> 6) & 63)]++;
        }
        for (size_t b = 0; b < (size_t)nb; b++) {  // counts -> exclusive prefix
            uint16_t run = 0;
            for (int s = 0; s < 64; s++) {
                const uint16_t c = out[b * 64 + s];
                out[b * 64 + s] = run;
                run = (uint16_t)(run + c);
            }
        }
    };
    fill_sub(buf.data(), cn, sub.data());
    fill_sub(buf.data() + 2 * cn, sn, sub.data() + (size_t)nb * 64);
    buf.insert(buf.end(), bk.begin(), bk.end());
    const size_t sub_words = sub.size() / 2;
    const size_t sub_at = buf.size();
    buf.resize(buf.size() + sub_words);
    std::memcpy(&buf[sub_at], sub.data(), sub.size() * sizeof(uint16_t));
    if (cudaMalloc(&g_exc_dev, std::max<size_t>(4, buf.size() * 4)) != cudaSuccess) return ORBGPU_ERR_OOM;
    cudaMemcpy(g_exc_dev, buf.data(), buf.size() * 4, cudaMemcpyHostToDevice);
    const uint32_t* ck = g_exc_dev;
    const float* cv = (const float*)(g_exc_dev + cn);
    const uint32_t* sk = g_exc_dev + 2 * cn;
    const float* sv = (const float*)(g_exc_dev + 2 * cn + sn);
    const int* cb = (const int*)(g_exc_dev + 2 * (cn + sn));
    const int* sb = cb + nb + 1;
    const uint16_t* csub = (const uint16_t*)(g_exc_dev + sub_at);
    const uint16_t* ssub = csub + (size_t)nb * 64;
    set_sincos_exceptions(ck, cv, cn, sk, sv, sn, cb, sb, csub, ssub, nb);
    return ORBGPU_OK;
}

// The constant tables every kernel shares (Gaussian taps, IC_Angle row
// bounds, rBRIEF pattern): the same for every configuration, uploaded once.
static std::once_flag g_const_once;
static int g_const_status = ORBGPU_OK;
int ensure_constants() {
    std::call_once(g_const_once, []() {
        const ExtractorTables t = make_tables(1000, 1.2f, 8);
        upload_constants(0, t.taps, t.umax);
        g_const_status = cudaStreamSynchronize(0) == cudaSuccess ? ORBGPU_OK : ORBGPU_ERR_CUDA;
    });
    return g_const_status;
}

int ensure_sincos_exceptions() {
    std::call_once(g_exc_once, []() {
        const char* p = std::getenv("ORBGPU_SINCOS_TABLE");
        std::string path = p ? p : default_sincos_table_path();
        g_exc_status = load_sincos_exceptions(path.c_str());
        if (g_exc_status != ORBGPU_OK) {
            std::string msg = "sin/cos exception table not found or invalid: " + path;
            orbgpu_set_last_error(msg.c_str(), __FILE__, __LINE__);
        }
    });
    return g_exc_status;
}

}  // namespace orbgpu

using namespace orbgpu;

// Everything that depends on the image size: level geometry, the device
// arena with the resize tables, the work lists.  An extractor keeps the plans
// of the last few sizes it saw, so alternating sizes cost no re-planning.
struct SizePlan {
    int w = -1, h = -1;
    std::vector<LevelGeom> geom;
    FrameLayout layout;
    uint8_t* arena = nullptr;
    int* d_items = nullptr;  // block-range prefix arrays
    std::vector<int> rb_first, rb_count;
    int rows = 22;  // strip rows of the resize / blur launches
    int fast_first = 0, fast_count = 0;
    int max_kept = 0, sort_cap = 0;
    uint64_t last_use = 0;
    int gen = -1;  // tuning generation of the work lists
};

struct orbgpu_extractor {
    int nfeatures, nlevels, ini_th, min_th;
    float scale_factor;
    int max_w, max_h;
    ExtractorTables tables;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // the resize chain of levels 1.. runs on a second stream beside the
    // strips of the levels already resized (ev_level[l]: level l is written)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_level[ORBGPU_MAX_LEVELS] = {};
    std::vector<SizePlan*> plans;
    SizePlan* cur = nullptr;
    uint64_t use_clock = 0;
    // current geometry (mirrors cur)
    int cur_w = -1, cur_h = -1;
    LevelDesc* d_descs = nullptr;
    int* d_status = nullptr;
    // output staging
    orbgpu_keypoint* d_kps = nullptr;
    uint8_t* d_desc = nullptr;
    int out_cap = 0;
    int* h_pinned = nullptr;  // status + counts
};

static void free_plan(SizePlan* p) {
    if (!p) return;
    cudaFree(p->arena);
    cudaFree(p->d_items);
    delete p;
}

static int build_plan(orbgpu_extractor* ex, int w, int h, SizePlan** out) {
    SizePlan* P = new SizePlan();
    int rc = level_geometry(ex->tables, w, h, P->geom);
    if (rc != ORBGPU_OK) {
        delete P;
        orbgpu_set_last_error("image size not supported by the level geometry", __FILE__, __LINE__);
        return rc;
    }
    const std::vector<LevelGeom>& g = P->geom;
    P->layout.plan(g, 0);
    if (dev_malloc(&P->arena, P->layout.bytes) != cudaSuccess) {
        delete P;
        orbgpu_set_last_error("device allocation failed", __FILE__, __LINE__);
        return ORBGPU_ERR_OOM;
    }
    // resize tables, level by level
    for (size_t l = 1; l < g.size(); l++) {
        const LevelOffsets& o = P->layout.lv[l];
        const size_t lo = o.xofs, hi = o.ybeta + sizeof(short) * 2 * g[l].h;
        std::vector<uint8_t> host(hi - lo, 0);
        if (!resize_tables(g[l - 1].w, g[l - 1].h, g[l].w, g[l].h, (int*)&host[o.xofs - lo],
                           (short*)&host[o.xalpha - lo], (int*)&host[o.yofs - lo], (short*)&host[o.ybeta - lo])) {
            free_plan(P);
            orbgpu_set_last_error("resize weights out of range", __FILE__, __LINE__);
            return ORBGPU_ERR_BAD_ARG;
        }
        if (cudaMemcpy(P->arena + lo, host.data(), hi - lo, cudaMemcpyHostToDevice) != cudaSuccess) {
            free_plan(P);
            return ORBGPU_ERR_CUDA;
        }
    }
    // the descriptor kernel's tensor maps of this arena
    std::vector<uint8_t> maps;
    rc = encode_patch_maps(g, P->layout, P->arena, maps);
    if (rc == ORBGPU_OK &&
        cudaMemcpy(P->arena + P->layout.patch_maps, maps.data(), maps.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        rc = ORBGPU_ERR_CUDA;
    if (rc != ORBGPU_OK) {
        free_plan(P);
        return rc;
    }
    // block ranges: per level the resize/blur tiles (one entry), then the
    // cells of every level (one entry per level)
    std::vector<int> pre;
    P->rb_first.assign(g.size(), 0);
    P->rb_count.assign(g.size(), 0);
    P->rows = strip_rows((long)g[0].w * g[0].h);
    for (size_t l = 0; l < g.size(); l++) {
        P->rb_first[l] = (int)pre.size();
        const int tiles = resize_blur_tiles(g[l].w, g[l].h, P->rows);
        pre.push_back(0);
        pre.push_back(tiles);
        P->rb_count[l] = tiles;
    }
    P->fast_first = (int)pre.size();
    int acc = 0;
    for (size_t l = 0; l < g.size(); l++) {
        pre.push_back(acc);
        acc += g[l].ncells;
    }
    pre.push_back(acc);
    P->fast_count = acc;
    if (dev_malloc(&P->d_items, pre.size() * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(P->d_items, pre.data(), pre.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
        free_plan(P);
        return ORBGPU_ERR_OOM;
    }
    P->max_kept = 0;
    P->sort_cap = 1;
    for (auto& L : g) {
        P->max_kept = std::max(P->max_kept, L.node_cap);
        while (P->sort_cap < L.node_cap) P->sort_cap <<= 1;
    }
    P->w = w;
    P->h = h;
    *out = P;
    return ORBGPU_OK;
}

static int setup_geometry(orbgpu_extractor* ex, int w, int h) {
    ex->use_clock++;
    if (ex->cur && ex->cur->w == w && ex->cur->h == h && ex->cur->gen == tune_generation()) {
        ex->cur->last_use = ex->use_clock;
        return ORBGPU_OK;
    }
    // work lists counted for other launch shapes are rebuilt
    bool stale = false;
    for (SizePlan* p : ex->plans) stale |= p->gen != tune_generation();
    if (stale) {
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(ex->stream));
        for (SizePlan* p : ex->plans) free_plan(p);
        ex->plans.clear();
        ex->cur = nullptr;
    }
    SizePlan* found = nullptr;
    for (SizePlan* p : ex->plans)
        if (p->w == w && p->h == h) found = p;
    if (!found) {
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(ex->stream));
        if (ex->plans.size() >= 8) {  // drop the least recently used plan
            auto it = std::min_element(ex->plans.begin(), ex->plans.end(),
                                       [](SizePlan* a, SizePlan* b) { return a->last_use < b->last_use; });
            free_plan(*it);
            ex->plans.erase(it);
        }
        int rc = build_plan(ex, w, h, &found);
        if (rc != ORBGPU_OK) return rc;
        found->gen = tune_generation();
        ex->plans.push_back(found);
    }
    found->last_use = ex->use_clock;
    ex->cur = found;
    ex->cur_w = w;
    ex->cur_h = h;
    return ORBGPU_OK;
}

static int ensure_out(orbgpu_extractor* ex, int cap) {
    if (cap <= ex->out_cap) return ORBGPU_OK;
    if (ex->d_kps) cudaFree(ex->d_kps);
    if (ex->d_desc) cudaFree(ex->d_desc);
    ex->d_kps = nullptr;
    ex->d_desc = nullptr;
    ORBGPU_CUDA_TRY(cudaMalloc(&ex->d_kps, sizeof(orbgpu_keypoint) * (size_t)cap));
    ORBGPU_CUDA_TRY(cudaMalloc(&ex->d_desc, 32 * (size_t)cap));
    ex->out_cap = cap;
    return ORBGPU_OK;
}

extern "C" int orbgpu_extractor_create(int nfeatures, float scale_factor, int nlevels, int ini_th_fast,
                                       int min_th_fast, int max_width, int max_height, void* stream,
                                       orbgpu_extractor** out) {
    if (!out || nfeatures < 0 || nlevels < 1 || nlevels > ORBGPU_MAX_LEVELS || !(scale_factor > 1.0f) ||
        max_width < 0 || max_height < 0 || max_width > ORBGPU_MAX_DIM || max_height > ORBGPU_MAX_DIM) {
        orbgpu_set_last_error("invalid extractor parameters", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    int dev = 0;
    ORBGPU_CUDA_TRY(cudaGetDevice(&dev));
    int rc = ensure_sincos_exceptions();
    if (rc != ORBGPU_OK) return rc;
    orbgpu_extractor* ex = new orbgpu_extractor();
    ex->nfeatures = nfeatures;
    ex->scale_factor = scale_factor;
    ex->nlevels = nlevels;
    ex->ini_th = ini_th_fast;
    ex->min_th = min_th_fast;
    ex->max_w = max_width;
    ex->max_h = max_height;
    ex->tables = make_tables(nfeatures, scale_factor, nlevels);
    if (stream) ex->stream = (cudaStream_t)stream;
    else {
        cudaError_t e = cudaStreamCreateWithFlags(&ex->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete ex;
            orbgpu_set_last_error(cudaGetErrorString(e), __FILE__, __LINE__);
            return ORBGPU_ERR_CUDA;
        }
        ex->own_stream = true;
    }
    bool side_ok = cudaStreamCreateWithFlags(&ex->side, cudaStreamNonBlocking) == cudaSuccess &&
                   cudaEventCreateWithFlags(&ex->ev_fork, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 1; i < ORBGPU_MAX_LEVELS && side_ok; i++)
        side_ok = cudaEventCreateWithFlags(&ex->ev_level[i], cudaEventDisableTiming) == cudaSuccess;
    if (!side_ok) {
        orbgpu_set_last_error("stream or event creation failed", __FILE__, __LINE__);
        orbgpu_extractor_destroy(ex);
        return ORBGPU_ERR_CUDA;
    }
    cudaError_t e1 = cudaMalloc(&ex->d_descs, sizeof(LevelDesc) * ORBGPU_MAX_LEVELS);
    cudaError_t e2 = cudaMalloc(&ex->d_status, sizeof(int) * 4);
    cudaError_t e3 = cudaMallocHost(&ex->h_pinned, sizeof(int) * 32);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
        orbgpu_set_last_error("device allocation failed", __FILE__, __LINE__);
        orbgpu_extractor_destroy(ex);
        return ORBGPU_ERR_OOM;
    }
    rc = ensure_constants();
    if (rc != ORBGPU_OK) {
        orbgpu_extractor_destroy(ex);
        return rc;
    }
    if (max_width > 0 && max_height > 0) {
        rc = setup_geometry(ex, max_width, max_height);
        if (rc != ORBGPU_OK) {
            orbgpu_extractor_destroy(ex);
            return rc;
        }
    }
    *out = ex;
    return ORBGPU_OK;
}

extern "C" int orbgpu_extractor_destroy(orbgpu_extractor* ex) {
    if (!ex) return ORBGPU_OK;
    if (ex->stream) cudaStreamSynchronize(ex->stream);
    if (ex->side) cudaStreamSynchronize(ex->side);
    for (int i = 0; i < ORBGPU_MAX_LEVELS; i++)
        if (ex->ev_level[i]) cudaEventDestroy(ex->ev_level[i]);
    if (ex->ev_fork) cudaEventDestroy(ex->ev_fork);
    if (ex->side) cudaStreamDestroy(ex->side);
    for (SizePlan* p : ex->plans) free_plan(p);
    ex->plans.clear();
    cudaFree(ex->d_descs);
    cudaFree(ex->d_status);
    cudaFree(ex->d_kps);
    cudaFree(ex->d_desc);
    cudaFreeHost(ex->h_pinned);
    if (ex->own_stream) cudaStreamDestroy(ex->stream);
    delete ex;
    return ORBGPU_OK;
}

extern "C" int orbgpu_extract(orbgpu_extractor* ex, const uint8_t* image, int width, int height, size_t step,
                              int image_mem, orbgpu_keypoint* keypoints, uint8_t* descriptors, int capacity,
                              int out_mem, int* n_keypoints) {
    if (!ex || !n_keypoints) {
        orbgpu_set_last_error("null handle or count pointer", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    *n_keypoints = 0;
    // an empty image returns without output (src/ORBextractor.cc:1537)
    if (image == nullptr || width == 0 || height == 0) return ORBGPU_OK;
    if (width < 0 || height < 0 || width > ORBGPU_MAX_DIM || height > ORBGPU_MAX_DIM || step < (size_t)width ||
        capacity < 0 || (capacity > 0 && (!keypoints || !descriptors)) ||
        (ex->max_w > 0 && (width > ex->max_w || height > ex->max_h))) {
        orbgpu_set_last_error("invalid image or output arguments", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    int rc = setup_geometry(ex, width, height);
    if (rc != ORBGPU_OK) return rc;
    const SizePlan& P = *ex->cur;
    const std::vector<LevelGeom>& g = P.geom;
    const int nl = (int)g.size();
    // descriptors of this call (outputs go to the caller's device arrays or
    // to the staging buffers)
    orbgpu_keypoint* okps;
    uint8_t* odesc;
    if (out_mem == ORBGPU_MEM_DEVICE) {
        okps = keypoints;
        odesc = descriptors;
    } else {
        rc = ensure_out(ex, std::max(capacity, 1));
        if (rc != ORBGPU_OK) return rc;
        okps = ex->d_kps;
        odesc = ex->d_desc;
    }
    LevelDesc hd[ORBGPU_MAX_LEVELS];
    fill_descs(g, ex->tables, P.layout, P.arena, 0, ex->ini_th, ex->min_th, 0, capacity, hd);
    cudaStream_t st = ex->stream;
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(ex->d_descs, hd, sizeof(LevelDesc) * nl, cudaMemcpyHostToDevice, st));
    ORBGPU_CUDA_TRY(cudaMemsetAsync(ex->d_status, 0, sizeof(int) * 4, st));
    // level 0 = the image
    ORBGPU_CUDA_TRY(cudaMemcpy2DAsync(hd[0].dst, hd[0].pitch, image, step, width, height,
                                      image_mem == ORBGPU_MEM_DEVICE ? cudaMemcpyDeviceToDevice
                                                                     : cudaMemcpyHostToDevice,
                                      st));
    // levels 1.. resized in a chain on the side stream while the strips of
    // the levels already resized run on the extractor's stream
    ORBGPU_CUDA_TRY(cudaEventRecord(ex->ev_fork, st));
    ORBGPU_CUDA_TRY(cudaStreamWaitEvent(ex->side, ex->ev_fork, 0));
    for (int l = 1; l < nl; l++) {
        launch_level_resize(ex->d_descs, RangeMap{P.d_items + P.rb_first[l], 1, l, 0}, P.rb_count[l], P.rows, ex->side);
        ORBGPU_CUDA_TRY(cudaEventRecord(ex->ev_level[l], ex->side));
    }
    for (int l = 0; l < nl; l++) {
        if (l > 0) ORBGPU_CUDA_TRY(cudaStreamWaitEvent(st, ex->ev_level[l], 0));
        launch_level_strip(ex->d_descs, RangeMap{P.d_items + P.rb_first[l], 1, l, 0}, P.rb_count[l], P.rows, st);
    }
    int mwc = 1, mhc = 1, mbox = 0;
    for (const LevelGeom& L : g) {
        mwc = std::max(mwc, L.wCell);
        mhc = std::max(mhc, L.hCell);
        if (L.ncells > 0) mbox = std::max(mbox, fast_cell_box_w(L.wCell) * (L.hCell + 6));
    }
    launch_fast(ex->d_descs, RangeMap{P.d_items + P.fast_first, nl, 0, 1}, P.fast_count, ex->d_status, mwc, mhc, mbox,
                st);
    launch_distribute(ex->d_descs, nl, P.sort_cap, P.max_kept, ex->d_status, st);
    launch_describe(ex->d_descs, nl, P.max_kept, okps, odesc, ex->d_status, st);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(ex->h_pinned, ex->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(ex->h_pinned + 4, hd[0].frame_total, sizeof(int), cudaMemcpyDeviceToHost, st));
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
    const int status = ex->h_pinned[0];
    const int total = ex->h_pinned[4];
    *n_keypoints = total;
    if (status & ~16) {
        char msg[128];
        std::snprintf(msg, sizeof(msg), "device-side capacity check failed (status 0x%x)", status);
        orbgpu_set_last_error(msg, __FILE__, __LINE__);
        return ORBGPU_ERR_CUDA;
    }
    if (total > capacity) {
        orbgpu_set_last_error("output capacity too small", __FILE__, __LINE__);
        return ORBGPU_ERR_CAPACITY;
    }
    if (out_mem != ORBGPU_MEM_DEVICE && total > 0) {
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(keypoints, okps, sizeof(orbgpu_keypoint) * total, cudaMemcpyDeviceToHost, st));
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(descriptors, odesc, 32 * (size_t)total, cudaMemcpyDeviceToHost, st));
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
    }
    return ORBGPU_OK;
}

extern "C" int orbgpu_extractor_tables(const orbgpu_extractor* ex, int* nlevels, float* scale_factors,
                                       float* inv_scale_factors, float* sigma2, float* inv_sigma2,
                                       int* features_per_level) {
    if (!ex) return ORBGPU_ERR_BAD_ARG;
    const ExtractorTables& t = ex->tables;
    if (nlevels) *nlevels = t.nlevels;
    for (int l = 0; l < t.nlevels; l++) {
        if (scale_factors) scale_factors[l] = t.scale[l];
        if (inv_scale_factors) inv_scale_factors[l] = t.inv_scale[l];
        if (sigma2) sigma2[l] = t.sigma2[l];
        if (inv_sigma2) inv_sigma2[l] = t.inv_sigma2[l];
        if (features_per_level) features_per_level[l] = t.nfeat[l];
    }
    return ORBGPU_OK;
}

extern "C" int orbgpu_extractor_pyramid_level(const orbgpu_extractor* ex, int level, const uint8_t** dev_ptr,
                                              int* width, int* height, size_t* pitch) {
    if (!ex || level < 0 || level >= ex->nlevels || ex->cur_w < 0) return ORBGPU_ERR_BAD_ARG;
    const LevelGeom& L = ex->cur->geom[level];
    if (dev_ptr) *dev_ptr = ex->cur->arena + ex->cur->layout.lv[level].pyr;
    if (width) *width = L.w;
    if (height) *height = L.h;
    if (pitch) *pitch = L.pitch;
    return ORBGPU_OK;
}

extern "C" void* orbgpu_extractor_stream(const orbgpu_extractor* ex) { return ex ? (void*)ex->stream : nullptr; }

// blurred level accessor used by the kernel tests
extern "C" int orbgpu_extractor_blurred_level(const orbgpu_extractor* ex, int level, const uint8_t** dev_ptr) {
    if (!ex || level < 0 || level >= ex->nlevels || ex->cur_w < 0) return ORBGPU_ERR_BAD_ARG;
    *dev_ptr = ex->cur->arena + ex->cur->layout.lv[level].blur;
    return ORBGPU_OK;
}

// Synchronous device-to-host copy of library-owned buffers (tests, tools).
extern "C" int orbgpu_copy_to_host(void* dst, const void* src, size_t bytes) {
    ORBGPU_CUDA_TRY(cudaDeviceSynchronize());
    ORBGPU_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return ORBGPU_OK;
}

// Internal per-level arrays of the last extraction, for stage-level tests:
// what = 0 cell counts (ncells ints), 1 cell slots (ncells*cell_cap uint32),
// 2 distributed keypoints (node_cap uint32), 3 geometry (8 ints: nCols,
// nRows, wCell, hCell, cell_cap, nIni, node_cap, level count).
extern "C" int orbgpu_extractor_debug_level(const orbgpu_extractor* ex, int level, int what, void* dst, size_t cap) {
    if (!ex || level < 0 || level >= ex->nlevels || ex->cur_w < 0) return ORBGPU_ERR_BAD_ARG;
    const LevelGeom& L = ex->cur->geom[level];
    const LevelOffsets& o = ex->cur->layout.lv[level];
    uint8_t* arena = ex->cur->arena;
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(ex->stream));
    size_t bytes = 0;
    const void* src = nullptr;
    if (what == 0) { src = arena + o.cell_count; bytes = sizeof(int) * L.ncells; }
    else if (what == 1) { src = arena + o.slots; bytes = sizeof(uint32_t) * (size_t)L.cand_cap; }
    else if (what == 2) { src = arena + o.kept; bytes = sizeof(uint32_t) * (size_t)L.node_cap; }
    else if (what == 3) {
        int cnt = 0;
        ORBGPU_CUDA_TRY(cudaMemcpy(&cnt, arena + ex->cur->layout.level_counts + sizeof(int) * level, sizeof(int),
                                   cudaMemcpyDeviceToHost));
        const int g[8] = {L.nCols, L.nRows, L.wCell, L.hCell, L.cell_cap, L.nIni, L.node_cap, cnt};
        if (cap < sizeof(g)) return ORBGPU_ERR_CAPACITY;
        std::memcpy(dst, g, sizeof(g));
        return ORBGPU_OK;
    } else return ORBGPU_ERR_BAD_ARG;
    if (bytes > cap) return ORBGPU_ERR_CAPACITY;
    ORBGPU_CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return ORBGPU_OK;
}
