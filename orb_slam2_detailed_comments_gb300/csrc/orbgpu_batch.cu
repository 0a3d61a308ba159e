// orbgpu_batch.cu -- batched extraction and projection matching over a
// ragged list of frames.
//
// Frames of different sizes and feature budgets go through the same stage
// kernels as the per-frame path, but each stage is ONE launch over the work
// items of every frame: 8 resize/blur launches (one per level), one FAST
// launch over all cells of all levels of all frames, one DistributeOctTree
// launch over all (frame, level) pairs, one describe launch.  The launch
// sequence for a given frame list is captured once in a CUDA graph and
// replayed while the list repeats.  Images are gathered from the caller's
// pointers into the level-0 planes by one kernel, so the graph does not
// depend on where the images live.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "orbgpu_host.h"

namespace orbgpu {

struct ImageSrc {
    const uint8_t* ptr;
    int w, h;
    int step;
    uint8_t* dst;
    int pitch;
};

// Copies every frame's image into its level-0 plane: one block row per
// frame row band.
__global__ void k_gather_images(const ImageSrc* src, int nframes) {
    const int f = blockIdx.y;
    if (f >= nframes) return;
    const ImageSrc s = src[f];
    const int rows_per_block = 8;
    const int y0 = blockIdx.x * rows_per_block;
    if (y0 >= s.h) return;
    const int y1 = min(s.h, y0 + rows_per_block);
    for (int y = y0; y < y1; y++) {
        const uint8_t* a = s.ptr + (size_t)y * s.step;
        uint8_t* b = s.dst + (size_t)y * s.pitch;
        for (int x = threadIdx.x; x < s.w; x += blockDim.x) b[x] = a[x];
    }
}

}  // namespace orbgpu

using namespace orbgpu;

struct orbgpu_batch {
    int max_frames, max_w, max_h, max_nf;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // plan of the last frame list
    std::vector<int> sig;
    int nframes = 0, nlevels = 0;
    std::vector<ExtractorTables> tables;  // per frame
    std::vector<std::vector<LevelGeom>> geoms;
    std::vector<FrameLayout> layouts;
    std::vector<size_t> frame_base;
    uint8_t* arena = nullptr;
    size_t arena_bytes = 0;
    LevelDesc* d_descs = nullptr;
    size_t descs_cap = 0;
    WorkItem* d_items = nullptr;
    size_t items_cap = 0;
    std::vector<int> rb_first, rb_count;
    int fast_first = 0, fast_count = 0;
    int max_kept = 0, sort_cap = 0;
    ImageSrc* d_src = nullptr;
    ImageSrc* h_src = nullptr;  // pinned
    int src_cap = 0;
    int* d_status = nullptr;
    int* d_totals = nullptr;  // per frame
    int* h_pinned = nullptr;
    int ndesc = 0;
    cudaGraphExec_t graph = nullptr;
    orbgpu_keypoint* graph_kps = nullptr;
    uint8_t* graph_desc = nullptr;
    int graph_cap = 0;
    int launches_per_run = 0;
};

static void destroy_graph(orbgpu_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
}

extern "C" int orbgpu_batch_create(int max_frames, int max_width, int max_height, int max_nfeatures, void* stream,
                                   orbgpu_batch** out) {
    if (!out || max_frames < 1 || max_width < 1 || max_height < 1 || max_width > ORBGPU_MAX_DIM ||
        max_height > ORBGPU_MAX_DIM || max_nfeatures < 1)
        return ORBGPU_ERR_BAD_ARG;
    int dev;
    ORBGPU_CUDA_TRY(cudaGetDevice(&dev));
    int rc = ensure_sincos_exceptions();
    if (rc != ORBGPU_OK) return rc;
    orbgpu_batch* b = new orbgpu_batch();
    b->max_frames = max_frames;
    b->max_w = max_width;
    b->max_h = max_height;
    b->max_nf = max_nfeatures;
    if (stream) b->stream = (cudaStream_t)stream;
    else {
        if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete b;
            return ORBGPU_ERR_CUDA;
        }
        b->own_stream = true;
    }
    if (cudaMalloc(&b->d_status, sizeof(int) * 4) != cudaSuccess ||
        cudaMalloc(&b->d_totals, sizeof(int) * max_frames) != cudaSuccess ||
        cudaMallocHost(&b->h_pinned, sizeof(int) * (8 + max_frames)) != cudaSuccess ||
        cudaMalloc(&b->d_src, sizeof(ImageSrc) * max_frames) != cudaSuccess ||
        cudaMallocHost(&b->h_src, sizeof(ImageSrc) * max_frames) != cudaSuccess) {
        orbgpu_batch_destroy(b);
        return ORBGPU_ERR_OOM;
    }
    b->src_cap = max_frames;
    *out = b;
    return ORBGPU_OK;
}

extern "C" int orbgpu_batch_destroy(orbgpu_batch* b) {
    if (!b) return ORBGPU_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    destroy_graph(b);
    cudaFree(b->arena);
    cudaFree(b->d_descs);
    cudaFree(b->d_items);
    cudaFree(b->d_status);
    cudaFree(b->d_totals);
    cudaFree(b->d_src);
    cudaFreeHost(b->h_src);
    cudaFreeHost(b->h_pinned);
    if (b->own_stream) cudaStreamDestroy(b->stream);
    delete b;
    return ORBGPU_OK;
}

// Builds the plan (geometry, arena, descriptors, work lists) of a frame list.
static int plan_batch(orbgpu_batch* b, int nframes, const int* widths, const int* heights, const int* nfeatures,
                      float scale_factor, int nlevels, int ini_th, int min_th, int per_frame_cap) {
    std::vector<int> sig = {nframes, nlevels, ini_th, min_th, per_frame_cap};
    int sfb;
    std::memcpy(&sfb, &scale_factor, 4);
    sig.push_back(sfb);
    for (int f = 0; f < nframes; f++) {
        sig.push_back(widths[f]);
        sig.push_back(heights[f]);
        sig.push_back(nfeatures[f]);
    }
    if (sig == b->sig) return ORBGPU_OK;
    destroy_graph(b);
    b->sig.clear();
    b->nframes = nframes;
    b->nlevels = nlevels;
    b->tables.clear();
    b->geoms.assign(nframes, {});
    b->layouts.assign(nframes, {});
    b->frame_base.assign(nframes, 0);
    size_t off = 0;
    for (int f = 0; f < nframes; f++) {
        b->tables.push_back(make_tables(nfeatures[f], scale_factor, nlevels));
        int rc = level_geometry(b->tables.back(), widths[f], heights[f], b->geoms[f]);
        if (rc != ORBGPU_OK) {
            orbgpu_set_last_error("frame size not supported by the level geometry", __FILE__, __LINE__);
            return rc;
        }
        b->frame_base[f] = off;
        off = b->layouts[f].plan(b->geoms[f], off);
    }
    if (off > b->arena_bytes) {
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(b->stream));
        if (b->arena) cudaFree(b->arena);
        b->arena = nullptr;
        b->arena_bytes = 0;
        ORBGPU_CUDA_TRY(cudaMalloc(&b->arena, off));
        b->arena_bytes = off;
    }
    // resize tables of every frame
    std::vector<uint8_t> host(off, 0);
    for (int f = 0; f < nframes; f++) fill_tables(b->geoms[f], b->layouts[f], host, 0);
    ORBGPU_CUDA_TRY(cudaMemcpy(b->arena, host.data(), off, cudaMemcpyHostToDevice));
    // descriptors
    const int ndesc = nframes * nlevels;
    if ((size_t)ndesc > b->descs_cap) {
        if (b->d_descs) cudaFree(b->d_descs);
        b->d_descs = nullptr;
        ORBGPU_CUDA_TRY(cudaMalloc(&b->d_descs, sizeof(LevelDesc) * ndesc));
        b->descs_cap = ndesc;
    }
    std::vector<LevelDesc> hd(ndesc);
    for (int f = 0; f < nframes; f++) {
        fill_descs(b->geoms[f], b->tables[f], b->layouts[f], b->arena, f, ini_th, min_th, f * per_frame_cap,
                   per_frame_cap, &hd[(size_t)f * nlevels]);
        for (int l = 0; l < nlevels; l++) hd[(size_t)f * nlevels + l].frame_total = b->d_totals + f;
    }
    ORBGPU_CUDA_TRY(cudaMemcpy(b->d_descs, hd.data(), sizeof(LevelDesc) * ndesc, cudaMemcpyHostToDevice));
    // work lists: resize/blur tiles per level (all frames), then all cells
    std::vector<WorkItem> items;
    b->rb_first.assign(nlevels, 0);
    b->rb_count.assign(nlevels, 0);
    for (int l = 0; l < nlevels; l++) {
        b->rb_first[l] = (int)items.size();
        for (int f = 0; f < nframes; f++) {
            const LevelGeom& L = b->geoms[f][l];
            const int tiles = ((L.w + 63) / 64) * ((L.h + 15) / 16);
            for (int i = 0; i < tiles; i++) items.push_back({f * nlevels + l, i});
        }
        b->rb_count[l] = (int)items.size() - b->rb_first[l];
    }
    b->fast_first = (int)items.size();
    // larger levels first so the long blocks start early
    for (int l = 0; l < nlevels; l++)
        for (int f = 0; f < nframes; f++)
            for (int c = 0; c < b->geoms[f][l].ncells; c++) items.push_back({f * nlevels + l, c});
    b->fast_count = (int)items.size() - b->fast_first;
    if (items.size() > b->items_cap) {
        if (b->d_items) cudaFree(b->d_items);
        b->d_items = nullptr;
        ORBGPU_CUDA_TRY(cudaMalloc(&b->d_items, items.size() * sizeof(WorkItem)));
        b->items_cap = items.size();
    }
    ORBGPU_CUDA_TRY(cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice));
    b->max_kept = 0;
    b->sort_cap = 1;
    for (auto& g : b->geoms)
        for (auto& L : g) {
            b->max_kept = std::max(b->max_kept, L.node_cap);
            while (b->sort_cap < L.node_cap) b->sort_cap <<= 1;
        }
    b->ndesc = ndesc;
    b->sig = sig;
    return ORBGPU_OK;
}

static void enqueue_pipeline(orbgpu_batch* b, orbgpu_keypoint* kps, uint8_t* desc) {
    cudaStream_t st = b->stream;
    int maxh = 0;
    for (int f = 0; f < b->nframes; f++) maxh = std::max(maxh, b->geoms[f][0].h);
    dim3 g((maxh + 7) / 8, b->nframes);
    k_gather_images<<<g, 256, 0, st>>>(b->d_src, b->nframes);
    for (int l = 0; l < b->nlevels; l++)
        launch_resize_blur(b->d_descs, b->d_items + b->rb_first[l], b->rb_count[l], l == 0, st);
    launch_fast(b->d_descs, b->d_items + b->fast_first, b->fast_count, b->d_status, st);
    launch_distribute(b->d_descs, b->ndesc, b->sort_cap, b->d_status, st);
    launch_describe(b->d_descs, b->ndesc, b->max_kept, kps, desc, b->d_status, st);
    b->launches_per_run = 1 + b->nlevels + 3;
}

extern "C" int orbgpu_batch_extract(orbgpu_batch* b, int nframes, const uint8_t* const* images, const int* widths,
                                    const int* heights, const size_t* steps, const int* nfeatures, float scale_factor,
                                    int nlevels, int ini_th_fast, int min_th_fast, orbgpu_keypoint* keypoints,
                                    uint8_t* descriptors, int per_frame_capacity, int out_mem, int* n_keypoints) {
    if (!b || nframes < 0 || nframes > b->max_frames || !images || !widths || !heights || !steps || !nfeatures ||
        nlevels < 1 || nlevels > ORBGPU_MAX_LEVELS || !(scale_factor > 1.0f) || per_frame_capacity < 1 ||
        !keypoints || !descriptors || !n_keypoints || out_mem != ORBGPU_MEM_DEVICE) {
        orbgpu_set_last_error("invalid batch arguments (outputs must be device memory)", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (nframes == 0) return ORBGPU_OK;
    for (int f = 0; f < nframes; f++)
        if (!images[f] || widths[f] < 1 || heights[f] < 1 || widths[f] > b->max_w || heights[f] > b->max_h ||
            steps[f] < (size_t)widths[f] || nfeatures[f] < 0 || nfeatures[f] > b->max_nf) {
            orbgpu_set_last_error("invalid frame in batch", __FILE__, __LINE__);
            return ORBGPU_ERR_BAD_ARG;
        }
    int rc = plan_batch(b, nframes, widths, heights, nfeatures, scale_factor, nlevels, ini_th_fast, min_th_fast,
                        per_frame_capacity);
    if (rc != ORBGPU_OK) return rc;
    cudaStream_t st = b->stream;
    // image sources of this call (read by the gather kernel at run time)
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
    for (int f = 0; f < nframes; f++) {
        const LevelGeom& L0 = b->geoms[f][0];
        b->h_src[f] = {images[f], widths[f], heights[f], (int)steps[f], b->arena + b->layouts[f].lv[0].pyr, L0.pitch};
    }
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(b->d_src, b->h_src, sizeof(ImageSrc) * nframes, cudaMemcpyHostToDevice, st));
    ORBGPU_CUDA_TRY(cudaMemsetAsync(b->d_status, 0, sizeof(int) * 4, st));
    if (!b->graph || b->graph_kps != keypoints || b->graph_desc != descriptors) {
        destroy_graph(b);
        cudaGraph_t g;
        ORBGPU_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        enqueue_pipeline(b, keypoints, descriptors);
        ORBGPU_CUDA_TRY(cudaStreamEndCapture(st, &g));
        ORBGPU_CUDA_TRY(cudaGraphInstantiate(&b->graph, g, 0));
        cudaGraphDestroy(g);
        b->graph_kps = keypoints;
        b->graph_desc = descriptors;
    }
    ORBGPU_CUDA_TRY(cudaGraphLaunch(b->graph, st));
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(n_keypoints, b->d_totals, sizeof(int) * nframes, cudaMemcpyDeviceToDevice, st));
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(b->h_pinned, b->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
    if (b->h_pinned[0] & ~16) {
        char msg[128];
        std::snprintf(msg, sizeof(msg), "device-side capacity check failed (status 0x%x)", b->h_pinned[0]);
        orbgpu_set_last_error(msg, __FILE__, __LINE__);
        return ORBGPU_ERR_CUDA;
    }
    if (b->h_pinned[0] & 16) {
        orbgpu_set_last_error("per-frame output capacity too small", __FILE__, __LINE__);
        return ORBGPU_ERR_CAPACITY;
    }
    return ORBGPU_OK;
}

// Kernels launched by one orbgpu_batch_extract call.
extern "C" int orbgpu_batch_launch_count(const orbgpu_batch* b) { return b ? b->launches_per_run : 0; }
extern "C" void* orbgpu_batch_stream(const orbgpu_batch* b) { return b ? (void*)b->stream : nullptr; }
