// orbgpu_batch.cu -- batched extraction and projection matching over a
// ragged list of frames.
//
// Frames of different sizes and feature budgets go through the same stage
// kernels as the per-frame path, but each stage is ONE launch over the work
// items of every frame: per level one resize launch (levels >= 1) and one
// blur / FAST-strength launch, one FAST
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
#include "orbgpu_stereo.cuh"

namespace orbgpu {

struct ImageSrc {
    const uint8_t* ptr;
    int w, h;
    int step;
    uint8_t* dst;
    int pitch;
};

// Copies every frame's image into its level-0 plane: a block takes 8 rows of
// a frame, one warp per row, and every row moves in 16-byte vectors.  Plane
// vector j (plane rows are 64-byte aligned) takes source bytes [16 j, 16 j +
// 16) of the row from the two 16-byte aligned source vectors that hold them,
// funnel-shifted by the row start's offset.  An aligned 16-byte load that
// holds a byte of the row cannot leave the row's pages; the second vector is
// loaded only when it holds one.  Bytes past the image width land in the row
// padding.
__device__ __forceinline__ uint4 gather_shift(const uint32_t (&w)[8], int k, int sh) {
    switch (k) {  // the row start's word offset: uniform over the warp
        case 0:
            return make_uint4(__funnelshift_r(w[0], w[1], sh), __funnelshift_r(w[1], w[2], sh),
                              __funnelshift_r(w[2], w[3], sh), __funnelshift_r(w[3], w[4], sh));
        case 1:
            return make_uint4(__funnelshift_r(w[1], w[2], sh), __funnelshift_r(w[2], w[3], sh),
                              __funnelshift_r(w[3], w[4], sh), __funnelshift_r(w[4], w[5], sh));
        case 2:
            return make_uint4(__funnelshift_r(w[2], w[3], sh), __funnelshift_r(w[3], w[4], sh),
                              __funnelshift_r(w[4], w[5], sh), __funnelshift_r(w[5], w[6], sh));
        default:
            return make_uint4(__funnelshift_r(w[3], w[4], sh), __funnelshift_r(w[4], w[5], sh),
                              __funnelshift_r(w[5], w[6], sh), __funnelshift_r(w[6], w[7], sh));
    }
}
__global__ void __launch_bounds__(256) k_gather_images(const ImageSrc* src, int nframes) {
    const int f = blockIdx.y;
    if (f >= nframes) return;
    const ImageSrc s = src[f];
    const int y = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (y >= s.h) return;
    const uint8_t* a = s.ptr + (size_t)y * s.step;
    const int off = (int)(reinterpret_cast<uintptr_t>(a) & 15);
    const uint4* a16 = reinterpret_cast<const uint4*>(a - off);
    uint4* b16 = reinterpret_cast<uint4*>(s.dst + (size_t)y * s.pitch);
    const int nv = (s.w + 15) >> 4;  // plane vectors of the row
    const int span = off + s.w;      // bytes from a16 to the row's end
    const int k = off >> 2, sh = 8 * (off & 3);
    for (int j = lane; j < nv; j += 32) {
        const uint4 v0 = a16[j];
        uint4 v1 = make_uint4(0u, 0u, 0u, 0u);
        if (off != 0 && 16 * (j + 1) < span) v1 = a16[j + 1];
        const uint32_t w[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
        b16[j] = gather_shift(w, k, sh);
    }
}

}  // namespace orbgpu

using namespace orbgpu;

// Everything about one frame configuration (size, feature budget) that the
// batch needs: geometry, relative arena layout, the resize tables as a host
// blob per level, and the block counts of its stages.
struct FramePlan {
    int w, h, nf;
    ExtractorTables tables;
    std::vector<LevelGeom> geom;
    FrameLayout layout;  // offsets relative to the frame's slot
    std::vector<std::vector<uint8_t>> table_blob;  // per level (l >= 1): xofs..ybeta region
    int gen = -1;                                   // tuning generation when the plan was made
};

struct orbgpu_batch {
    int max_frames, max_w, max_h, max_nf;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int nlevels = 0;
    float scale_factor = 0.f;
    int ini_th = 0, min_th = 0;
    std::vector<FramePlan*> plans;   // cache of frame configurations
    // one arena slot per frame position; slot_plan[f] is what its tables hold
    uint8_t* arena = nullptr;
    size_t slot_bytes = 0;
    std::vector<const FramePlan*> slot_plan;
    std::vector<int> slot_gen;  // tuning generation of the tables in each slot
    // current batch
    std::vector<const FramePlan*> cur;
    int nframes = 0;
    std::vector<int> sig;
    std::vector<int> h_prefix;  // host copy of the block-range prefix arrays
    int* d_prefix = nullptr;
    size_t prefix_cap = 0;
    std::vector<int> rb_off, rb_count;
    int rows = 22;  // strip rows of the current batch's resize / blur launches
    int fast_off = 0, fast_count = 0;
    LevelDesc* d_descs = nullptr;
    size_t descs_cap = 0;
    int ndesc = 0;
    int max_kept = 0, sort_cap = 0;
    ImageSrc* d_src = nullptr;
    ImageSrc* h_src = nullptr;  // pinned
    bool pending = false;       // an asynchronous extraction whose status has not been read
    int* d_status = nullptr;
    int* d_totals = nullptr;  // per frame
    int* h_pinned = nullptr;
    cudaGraphExec_t graph = nullptr;
    std::vector<int> graph_sig;
    orbgpu_keypoint* graph_kps = nullptr;
    uint8_t* graph_desc = nullptr;
    int same_sig_runs = 0;
    int launches_per_run = 0;
    cudaEvent_t ev[6] = {};
    // the resize chain of levels 1.. runs on a second stream beside the
    // strips (a level's strip waits for its resize only)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_level[ORBGPU_MAX_LEVELS] = {};

    // frame configuration handed to the accessors of the last batch
    std::vector<float> frame_scale;  // nframes * 16
    std::vector<int> frame_w, frame_h;
    int frame_cap = 0;
    // scratch of the batched stereo search (grown on demand)
    uint8_t* st_scratch = nullptr;
    size_t st_bytes = 0;
    int* st_pinned = nullptr;
};

static void destroy_graph(orbgpu_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_sig.clear();
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
    rc = ensure_constants();
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
    for (int i = 0; i < 6; i++)
        if (cudaEventCreate(&b->ev[i]) != cudaSuccess) {
            orbgpu_batch_destroy(b);
            return ORBGPU_ERR_CUDA;
        }
    bool side_ok = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) == cudaSuccess &&
                   cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; side_ok && i < ORBGPU_MAX_LEVELS; i++)
        side_ok = cudaEventCreateWithFlags(&b->ev_level[i], cudaEventDisableTiming) == cudaSuccess;
    if (!side_ok) {
        orbgpu_batch_destroy(b);
        return ORBGPU_ERR_CUDA;
    }
    b->slot_plan.assign(max_frames, nullptr);
    b->slot_gen.assign(max_frames, -1);
    *out = b;
    return ORBGPU_OK;
}

extern "C" int orbgpu_batch_destroy(orbgpu_batch* b) {
    if (!b) return ORBGPU_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    destroy_graph(b);
    cudaFree(b->arena);
    cudaFree(b->d_descs);
    cudaFree(b->d_prefix);
    cudaFree(b->d_status);
    cudaFree(b->d_totals);
    cudaFree(b->st_scratch);
    if (b->st_pinned) cudaFreeHost(b->st_pinned);
    cudaFree(b->d_src);
    cudaFreeHost(b->h_src);
    cudaFreeHost(b->h_pinned);
    for (int i = 0; i < 6; i++)
        if (b->ev[i]) cudaEventDestroy(b->ev[i]);
    if (b->side) cudaStreamSynchronize(b->side);
    for (int i = 0; i < ORBGPU_MAX_LEVELS; i++)
        if (b->ev_level[i]) cudaEventDestroy(b->ev_level[i]);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->side) cudaStreamDestroy(b->side);

    for (FramePlan* p : b->plans) delete p;
    if (b->own_stream) cudaStreamDestroy(b->stream);
    delete b;
    return ORBGPU_OK;
}

static int get_plan(orbgpu_batch* b, int w, int h, int nf, const FramePlan** out) {
    for (FramePlan* p : b->plans)
        if (p->w == w && p->h == h && p->nf == nf) {
            *out = p;
            return ORBGPU_OK;
        }
    FramePlan* P = new FramePlan();
    P->w = w;
    P->h = h;
    P->nf = nf;
    P->tables = make_tables(nf, b->scale_factor, b->nlevels);
    int rc = level_geometry(P->tables, w, h, P->geom);
    if (rc != ORBGPU_OK) {
        delete P;
        orbgpu_set_last_error("frame size not supported by the level geometry", __FILE__, __LINE__);
        return rc;
    }
    P->layout.plan(P->geom, 0);
    P->table_blob.assign(b->nlevels, {});
    for (int l = 0; l < b->nlevels; l++) {
        const LevelGeom& L = P->geom[l];
        if (l == 0) continue;
        const LevelOffsets& o = P->layout.lv[l];
        const size_t lo = o.xofs, hi = o.ybeta + sizeof(short) * 2 * L.h;
        std::vector<uint8_t>& blob = P->table_blob[l];
        blob.assign(hi - lo, 0);
        if (!resize_tables(P->geom[l - 1].w, P->geom[l - 1].h, L.w, L.h, (int*)&blob[o.xofs - lo],
                           (short*)&blob[o.xalpha - lo], (int*)&blob[o.yofs - lo], (short*)&blob[o.ybeta - lo])) {
            delete P;
            orbgpu_set_last_error("resize weights out of range", __FILE__, __LINE__);
            return ORBGPU_ERR_BAD_ARG;
        }
    }
    P->gen = tune_generation();
    b->plans.push_back(P);
    *out = P;
    return ORBGPU_OK;
}

// Plans the batch: frame configurations, arena slots (tables written only
// where a slot changes configuration), descriptors and block ranges.
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
    // launch shapes: a new tuning makes a new signature
    sig.push_back(tune_generation());
    if (sig == b->sig) {
        b->same_sig_runs++;
        return ORBGPU_OK;
    }
    b->same_sig_runs = 0;
    b->frame_w.assign(widths, widths + nframes);
    b->frame_h.assign(heights, heights + nframes);
    b->frame_cap = per_frame_cap;
    if (nlevels != b->nlevels || scale_factor != b->scale_factor) {  // configuration cache is per pyramid shape
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(b->stream));
        for (FramePlan* p : b->plans) delete p;
        b->plans.clear();
        std::fill(b->slot_plan.begin(), b->slot_plan.end(), nullptr);
        b->nlevels = nlevels;
        b->scale_factor = scale_factor;
    }
    b->ini_th = ini_th;
    b->min_th = min_th;
    b->cur.assign(nframes, nullptr);
    size_t need = b->slot_bytes;
    for (int f = 0; f < nframes; f++) {
        int rc = get_plan(b, widths[f], heights[f], nfeatures[f], &b->cur[f]);
        if (rc != ORBGPU_OK) return rc;
        need = std::max(need, (b->cur[f]->layout.bytes + 4095) & ~(size_t)4095);
    }
    cudaStream_t st = b->stream;
    if (need > b->slot_bytes || !b->arena) {
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
        destroy_graph(b);
        if (b->arena) cudaFree(b->arena);
        b->arena = nullptr;
        ORBGPU_CUDA_TRY(dev_malloc(&b->arena, need * b->max_frames));
        b->slot_bytes = need;
        std::fill(b->slot_plan.begin(), b->slot_plan.end(), nullptr);
    }
    // resize tables of slots whose configuration changed
    for (int f = 0; f < nframes; f++) {
        const FramePlan* P = b->cur[f];
        if (b->slot_plan[f] == P && b->slot_gen[f] == P->gen) continue;
        uint8_t* base = b->arena + (size_t)f * b->slot_bytes;
        for (int l = 1; l < nlevels; l++)
            ORBGPU_CUDA_TRY(cudaMemcpyAsync(base + P->layout.lv[l].xofs, P->table_blob[l].data(), P->table_blob[l].size(),
                                            cudaMemcpyHostToDevice, st));
        // the descriptor kernel's tensor maps of this slot (a pageable
        // source: the copy has taken the bytes when it returns)
        std::vector<uint8_t> maps;
        const int mrc = encode_patch_maps(P->geom, P->layout, base, maps);
        if (mrc != ORBGPU_OK) return mrc;
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(base + P->layout.patch_maps, maps.data(), maps.size(), cudaMemcpyHostToDevice, st));
        b->slot_plan[f] = P;
        b->slot_gen[f] = P->gen;
    }
    // descriptors
    const int ndesc = nframes * nlevels;
    if ((size_t)ndesc > b->descs_cap) {
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
        if (b->d_descs) cudaFree(b->d_descs);
        b->d_descs = nullptr;
        ORBGPU_CUDA_TRY(dev_malloc(&b->d_descs, sizeof(LevelDesc) * b->max_frames * nlevels));
        b->descs_cap = (size_t)b->max_frames * nlevels;
    }
    std::vector<LevelDesc> hd(ndesc);
    b->frame_scale.assign((size_t)nframes * 16, 1.0f);
    for (int f = 0; f < nframes; f++) {
        const FramePlan* P = b->cur[f];
        fill_descs(P->geom, P->tables, P->layout, b->arena + (size_t)f * b->slot_bytes, f, ini_th, min_th,
                   f * per_frame_cap, per_frame_cap, &hd[(size_t)f * nlevels]);
        for (int l = 0; l < nlevels; l++) {
            hd[(size_t)f * nlevels + l].frame_total = b->d_totals + f;
            b->frame_scale[(size_t)f * 16 + l] = P->tables.scale[l];
        }
    }
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(b->d_descs, hd.data(), sizeof(LevelDesc) * ndesc, cudaMemcpyHostToDevice, st));
    // block ranges: per level the tiles of every frame (strips of the rows
    // that suit the batch's level-0 pixel count), then the cells of every
    // (frame, level) pair
    long px = 0;
    for (int f = 0; f < nframes; f++) px += (long)widths[f] * heights[f];
    b->rows = strip_rows(px);
    std::vector<int>& pre = b->h_prefix;
    pre.clear();
    b->rb_off.assign(nlevels, 0);
    b->rb_count.assign(nlevels, 0);
    for (int l = 0; l < nlevels; l++) {
        b->rb_off[l] = (int)pre.size();
        int acc = 0;
        for (int f = 0; f < nframes; f++) {
            pre.push_back(acc);
            acc += resize_blur_tiles(b->cur[f]->geom[l].w, b->cur[f]->geom[l].h, b->rows);
        }
        pre.push_back(acc);
        b->rb_count[l] = acc;
    }
    b->fast_off = (int)pre.size();
    int acc = 0;
    for (int f = 0; f < nframes; f++)
        for (int l = 0; l < nlevels; l++) {
            pre.push_back(acc);
            acc += b->cur[f]->geom[l].ncells;
        }
    pre.push_back(acc);
    b->fast_count = acc;
    if (pre.size() > b->prefix_cap) {
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
        if (b->d_prefix) cudaFree(b->d_prefix);
        b->d_prefix = nullptr;
        const size_t cap = (size_t)(b->max_frames + 1) * nlevels + (size_t)b->max_frames * nlevels + 1;
        ORBGPU_CUDA_TRY(dev_malloc(&b->d_prefix, sizeof(int) * std::max(cap, pre.size())));
        b->prefix_cap = std::max(cap, pre.size());
    }
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(b->d_prefix, pre.data(), sizeof(int) * pre.size(), cudaMemcpyHostToDevice, st));
    b->max_kept = 0;
    b->sort_cap = 1;
    for (int f = 0; f < nframes; f++)
        for (auto& L : b->cur[f]->geom) {
            b->max_kept = std::max(b->max_kept, L.node_cap);
            while (b->sort_cap < L.node_cap) b->sort_cap <<= 1;
        }
    b->nframes = nframes;
    b->ndesc = ndesc;
    b->sig = sig;
    // the block-range and descriptor uploads above read pageable host
    // memory: complete them before the host vectors change
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
    return ORBGPU_OK;
}

static void enqueue_pipeline(orbgpu_batch* b, orbgpu_keypoint* kps, uint8_t* desc, bool capturing) {
    cudaStream_t st = b->stream;
    // inside a capture the stage events become external event nodes (timed by
    // the host on every replay); outside, plain records
    auto mark = [&](int i) {
        if (capturing) cudaEventRecordWithFlags(b->ev[i], st, cudaEventRecordExternal);
        else cudaEventRecord(b->ev[i], st);
    };
    int maxh = 0;
    for (int f = 0; f < b->nframes; f++) maxh = std::max(maxh, b->cur[f]->geom[0].h);
    dim3 g((maxh + 7) / 8, b->nframes);
    // stage boundaries are recorded as external events (event record nodes
    // in the graph that the host can time), so the per-stage device time of
    // every replay can be read back
    mark(0);
    k_gather_images<<<g, 256, 0, st>>>(b->d_src, b->nframes);
    mark(1);
    // levels 1.. are resized in a chain on the side stream while the strips
    // of the levels already resized run on the batch's stream
    cudaEventRecord(b->ev_fork, st);
    cudaStreamWaitEvent(b->side, b->ev_fork, 0);
    for (int l = 1; l < b->nlevels; l++) {
        launch_level_resize(b->d_descs, RangeMap{b->d_prefix + b->rb_off[l], b->nframes, l, b->nlevels},
                            b->rb_count[l], b->rows, b->side);
        cudaEventRecord(b->ev_level[l], b->side);
    }
    for (int l = 0; l < b->nlevels; l++) {
        if (l > 0) cudaStreamWaitEvent(st, b->ev_level[l], 0);
        launch_level_strip(b->d_descs, RangeMap{b->d_prefix + b->rb_off[l], b->nframes, l, b->nlevels},
                           b->rb_count[l], b->rows, st);
    }
    mark(2);
    int mwc = 1, mhc = 1, mbox = 0;
    for (int f = 0; f < b->nframes; f++)
        for (const LevelGeom& L : b->cur[f]->geom) {
            mwc = std::max(mwc, L.wCell);
            mhc = std::max(mhc, L.hCell);
            if (L.ncells > 0) mbox = std::max(mbox, fast_cell_box_w(L.wCell) * (L.hCell + 6));
        }
    launch_fast(b->d_descs, RangeMap{b->d_prefix + b->fast_off, b->ndesc, 0, 1}, b->fast_count, b->d_status, mwc, mhc,
                mbox, st);
    mark(3);
    launch_distribute(b->d_descs, b->ndesc, b->sort_cap, b->max_kept, b->d_status, st);
    mark(4);
    launch_describe(b->d_descs, b->ndesc, b->max_kept, kps, desc, b->d_status, st);
    mark(5);
    // gather, strip per level, resize per level >= 1, FAST cells,
    // DistributeOctTree, describe
    b->launches_per_run = 1 + 2 * b->nlevels - 1 + 3;
}

// The device status of the last extraction (copied to h_pinned[0] at its end)
// as a return code; the stream must have been synchronised.
static int batch_status(orbgpu_batch* b) {
    b->pending = false;
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

extern "C" int orbgpu_batch_wait(orbgpu_batch* b) {
    if (!b) return ORBGPU_ERR_BAD_ARG;
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(b->stream));
    return b->pending ? batch_status(b) : ORBGPU_OK;
}

static int batch_extract(orbgpu_batch* b, int nframes, const uint8_t* const* images, const int* widths,
                         const int* heights, const size_t* steps, const int* nfeatures, float scale_factor, int nlevels,
                         int ini_th_fast, int min_th_fast, orbgpu_keypoint* keypoints, uint8_t* descriptors,
                         int per_frame_capacity, int out_mem, int* n_keypoints, bool wait) {
    if (b && b->pending) {  // the previous asynchronous extraction's status first
        const int rc = orbgpu_batch_wait(b);
        if (rc != ORBGPU_OK) return rc;
    }
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
    cudaStream_t st = b->stream;
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));  // h_src is rewritten below
    int rc = plan_batch(b, nframes, widths, heights, nfeatures, scale_factor, nlevels, ini_th_fast, min_th_fast,
                        per_frame_capacity);
    if (rc != ORBGPU_OK) return rc;
    // image sources of this call (read by the gather kernel at run time)
    for (int f = 0; f < nframes; f++) {
        const LevelGeom& L0 = b->cur[f]->geom[0];
        b->h_src[f] = {images[f], widths[f], heights[f], (int)steps[f],
                       b->arena + (size_t)f * b->slot_bytes + b->cur[f]->layout.lv[0].pyr, L0.pitch};
    }
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(b->d_src, b->h_src, sizeof(ImageSrc) * nframes, cudaMemcpyHostToDevice, st));
    ORBGPU_CUDA_TRY(cudaMemsetAsync(b->d_status, 0, sizeof(int) * 4, st));
    const bool graph_ok = b->graph && b->graph_sig == b->sig && b->graph_kps == keypoints && b->graph_desc == descriptors;
    if (graph_ok) {
        ORBGPU_CUDA_TRY(cudaGraphLaunch(b->graph, st));
    } else if (b->same_sig_runs >= 1) {
        // the same frame list came again: capture it once and replay from now on
        destroy_graph(b);
        cudaGraph_t g;
        ORBGPU_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        enqueue_pipeline(b, keypoints, descriptors, true);
        ORBGPU_CUDA_TRY(cudaStreamEndCapture(st, &g));
        ORBGPU_CUDA_TRY(cudaGraphInstantiate(&b->graph, g, 0));
        cudaGraphDestroy(g);
        b->graph_sig = b->sig;
        b->graph_kps = keypoints;
        b->graph_desc = descriptors;
        ORBGPU_CUDA_TRY(cudaGraphLaunch(b->graph, st));
    } else {
        enqueue_pipeline(b, keypoints, descriptors, false);
    }
    ORBGPU_CUDA_TRY(cudaGetLastError());
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(n_keypoints, b->d_totals, sizeof(int) * nframes, cudaMemcpyDeviceToDevice, st));
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(b->h_pinned, b->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (!wait) {
        b->pending = true;
        return ORBGPU_OK;
    }
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
    return batch_status(b);
}

extern "C" int orbgpu_batch_extract(orbgpu_batch* b, int nframes, const uint8_t* const* images, const int* widths,
                                    const int* heights, const size_t* steps, const int* nfeatures, float scale_factor,
                                    int nlevels, int ini_th_fast, int min_th_fast, orbgpu_keypoint* keypoints,
                                    uint8_t* descriptors, int per_frame_capacity, int out_mem, int* n_keypoints) {
    return batch_extract(b, nframes, images, widths, heights, steps, nfeatures, scale_factor, nlevels, ini_th_fast,
                         min_th_fast, keypoints, descriptors, per_frame_capacity, out_mem, n_keypoints, true);
}

extern "C" int orbgpu_batch_extract_async(orbgpu_batch* b, int nframes, const uint8_t* const* images,
                                          const int* widths, const int* heights, const size_t* steps,
                                          const int* nfeatures, float scale_factor, int nlevels, int ini_th_fast,
                                          int min_th_fast, orbgpu_keypoint* keypoints, uint8_t* descriptors,
                                          int per_frame_capacity, int out_mem, int* n_keypoints) {
    return batch_extract(b, nframes, images, widths, heights, steps, nfeatures, scale_factor, nlevels, ini_th_fast,
                         min_th_fast, keypoints, descriptors, per_frame_capacity, out_mem, n_keypoints, false);
}

// Device time of the stages of the last orbgpu_batch_extract call (ms):
// gather, resize+blur (all levels), FAST cells, DistributeOctTree, describe.
extern "C" int orbgpu_batch_stage_times(orbgpu_batch* b, float* ms, int n) {
    if (!b || !ms || n < 5) return ORBGPU_ERR_BAD_ARG;
    ORBGPU_CUDA_TRY(cudaEventSynchronize(b->ev[5]));
    for (int i = 0; i < 5; i++) ORBGPU_CUDA_TRY(cudaEventElapsedTime(&ms[i], b->ev[i], b->ev[i + 1]));
    return ORBGPU_OK;
}

// Kernels launched by one orbgpu_batch_extract call.
extern "C" int orbgpu_batch_launch_count(const orbgpu_batch* b) { return b ? b->launches_per_run : 0; }
extern "C" void* orbgpu_batch_stream(const orbgpu_batch* b) { return b ? (void*)b->stream : nullptr; }

// ---------------------------------------------------------------- batched SearchByProjection
// SearchByProjection(Frame&, vector<MapPoint*>, th) (src/ORBmatcher.cc:72-183)
// for every frame of the last batch at once: grid build, candidate listing
// (warp per map point, fixed-capacity slots) and the in-order resolution
// (one warp per frame), five launches for the whole batch.
namespace orbgpu {

struct BatchFrameInfo {
    float invW, invH;
    int n_cap;
    float scale[16];
};

__global__ void k_bgrid_count(const orbgpu_keypoint* kps, const int* counts, int cap, const BatchFrameInfo* info,
                              int* key_cell, int* cell_count) {
    const int f = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= min(counts[f], cap)) return;
    const orbgpu_keypoint kp = kps[(size_t)f * cap + i];
    const int px = (int)roundf(__fmul_rn(__fsub_rn(kp.x, 0.0f), info[f].invW));
    const int py = (int)roundf(__fmul_rn(__fsub_rn(kp.y, 0.0f), info[f].invH));
    int c = -1;
    if (px >= 0 && px < ORBGPU_GRID_COLS && py >= 0 && py < ORBGPU_GRID_ROWS) c = px * ORBGPU_GRID_ROWS + py;
    key_cell[(size_t)f * cap + i] = c;
    if (c >= 0) atomicAdd(&cell_count[f * (ORBGPU_GRID_COLS * ORBGPU_GRID_ROWS) + c], 1);
}

__global__ void k_bgrid_scan(const int* cell_count, int* cell_start, int* cursor) {
    __shared__ int s_scan[32];
    const int ncell = ORBGPU_GRID_COLS * ORBGPU_GRID_ROWS;
    const int f = blockIdx.x;
    const int* cc = cell_count + (size_t)f * ncell;
    int* cs = cell_start + (size_t)f * (ncell + 1);
    int* cu = cursor + (size_t)f * ncell;
    int base = 0;
    for (int b0 = 0; b0 < ncell; b0 += blockDim.x) {
        const int c = b0 + threadIdx.x;
        const int v = c < ncell ? cc[c] : 0;
        int tot;
        const int ex = block_exclusive_scan(v, s_scan, &tot);
        if (c < ncell) {
            cs[c] = base + ex;
            cu[c] = base + ex;
        }
        base += tot;
    }
    if (threadIdx.x == 0) cs[ncell] = base;
}

__global__ void k_bgrid_fill(const int* counts, int cap, const int* key_cell, int* cursor, int* cell_keys) {
    const int f = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= min(counts[f], cap)) return;
    const int c = key_cell[(size_t)f * cap + i];
    if (c >= 0) cell_keys[(size_t)f * cap + atomicAdd(&cursor[f * (ORBGPU_GRID_COLS * ORBGPU_GRID_ROWS) + c], 1)] = i;
}

// BPROJ_SEG lanes per map point (32 / BPROJ_SEG map points per warp): a
// window covers about a dozen grid cells and a handful of keypoints.
#define BPROJ_SEG 16
__global__ void k_bproj_candidates(const orbgpu_keypoint* kps, const uint8_t* desc, int cap, const BatchFrameInfo* info,
                                   const int* cell_start, const int* cell_keys, const int* key_cell,
                                   const orbgpu_mappoint* mps,
                                   const uint8_t* mp_desc, const int* mp_off, float th, float nnratio, int slot_cap,
                                   uint64_t* slots, int* slot_count, int* status) {
    // A candidate with nnratio * dist > TH_HIGH (nnratio <= 1) can neither be
    // accepted (dist > TH_HIGH) nor make an accepted best fail the ratio test
    // (best <= TH_HIGH < nnratio * dist), so the lists leave it out.
    constexpr int W = BPROJ_SEG;
    const bool drop_far = nnratio <= 1.0f;
    const int f = blockIdx.y;
    const int lane = threadIdx.x & 31, sl = lane & (W - 1), sbase = lane & ~(W - 1);
    const unsigned smask = (W == 32 ? 0xffffffffu : ((1u << W) - 1)) << sbase;
    const int local = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * (32 / W) + lane / W;
    const int imp = mp_off[f] + local;
    const bool have = imp < mp_off[f + 1];
    if (__all_sync(0xffffffffu, !have)) return;
    const BatchFrameInfo& I = info[f];
    const orbgpu_keypoint* K = kps + (size_t)f * cap;
    const uint8_t* D = desc + (size_t)f * cap * 32;
    const int* cs = cell_start + (size_t)f * (ORBGPU_GRID_COLS * ORBGPU_GRID_ROWS + 1);
    const int* ck = cell_keys + (size_t)f * cap;
    const int* kc = key_cell + (size_t)f * cap;
    orbgpu_mappoint mp{};
    if (have) mp = mps[imp];
    bool active = have && mp.track_in_view && !mp.bad && mp.track_scale_level >= 0 && mp.track_scale_level < 16;
    int x0 = 0, x1 = -1, y0 = 0, y1 = -1, level = 0;
    float x = 0.f, y = 0.f, rr = 0.f;
    if (active) {
        level = mp.track_scale_level;
        float r = mp.view_cos > 0.998f ? 2.5f : 4.0f;
        if (th != 1.0f) r = __fmul_rn(r, th);
        const float radius = __fmul_rn(r, I.scale[level]);
        x = mp.proj_x;
        y = mp.proj_y;
        x0 = max(0, (int)floorf(__fmul_rn(__fsub_rn(__fsub_rn(x, 0.0f), radius), I.invW)));
        x1 = min(ORBGPU_GRID_COLS - 1, (int)ceilf(__fmul_rn(__fadd_rn(__fsub_rn(x, 0.0f), radius), I.invW)));
        y0 = max(0, (int)floorf(__fmul_rn(__fsub_rn(__fsub_rn(y, 0.0f), radius), I.invH)));
        y1 = min(ORBGPU_GRID_ROWS - 1, (int)ceilf(__fmul_rn(__fadd_rn(__fsub_rn(y, 0.0f), radius), I.invH)));
        active = x0 < ORBGPU_GRID_COLS && x1 >= 0 && y0 < ORBGPU_GRID_ROWS && y1 >= 0 && x0 <= x1 && y0 <= y1;
        rr = __fmul_rn(radius, radius);
    }
    uint4 dm0 = make_uint4(0, 0, 0, 0), dm1 = dm0;  // the map point's descriptor
    if (active) {
        const uint4* dp = reinterpret_cast<const uint4*>(mp_desc + (size_t)imp * 32);
        dm0 = dp[0];
        dm1 = dp[1];
    }
    int total = 0;
    seg_window_cols<W>(cs, ck, ORBGPU_GRID_ROWS, active, x0, x1, y0, y1, [&](int idx, bool valid) {
        bool ok = false;
        int dist = 256, c = 0;
        if (valid) {
            c = kc[idx];
            const orbgpu_keypoint kp = K[idx];
            ok = kp.octave >= level - 1 && kp.octave <= level;
            if (ok) {
                const float dx = __fsub_rn(kp.x, x), dy = __fsub_rn(kp.y, y);
                ok = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) < rr;
            }
            if (ok) {
                const uint4* kd = reinterpret_cast<const uint4*>(D + (size_t)idx * 32);
                dist = hamming256(dm0, dm1, kd[0], kd[1]);
                ok = !(drop_far && __fmul_rn(nnratio, (float)dist) > (float)ORBGPU_TH_HIGH);
            }
        }
        const unsigned msk = __ballot_sync(0xffffffffu, ok) & smask;
        if (ok) {
            const int pos = total + __popc(msk & ((1u << lane) - 1));
            if (pos < slot_cap)
                slots[(size_t)imp * slot_cap + pos] =
                    ((uint64_t)(uint32_t)dist << 40) | ((uint64_t)(uint32_t)c << 20) | (uint64_t)(uint32_t)idx;
        }
        total += __popc(msk);
    });
    if (have && sl == 0) {
        slot_count[imp] = total;
        if (total > slot_cap) atomicMax(status, total);
    }
}

// Parallel resolution by fixed-point rounds.  In the reference a map point
// sees a keypoint as claimed iff an earlier map point of the same call took
// it.  Round r evaluates every map point against the claims made by the
// results of round r-1 (claim owner = smallest map point index that took the
// keypoint); once a round changes no result, every map point's result is
// consistent with the results of the map points before it, which by
// induction over the map point order is the sequential result.  Three claim
// arrays rotate: read (round r-1's claims), write (round r's), and the one
// cleared for round r+1.  A frame that has not converged after the last
// round is replayed serially by k_bproj_resolve.
#define BPROJ_ROUNDS 12
#define BPROJ_NONE 0x7f7f7f7f

__global__ void k_bproj_round(const orbgpu_keypoint* kps, int cap, const int* counts, const int* mp_off,
                              int slot_cap, const uint64_t* slots, const int* slot_count, float nnratio, int round,
                              int* claims3, int* res, int* changed, int* nwarp_frame) {
    const int f = blockIdx.y;
    const int lane = threadIdx.x & 31;
    const int local = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int n_mp = mp_off[f + 1] - mp_off[f];
    if (round > 0 && changed[(round - 1) * gridDim.y + f] == 0) return;  // converged
    int* claims_r = claims3 + (size_t)((round + 0) % 3) * gridDim.y * cap + (size_t)f * cap;
    int* claims_w = claims3 + (size_t)((round + 1) % 3) * gridDim.y * cap + (size_t)f * cap;
    int* claims_z = claims3 + (size_t)((round + 2) % 3) * gridDim.y * cap + (size_t)f * cap;
    // clear the array the next round writes into
    for (int i = local * 32 + lane; i < cap; i += (*nwarp_frame) * 32) claims_z[i] = BPROJ_NONE;
    if (local >= n_mp) return;
    const int imp = mp_off[f] + local;
    const orbgpu_keypoint* K = kps + (size_t)f * cap;
    const int cnt = min(slot_count[imp], slot_cap);
    const uint64_t* S = slots + (size_t)imp * slot_cap;
    uint64_t best = ~0ull, second = ~0ull;
    for (int b = 0; b < cnt; b += 32) {
        uint64_t key = ~0ull;
        if (b + lane < cnt) {
            key = S[b + lane];
            if (claims_r[(int)(key & 0xFFFFF)] < local || (int)(key >> 40) >= 256) key = ~0ull;
        }
        if (key < best) {
            second = best;
            best = key;
        } else if (key < second) {
            second = key;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t ob = __shfl_xor_sync(0xffffffffu, best, o);
        const uint64_t os = __shfl_xor_sync(0xffffffffu, second, o);
        if (ob < best) {
            second = best < os ? best : os;
            best = ob;
        } else {
            second = second < ob ? second : ob;
        }
    }
    int r = -1;
    if (best != ~0ull) {
        const int bestDist = (int)(best >> 40);
        const int bestIdx = (int)(best & 0xFFFFF);
        const int bestLevel = K[bestIdx].octave;
        const int bestDist2 = second == ~0ull ? 256 : (int)(second >> 40);
        const int bestLevel2 = second == ~0ull ? -1 : K[(int)(second & 0xFFFFF)].octave;
        if (bestDist <= ORBGPU_TH_HIGH &&
            !(bestLevel == bestLevel2 && (float)bestDist > __fmul_rn(nnratio, (float)bestDist2)))
            r = bestIdx;
    }
    if (lane == 0) {
        if (res[imp] != r) changed[round * gridDim.y + f] = 1;
        res[imp] = r;
        if (r >= 0) atomicMin(&claims_w[r], local);
    }
}

// The same fixed-point resolution with one block per frame and the whole
// frame in shared memory: the map points' candidate keys (32 bits: distance,
// GetFeaturesInArea cell, keypoint index -- the lexicographic order of the
// 64-bit keys, all distinct), the keypoints' octaves, the results and two
// claim arrays.  A map point's result is the best and second-best of its
// candidates not claimed by an earlier map point in the previous round, i.e.
// the first two such in key order: each thread keeps the four smallest keys
// of its map points in registers and reads the whole list only when fewer
// than two of them are unclaimed.  Rounds repeat until one changes nothing
// (at most M + 1 rounds: round r fixes the first r + 1 map points).  Used
// when every frame's candidates fit (smem_bytes of dynamic shared memory);
// the global-memory rounds above handle the rest.
#define BPROJ_MPT 4  // map points per thread with register top-4 lists (1024 threads: M <= 4096)
__global__ void __launch_bounds__(1024)
    k_bproj_resolve_smem(const orbgpu_keypoint* kps, int cap, const int* counts, const int* mp_off, int slot_cap,
                         const uint64_t* slots, const int* slot_count, float nnratio, int smem_bytes,
                         int* match_out, int* nmatches, int* status) {
    extern __shared__ __align__(16) int s_dyn[];
    __shared__ int s_scan[32];
    __shared__ int s_flag[3];
    const int f = blockIdx.x;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int mp0 = mp_off[f], M = mp_off[f + 1] - mp0;
    const int n = min(counts[f], cap);
    constexpr int NONE = 0x7fffffff;
    constexpr uint32_t NOKEY = 0xFFFFFFFFu;
    int* s_start = s_dyn;  // M + 1: candidate list of map point i
    int base = 0;
    for (int i0 = 0; i0 < M; i0 += nt) {
        const int i = i0 + tid;
        const int v = i < M ? min(slot_count[mp0 + i], slot_cap) : 0;
        int tot;
        const int ex = block_exclusive_scan(v, s_scan, &tot);
        if (i < M) s_start[i] = base + ex;
        base += tot;
    }
    if (4L * (2 * M + 1 + 2 * cap + base) + cap + 16 > smem_bytes) {  // the frame's candidates do not fit
        if (tid == 0) atomicOr(status + 2, 1);
        return;
    }
    int* s_res = s_start + (M + 1);                          // M
    int* cr = s_res + M;                                     // cap: claims of the previous round
    int* cw = cr + cap;                                      // cap: claims of this round
    uint32_t* s_key = reinterpret_cast<uint32_t*>(cw + cap);  // base
    uint8_t* s_oct = reinterpret_cast<uint8_t*>(s_key + base);  // cap
    if (tid == 0) s_start[M] = base;
    if (tid < 3) s_flag[tid] = 0;
    for (int k = tid; k < cap; k += nt) {
        cr[k] = NONE;
        cw[k] = NONE;
    }
    for (int k = tid; k < n; k += nt) s_oct[k] = (uint8_t)kps[(size_t)f * cap + k].octave;
    __syncthreads();
    // keys, one thread per map point (independent loads); the four smallest of
    // the thread's first BPROJ_MPT map points kept in registers
    uint32_t top[BPROJ_MPT][4];
    int tcnt[BPROJ_MPT];
#pragma unroll
    for (int q = 0; q < BPROJ_MPT; q++) {
        tcnt[q] = 0;
#pragma unroll
        for (int j = 0; j < 4; j++) top[q][j] = NOKEY;
    }
    for (int i = tid, q = 0; i < M; i += nt, q++) {
        const int s0 = s_start[i], cnt = s_start[i + 1] - s0;
        const uint64_t* S = slots + (size_t)(mp0 + i) * slot_cap;
        uint32_t t0 = NOKEY, t1 = NOKEY, t2 = NOKEY, t3 = NOKEY;
        for (int b = 0; b < cnt; b++) {
            const uint64_t key = S[b];
            const uint32_t dist = (uint32_t)(key >> 40), cell = (uint32_t)(key >> 20) & 0xFFFFFu,
                           idx = (uint32_t)key & 0xFFFFFu;
            const uint32_t k32 = dist >= 256 ? NOKEY : (dist << 24) | (cell << 12) | idx;
            s_key[s0 + b] = k32;
            // insertion into the sorted four
            if (k32 < t3) {
                if (k32 < t2) {
                    t3 = t2;
                    if (k32 < t1) {
                        t2 = t1;
                        if (k32 < t0) {
                            t1 = t0;
                            t0 = k32;
                        } else {
                            t1 = k32;
                        }
                    } else {
                        t2 = k32;
                    }
                } else {
                    t3 = k32;
                }
            }
        }
#pragma unroll
        for (int qq = 0; qq < BPROJ_MPT; qq++)
            if (qq == q) {
                top[qq][0] = t0;
                top[qq][1] = t1;
                top[qq][2] = t2;
                top[qq][3] = t3;
                tcnt[qq] = cnt;
            }
        s_res[i] = -2;
    }
    // map point i's result from claims cr: the first two candidates in key
    // order that no earlier map point claimed
    auto decide = [&](int i, uint32_t best, uint32_t second) -> int {
        if (best == NOKEY) return -1;
        const int bestDist = (int)(best >> 24);
        const int bestIdx = (int)(best & 0xFFFu);
        const int bestLevel = s_oct[bestIdx];
        const int bestDist2 = second == NOKEY ? 256 : (int)(second >> 24);
        const int bestLevel2 = second == NOKEY ? -1 : s_oct[second & 0xFFFu];
        if (bestDist <= ORBGPU_TH_HIGH && !(bestLevel == bestLevel2 && (float)bestDist > __fmul_rn(nnratio, (float)bestDist2)))
            return bestIdx;
        return -1;
    };
    auto full_scan = [&](int i, uint32_t& best, uint32_t& second) {
        best = NOKEY;
        second = NOKEY;
        for (int e = s_start[i]; e < s_start[i + 1]; e++) {
            const uint32_t key = s_key[e];
            if (key == NOKEY || cr[key & 0xFFFu] < i) continue;
            if (key < best) {
                second = best;
                best = key;
            } else if (key < second) {
                second = key;
            }
        }
    };
    bool converged = M == 0;
    int rounds_run = 0;
    for (int round = 0; round <= M + 1 && !converged; round++) {
        rounds_run = round + 1;
        if (tid == 0) s_flag[(round + 1) % 3] = 0;
        __syncthreads();
#pragma unroll
        for (int q = 0; q < BPROJ_MPT; q++) {
            const int i = tid + q * nt;
            if (i >= M) continue;
            uint32_t best = NOKEY, second = NOKEY;
            int found = 0;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const uint32_t key = top[q][j];
                if (found < 2 && key != NOKEY && !(cr[key & 0xFFFu] < i)) {
                    if (found == 0) best = key;
                    else second = key;
                    found++;
                }
            }
            if (found < 2 && tcnt[q] > 4) full_scan(i, best, second);
            const int r = decide(i, best, second);
            if (r != s_res[i]) {
                s_res[i] = r;
                s_flag[round % 3] = 1;
            }
            if (r >= 0) atomicMin(&cw[r], i);
        }
        for (int i = tid + BPROJ_MPT * nt; i < M; i += nt) {
            uint32_t best, second;
            full_scan(i, best, second);
            const int r = decide(i, best, second);
            if (r != s_res[i]) {
                s_res[i] = r;
                s_flag[round % 3] = 1;
            }
            if (r >= 0) atomicMin(&cw[r], i);
        }
        __syncthreads();
        converged = s_flag[round % 3] == 0;
        // this round's claims are read by the next; the array read now is cleared for writing
        int* t = cr;
        cr = cw;
        cw = t;
        if (!converged)
            for (int k = tid; k < cap; k += nt) cw[k] = NONE;
    }
    if (tid == 0) {
        if (!converged) atomicOr(status + 2, 2);
        atomicMax(status + 3, rounds_run);
    }
    int* Mo = match_out + (size_t)f * cap;
    for (int k = tid; k < cap; k += nt) Mo[k] = k < n ? -1 : -3;
    __syncthreads();
    int nm = 0;
    for (int i = tid; i < M; i += nt) {
        const int r = s_res[i];
        if (r >= 0) {
            Mo[r] = i;
            nm++;
        }
    }
    int tot;
    block_exclusive_scan(nm, s_scan, &tot);
    if (tid == 0) nmatches[f] = tot;
}

// Writes match_out / nmatches from the converged results; frames that did
// not converge are replayed serially (same code as k_bproj_resolve).
__global__ void k_bproj_finish(const orbgpu_keypoint* kps, int cap, const int* counts, const int* mp_off, int slot_cap,
                               const uint64_t* slots, const int* slot_count, float nnratio, const int* changed,
                               const int* res, int* match_out, int* nmatches, int* status) {
    const int f = blockIdx.x;
    const int lane = threadIdx.x;
    int* M = match_out + (size_t)f * cap;
    const int n = min(counts[f], cap);
    if (changed[(BPROJ_ROUNDS - 1) * gridDim.x + f] == 0) {
        for (int i = lane; i < cap; i += 32) M[i] = i < n ? -1 : -3;
        __syncwarp();
        int nm = 0;
        for (int imp = mp_off[f] + lane; imp < mp_off[f + 1]; imp += 32) {
            const int r = res[imp];
            if (r >= 0) {
                M[r] = imp - mp_off[f];
                nm++;
            }
        }
        nm = warp_sum(nm);
        if (lane == 0) nmatches[f] = nm;
        return;
    }
    if (lane == 0) atomicAdd(status + 1, 1);
    // serial replay
    const orbgpu_keypoint* K = kps + (size_t)f * cap;
    for (int i = lane; i < cap; i += 32) M[i] = i < n ? -1 : -3;
    __syncwarp();
    int nm = 0;
    for (int imp = mp_off[f]; imp < mp_off[f + 1]; imp++) {
        const int cnt = min(slot_count[imp], slot_cap);
        if (cnt == 0) continue;
        const uint64_t* S = slots + (size_t)imp * slot_cap;
        uint64_t best = ~0ull, second = ~0ull;
        for (int b = 0; b < cnt; b += 32) {
            uint64_t key = ~0ull;
            if (b + lane < cnt) {
                key = S[b + lane];
                if (M[(int)(key & 0xFFFFF)] != -1 || (int)(key >> 40) >= 256) key = ~0ull;
            }
            if (key < best) {
                second = best;
                best = key;
            } else if (key < second) {
                second = key;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const uint64_t ob = __shfl_xor_sync(0xffffffffu, best, o);
            const uint64_t os = __shfl_xor_sync(0xffffffffu, second, o);
            if (ob < best) {
                second = best < os ? best : os;
                best = ob;
            } else {
                second = second < ob ? second : ob;
            }
        }
        if (best == ~0ull) continue;
        const int bestDist = (int)(best >> 40);
        const int bestIdx = (int)(best & 0xFFFFF);
        const int bestLevel = K[bestIdx].octave;
        const int bestDist2 = second == ~0ull ? 256 : (int)(second >> 40);
        const int bestLevel2 = second == ~0ull ? -1 : K[(int)(second & 0xFFFFF)].octave;
        if (bestDist <= ORBGPU_TH_HIGH) {
            if (bestLevel == bestLevel2 && (float)bestDist > __fmul_rn(nnratio, (float)bestDist2)) continue;
            if (lane == 0) M[bestIdx] = imp - mp_off[f];
            nm++;
        }
        __syncwarp();
    }
    if (lane == 0) nmatches[f] = nm;
}

}  // namespace orbgpu

struct orbgpu_batch_proj {
    uint8_t* scratch = nullptr;
    size_t bytes = 0;
    int slot_cap = 64;
    int* h_pinned = nullptr;
    int* h_cands = nullptr;  // per-frame candidate totals (pinned)
    int h_cands_cap = 0;
    int last_serial_frames = 0;
    int last_launches = 0;
    int last_rounds = 0;  // fixed-point rounds of the slowest frame (shared-memory resolution)
    int mode = 0;  // 0: shared-memory resolution when the frames fit; 1: global-memory rounds
    // frame info and map point offsets as last uploaded (skipped when unchanged)
    std::vector<uint8_t> last_upload;
    uint8_t* h_stage = nullptr;  // pinned staging of the uploads
    size_t h_stage_cap = 0;
};
// one scratch per host thread (the search is synchronous)
static thread_local orbgpu_batch_proj g_bproj;

static int orbgpu_batch_search_last_launches() { return g_bproj.last_launches; }
extern "C" int orbgpu_batch_search_rounds(void) { return g_bproj.last_rounds; }

extern "C" int orbgpu_batch_search_mode(int mode) {
    if (mode != 0 && mode != 1) return ORBGPU_ERR_BAD_ARG;
    g_bproj.mode = mode;
    return ORBGPU_OK;
}

// Projection search over the frames of the last orbgpu_batch_extract call.
// kps/desc/counts: that call's outputs (device); mappoints / mp_descriptors:
// all frames' map points back to back (device), frame f owning
// [mp_offsets[f], mp_offsets[f+1]) (host array).  match_out: device,
// nframes * per_frame_capacity ints (map point index within the frame, -1
// none, -3 past the frame's keypoints); nmatches: device, nframes ints.
extern "C" int orbgpu_batch_search_by_projection(orbgpu_batch* b, const orbgpu_keypoint* kps, const uint8_t* desc,
                                                 const int* counts, const orbgpu_mappoint* mappoints,
                                                 const uint8_t* mp_descriptors, const int* mp_offsets, float th,
                                                 float nnratio, int* match_out, int* nmatches) {
    if (!b || b->nframes <= 0 || !kps || !desc || !counts || !mp_offsets || !match_out || !nmatches)
        return ORBGPU_ERR_BAD_ARG;
    const int nf = b->nframes;
    const int cap = b->frame_cap;
    const int ncell = ORBGPU_GRID_COLS * ORBGPU_GRID_ROWS;
    const int total_mp = mp_offsets[nf];
    int max_mp = 0;
    for (int f = 0; f < nf; f++) max_mp = std::max(max_mp, mp_offsets[f + 1] - mp_offsets[f]);
    orbgpu_batch_proj& P = g_bproj;
    if (!P.h_pinned) ORBGPU_CUDA_TRY(cudaMallocHost(&P.h_pinned, 64));
    cudaStream_t st = b->stream;
    for (int attempt = 0; attempt < 3; attempt++) {
        const size_t need = sizeof(BatchFrameInfo) * nf + sizeof(int) * ((size_t)nf * ncell * 2 + (size_t)nf * (ncell + 1) +
                                                                      (size_t)nf * cap * 5 + (nf + 1) + 2 * total_mp +
                                                                      BPROJ_ROUNDS * nf + nf + 16) +
                            sizeof(uint64_t) * (size_t)std::max(1, total_mp) * P.slot_cap + 8 * 256;
        if (need > P.bytes) {
            ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
            if (P.scratch) cudaFree(P.scratch);
            P.scratch = nullptr;
            ORBGPU_CUDA_TRY(dev_malloc(&P.scratch, need));
            P.bytes = need;
            P.last_upload.clear();
        }
        size_t off = 0;
        auto take = [&](size_t n) {
            off = (off + 255) & ~(size_t)255;
            uint8_t* p = P.scratch + off;
            off += n;
            return p;
        };
        BatchFrameInfo* info = (BatchFrameInfo*)take(sizeof(BatchFrameInfo) * nf);
        int* d_off = (int*)take(sizeof(int) * (nf + 1));  // uploaded with info in one copy
        int* cell_count = (int*)take(sizeof(int) * (size_t)nf * ncell);
        int* cursor = (int*)take(sizeof(int) * (size_t)nf * ncell);
        int* cell_start = (int*)take(sizeof(int) * (size_t)nf * (ncell + 1));
        int* key_cell = (int*)take(sizeof(int) * (size_t)nf * cap);
        int* cell_keys = (int*)take(sizeof(int) * (size_t)nf * cap);
        int* slot_count = (int*)take(sizeof(int) * std::max(1, total_mp));
        int* status = (int*)take(sizeof(int) * 4);
        uint64_t* slots = (uint64_t*)take(sizeof(uint64_t) * (size_t)std::max(1, total_mp) * P.slot_cap);
        int* claims3 = (int*)take(sizeof(int) * (size_t)3 * nf * cap);
        int* res = (int*)take(sizeof(int) * std::max(1, total_mp));
        int* changed = (int*)take(sizeof(int) * BPROJ_ROUNDS * nf);
        int* nwarp = (int*)take(sizeof(int) * 2);
        std::vector<BatchFrameInfo> hi(nf);
        for (int f = 0; f < nf; f++) {
            const int w = b->frame_w[f], h = b->frame_h[f];
            hi[f].invW = static_cast<float>(ORBGPU_GRID_COLS) / static_cast<float>((float)w - 0.0f);
            hi[f].invH = static_cast<float>(ORBGPU_GRID_ROWS) / static_cast<float>((float)h - 0.0f);
            hi[f].n_cap = cap;
            for (int l = 0; l < 16; l++) hi[f].scale[l] = b->frame_scale[(size_t)f * 16 + l];
        }
        {
            // frame info then offsets, contiguous in the scratch (info is 256-aligned and d_off follows it)
            const size_t ib = sizeof(BatchFrameInfo) * nf, ob = sizeof(int) * (nf + 1);
            const size_t gap = (size_t)((uint8_t*)d_off - (uint8_t*)info);
            std::vector<uint8_t> up(gap + ob, 0);
            std::memcpy(up.data(), hi.data(), ib);
            std::memcpy(up.data() + gap, mp_offsets, ob);
            if (up != P.last_upload) {
                if (P.h_stage_cap < up.size()) {
                    if (P.h_stage) cudaFreeHost(P.h_stage);
                    P.h_stage = nullptr;
                    ORBGPU_CUDA_TRY(cudaMallocHost(&P.h_stage, up.size()));
                    P.h_stage_cap = up.size();
                }
                std::memcpy(P.h_stage, up.data(), up.size());  // the previous call's copy has completed (it synchronised)
                ORBGPU_CUDA_TRY(cudaMemcpyAsync(info, P.h_stage, up.size(), cudaMemcpyHostToDevice, st));
                P.last_upload.swap(up);
            }
        }
        ORBGPU_CUDA_TRY(cudaMemsetAsync(cell_count, 0, sizeof(int) * (size_t)nf * ncell, st));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int) * 4, st));
        dim3 gk((cap + 255) / 256, nf);
        k_bgrid_count<<<gk, 256, 0, st>>>(kps, counts, cap, info, key_cell, cell_count);
        k_bgrid_scan<<<nf, 1024, 0, st>>>(cell_count, cell_start, cursor);
        k_bgrid_fill<<<gk, 256, 0, st>>>(counts, cap, key_cell, cursor, cell_keys);
        const int wpb = 8;
        const int mp_per_block = wpb * (32 / BPROJ_SEG);
        dim3 gc((std::max(1, max_mp) + mp_per_block - 1) / mp_per_block, nf);
        k_bproj_candidates<<<gc, 32 * wpb, 0, st>>>(kps, desc, cap, info, cell_start, cell_keys, key_cell, mappoints,
                                                   mp_descriptors, d_off, th, nnratio, P.slot_cap, slots, slot_count,
                                                   status);
        // every frame in shared memory when it fits (one launch, sized for up
        // to t_cap candidates per frame; the kernel reports a frame above it),
        // else the global-memory fixed-point rounds and the result write-out
        // (serial replay for any frame that did not converge)
        // s_start, s_res, two claim arrays (ints), octaves and dirty flags
        // (bytes), then 4 bytes per candidate (6 with the keypoint index):
        // the kernel lays its frame out once it knows the frame's candidates
        const size_t fixed = sizeof(int) * ((size_t)2 * max_mp + 1 + 2 * (size_t)cap) + (size_t)cap + (size_t)max_mp + 64;
        const size_t smem_max = 226 * 1024;  // below the 227 KiB per-block limit with the static part
        if (P.mode == 0 && cap < 4096 && fixed + 4 * 1024 <= smem_max) {
            const size_t smem = smem_max;
            ORBGPU_CUDA_TRY(allow_max_dynamic_smem(k_bproj_resolve_smem));
            k_bproj_resolve_smem<<<nf, 1024, smem, st>>>(kps, cap, counts, d_off, P.slot_cap, slots, slot_count, nnratio,
                                                         (int)smem, match_out, nmatches, status);
            ORBGPU_CUDA_TRY(cudaGetLastError());
            ORBGPU_CUDA_TRY(cudaMemcpyAsync(P.h_pinned, status, sizeof(int) * 4, cudaMemcpyDeviceToHost, st));
            ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
            if (P.h_pinned[0] > P.slot_cap) {  // a window held more candidates than the slots: widen and redo
                P.slot_cap = ((P.h_pinned[0] + 63) / 64) * 64;
                continue;
            }
            P.last_serial_frames = 0;
            P.last_launches = 4 + 1;
            P.last_rounds = P.h_pinned[3];
            if (P.h_pinned[2] & 2) {
                orbgpu_set_last_error("batched projection: shared-memory resolution failed", __FILE__, __LINE__);
                return ORBGPU_ERR_CUDA;
            }
            if (!(P.h_pinned[2] & 1)) return ORBGPU_OK;
            // a frame above t_cap: the global-memory rounds below
        } else {
            ORBGPU_CUDA_TRY(cudaMemcpyAsync(P.h_pinned, status, sizeof(int), cudaMemcpyDeviceToHost, st));
            ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
            if (P.h_pinned[0] > P.slot_cap) {
                P.slot_cap = ((P.h_pinned[0] + 63) / 64) * 64;
                continue;
            }
        }
        P.last_launches = 4 + BPROJ_ROUNDS + 1;
        const int warps = std::max((std::max(1, max_mp) + wpb - 1) / wpb * wpb, ((cap + 31) / 32 + wpb - 1) / wpb * wpb);
        P.h_pinned[1] = warps;
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(nwarp, &P.h_pinned[1], sizeof(int), cudaMemcpyHostToDevice, st));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(claims3, 0x7f, sizeof(int) * (size_t)3 * nf * cap, st));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(res, 0xfe, sizeof(int) * std::max(1, total_mp), st));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(changed, 0, sizeof(int) * BPROJ_ROUNDS * nf, st));
        dim3 gr(warps / wpb, nf);
        for (int r = 0; r < BPROJ_ROUNDS; r++)
            k_bproj_round<<<gr, 32 * wpb, 0, st>>>(kps, cap, counts, d_off, P.slot_cap, slots, slot_count, nnratio, r,
                                                  claims3, res, changed, nwarp);
        k_bproj_finish<<<nf, 32, 0, st>>>(kps, cap, counts, d_off, P.slot_cap, slots, slot_count, nnratio, changed, res,
                                         match_out, nmatches, status);
        ORBGPU_CUDA_TRY(cudaGetLastError());
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(P.h_pinned + 2, status + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
        P.last_serial_frames = P.h_pinned[2];
        return ORBGPU_OK;
    }
    return ORBGPU_ERR_CAPACITY;
}

extern "C" int orbgpu_batch_search_launch_count(void) {
    return orbgpu_batch_search_last_launches();
}

// ---------------------------------------------------------------- batched SearchByProjection(Frame, LastFrame)
// ORBmatcher::SearchByProjection(Frame& CurrentFrame, const Frame& LastFrame,
// th, bMono) (src/ORBmatcher.cc:1710-1879) for every frame of the last batch:
// CurrentFrame f is the batch's frame f, LastFrame f comes with its own
// keypoints, map points and pose.  Candidate keys are 32 bits (distance,
// GetFeaturesInArea cell, keypoint index), only those at or below TH_HIGH
// (no ratio test: the first minimum wins).  One block per frame resolves the
// in-order assignment (owners without observations block nothing), the
// owners, the rotation histogram, the three maxima and the resets.
namespace orbgpu {

struct BatchMotion {
    float T[12];
    float fx, fy, cx, cy, bf;
    float maxX, maxY;
    int level_mode;
};

__device__ __forceinline__ float bpose_row(const float* row, float X0, float X1, float X2) {
    double s = __dadd_rn(0.0, __dmul_rn((double)row[0], (double)X0));
    s = __dadd_rn(s, __dmul_rn((double)row[1], (double)X1));
    s = __dadd_rn(s, __dmul_rn((double)row[2], (double)X2));
    return __fadd_rn(__double2float_rn(s), row[3]);
}

__global__ void k_bpf_candidates(const orbgpu_keypoint* kps, const uint8_t* desc, int cap, const BatchFrameInfo* info,
                                 const int* cell_start, const int* cell_keys, const int* key_cell,
                                 const BatchMotion* motions,
                                 const orbgpu_keypoint* last_kps, const orbgpu_frame_mappoint* last_mps,
                                 const uint8_t* last_desc, const int* last_off, float th, int slot_cap,
                                 uint32_t* slots, int* slot_count, int* status, int* frame_cands) {
    const int ncell = ORBGPU_GRID_COLS * ORBGPU_GRID_ROWS;
    const int f = blockIdx.y;
    const int lane = threadIdx.x & 31;
    const int local = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int i = last_off[f] + local;
    if (i >= last_off[f + 1]) return;
    const orbgpu_frame_mappoint mp = last_mps[i];
    const BatchMotion& mo = motions[f];
    const BatchFrameInfo& I = info[f];
    const orbgpu_keypoint* K = kps + (size_t)f * cap;
    const uint8_t* D = desc + (size_t)f * cap * 32;
    const int* cs = cell_start + (size_t)f * (ncell + 1);
    const int* ck = cell_keys + (size_t)f * cap;
    const int* kc = key_cell + (size_t)f * cap;
    const int oct = last_kps[i].octave;
    int total = 0;
    bool live = (mp.flags & ORBGPU_MP_PRESENT) && !(mp.flags & ORBGPU_MP_OUTLIER) && oct >= 0 && oct < 16;
    float u = 0.f, v = 0.f;
    if (live) {
        const float xc = bpose_row(mo.T, mp.x, mp.y, mp.z);
        const float yc = bpose_row(mo.T + 4, mp.x, mp.y, mp.z);
        const float zc = bpose_row(mo.T + 8, mp.x, mp.y, mp.z);
        const float invzc = __double2float_rn(__ddiv_rn(1.0, (double)zc));
        u = __fadd_rn(__fmul_rn(__fmul_rn(mo.fx, xc), invzc), mo.cx);
        v = __fadd_rn(__fmul_rn(__fmul_rn(mo.fy, yc), invzc), mo.cy);
        live = !(invzc < 0.f) && isfinite(u) && isfinite(v) && !(u < 0.0f || u > mo.maxX) && !(v < 0.0f || v > mo.maxY);
    }
    if (live) {
        const float radius = __fmul_rn(th, I.scale[oct]);
        int minL, maxL;
        if (mo.level_mode == 1) {
            minL = oct;
            maxL = -1;
        } else if (mo.level_mode == 2) {
            minL = 0;
            maxL = oct;
        } else {
            minL = oct - 1;
            maxL = oct + 1;
        }
        const bool check = (minL > 0) || (maxL >= 0);  // GetFeaturesInArea's level test (src/Frame.cc:628)
        const int x0 = max(0, (int)floorf(__fmul_rn(__fsub_rn(__fsub_rn(u, 0.0f), radius), I.invW)));
        const int x1 = min(ORBGPU_GRID_COLS - 1, (int)ceilf(__fmul_rn(__fadd_rn(__fsub_rn(u, 0.0f), radius), I.invW)));
        const int y0 = max(0, (int)floorf(__fmul_rn(__fsub_rn(__fsub_rn(v, 0.0f), radius), I.invH)));
        const int y1 = min(ORBGPU_GRID_ROWS - 1, (int)ceilf(__fmul_rn(__fadd_rn(__fsub_rn(v, 0.0f), radius), I.invH)));
        if (x0 < ORBGPU_GRID_COLS && x1 >= 0 && y0 < ORBGPU_GRID_ROWS && y1 >= 0) {
            const uint8_t* dmp = last_desc + (size_t)i * 32;
            const float rr = __fmul_rn(radius, radius);
            warp_window_keys(cs, ck, kc, ORBGPU_GRID_ROWS, x0, x1, y0, y1, [&](int idx, int c, bool valid) {
                bool ok = false;
                int dist = 256;
                if (valid) {
                    const orbgpu_keypoint kp = K[idx];
                    ok = !(check && (kp.octave < minL || (maxL >= 0 && kp.octave > maxL)));
                    if (ok) {
                        const float dx = __fsub_rn(kp.x, u), dy = __fsub_rn(kp.y, v);
                        ok = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) < rr;
                    }
                    if (ok) {
                        dist = hamming256_ptr(dmp, D + (size_t)idx * 32);
                        ok = dist <= ORBGPU_TH_HIGH;
                    }
                }
                const unsigned msk = __ballot_sync(0xffffffffu, ok);
                if (ok) {
                    const int pos = total + __popc(msk & ((1u << lane) - 1));
                    if (pos < slot_cap)
                        slots[(size_t)i * slot_cap + pos] = ((uint32_t)dist << 24) | ((uint32_t)c << 12) | (uint32_t)idx;
                }
                total += __popc(msk);
            });
        }
    }
    if (lane == 0) {
        slot_count[i] = total;
        if (total > slot_cap) atomicMax(status, total);
        if (total > 0) atomicAdd(&frame_cands[f], min(total, slot_cap));
    }
}

// One block per frame.  Shared memory: list starts (M + 1), results (M),
// two claim arrays (cap), observed flags and histogram bins (M bytes each),
// and the keys when t_cap > 0 (else they are read from the global slots).
__global__ void __launch_bounds__(1024)
    k_bpf_resolve(const orbgpu_keypoint* kps, int cap, const int* counts, const orbgpu_keypoint* last_kps,
                  const orbgpu_frame_mappoint* last_mps, const int* last_off, int slot_cap, const uint32_t* slots,
                  const int* slot_count, int check_ori, int t_cap, int* match_out, int* nmatches, int* status) {
    extern __shared__ __align__(16) int s_dyn[];
    __shared__ int s_scan[32];
    __shared__ int s_flag[3];
    __shared__ int hist[ORBGPU_HISTO_LENGTH];
    __shared__ int s_ind[3];
    const int f = blockIdx.x;
    const int tid = threadIdx.x;
    const int mp0 = last_off[f], M = last_off[f + 1] - mp0;
    const int n = min(counts[f], cap);
    int* s_start = s_dyn;               // M + 1
    int* s_res = s_start + (M + 1);     // M
    int* cr = s_res + M;                // cap
    int* cw = cr + cap;                 // cap
    uint32_t* s_key = reinterpret_cast<uint32_t*>(cw + cap);            // t_cap
    uint8_t* s_obs = reinterpret_cast<uint8_t*>(s_key + t_cap);         // M
    uint8_t* s_bin = s_obs + M;                                         // M
    int base = 0;
    for (int i0 = 0; i0 < M; i0 += blockDim.x) {
        const int i = i0 + tid;
        const int v = i < M ? min(slot_count[mp0 + i], slot_cap) : 0;
        int tot;
        const int ex = block_exclusive_scan(v, s_scan, &tot);
        if (i < M) s_start[i] = base + ex;
        base += tot;
    }
    const bool in_smem = t_cap > 0;
    if (in_smem && base > t_cap) {
        if (tid == 0) atomicOr(status + 2, 1);
        return;
    }
    if (tid == 0) s_start[M] = base;
    if (tid < 3) s_flag[tid] = 0;
    if (tid < ORBGPU_HISTO_LENGTH) hist[tid] = 0;
    __syncthreads();
    if (in_smem)  // every candidate entry by one thread: the slot loads are independent
        for (int t = tid; t < base; t += blockDim.x) {
            int lo = 0, hi = M - 1;  // last i with s_start[i] <= t
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_start[mid] <= t) lo = mid;
                else hi = mid - 1;
            }
            s_key[t] = slots[(size_t)(mp0 + lo) * slot_cap + (t - s_start[lo])];
        }
    for (int i = tid; i < M; i += blockDim.x) {
        s_res[i] = -2;
        s_obs[i] = (last_mps[mp0 + i].flags & ORBGPU_MP_OBSERVED) ? 1 : 0;
    }
    for (int k = tid; k < cap; k += blockDim.x) {
        cr[k] = 0x7fffffff;
        cw[k] = 0x7fffffff;
    }
    bool converged = M == 0;
    for (int round = 0; round <= M + 1 && !converged; round++) {
        if (tid == 0) s_flag[(round + 1) % 3] = 0;
        __syncthreads();
        for (int i = tid; i < M; i += blockDim.x) {
            const int cnt = s_start[i + 1] - s_start[i];
            const uint32_t* L = in_smem ? s_key + s_start[i] : slots + (size_t)(mp0 + i) * slot_cap;
            uint32_t best = 0xFFFFFFFFu;
            for (int e = 0; e < cnt; e++) {
                const uint32_t key = L[e];
                if (!(cr[key & 0xFFFu] < i) && key < best) best = key;
            }
            const int r = best == 0xFFFFFFFFu ? -1 : (int)(best & 0xFFFu);
            if (r != s_res[i]) {
                s_res[i] = r;
                s_flag[round % 3] = 1;
            }
            if (r >= 0 && s_obs[i]) atomicMin(&cw[r], i);
        }
        __syncthreads();
        converged = s_flag[round % 3] == 0;
        int* t = cr;
        cr = cw;
        cw = t;
        if (!converged)
            for (int k = tid; k < cap; k += blockDim.x) cw[k] = 0x7fffffff;
    }
    if (!converged && tid == 0) atomicOr(status + 2, 2);
    // owners (the last map point that assigned each keypoint), rotation histogram
    int* owner = cr;
    int* nulled = cw;
    __syncthreads();
    for (int k = tid; k < cap; k += blockDim.x) {
        owner[k] = -1;
        nulled[k] = 0;
    }
    __syncthreads();
    const orbgpu_keypoint* K = kps + (size_t)f * cap;
    const float factor = __fdiv_rn((float)ORBGPU_HISTO_LENGTH, 360.0f);
    int nm = 0;
    for (int i = tid; i < M; i += blockDim.x) {
        const int r = s_res[i];
        uint8_t bin = 0xFF;
        if (r >= 0) {
            nm++;
            atomicMax(&owner[r], i);
            if (check_ori) {
                float rot = __fsub_rn(last_kps[mp0 + i].angle, K[r].angle);
                if (rot < 0.0f) rot = __fadd_rn(rot, 360.0f);
                int bb = (int)roundf(__fmul_rn(rot, factor));
                if (bb == ORBGPU_HISTO_LENGTH) bb = 0;
                bin = (uint8_t)bb;
                atomicAdd(&hist[bb], 1);
            }
        }
        s_bin[i] = bin;
    }
    __syncthreads();
    if (tid == 0) {
        int ind1 = -1, ind2 = -1, ind3 = -1;
        if (check_ori) {
            int max1 = 0, max2 = 0, max3 = 0;
            for (int b = 0; b < ORBGPU_HISTO_LENGTH; b++) {  // ComputeThreeMaxima, src/ORBmatcher.cc:2035-2077
                const int sz = hist[b];
                if (sz > max1) {
                    max3 = max2; max2 = max1; max1 = sz;
                    ind3 = ind2; ind2 = ind1; ind1 = b;
                } else if (sz > max2) {
                    max3 = max2; max2 = sz;
                    ind3 = ind2; ind2 = b;
                } else if (sz > max3) {
                    max3 = sz;
                    ind3 = b;
                }
            }
            if ((float)max2 < __fmul_rn(0.1f, (float)max1)) {
                ind2 = -1;
                ind3 = -1;
            } else if ((float)max3 < __fmul_rn(0.1f, (float)max1)) {
                ind3 = -1;
            }
        }
        s_ind[0] = ind1;
        s_ind[1] = ind2;
        s_ind[2] = ind3;
    }
    __syncthreads();
    int removed = 0;
    if (check_ori)
        for (int i = tid; i < M; i += blockDim.x) {
            const int b = s_bin[i];
            if (b == 0xFF || b == s_ind[0] || b == s_ind[1] || b == s_ind[2]) continue;
            nulled[s_res[i]] = 1;
            removed++;
        }
    __syncthreads();
    int* Mo = match_out + (size_t)f * cap;
    for (int k = tid; k < cap; k += blockDim.x) Mo[k] = k >= n ? -3 : nulled[k] ? -4 : (owner[k] >= 0 ? owner[k] : -1);
    int tot;
    block_exclusive_scan(nm - removed, s_scan, &tot);
    if (tid == 0) nmatches[f] = tot;
}

}  // namespace orbgpu

extern "C" int orbgpu_batch_search_by_projection_frame(orbgpu_batch* b, const orbgpu_keypoint* kps, const uint8_t* desc,
                                                       const int* counts, const orbgpu_keypoint* last_kps,
                                                       const orbgpu_frame_mappoint* last_mps,
                                                       const uint8_t* last_desc, const int* last_offsets,
                                                       const orbgpu_frame_motion* motions, float th, int mono,
                                                       int check_ori, int* match_out, int* nmatches) {
    if (!b || b->nframes <= 0 || !kps || !desc || !counts || !last_offsets || !motions || !match_out || !nmatches)
        return ORBGPU_ERR_BAD_ARG;
    const int nf = b->nframes;
    const int cap = b->frame_cap;
    const int ncell = ORBGPU_GRID_COLS * ORBGPU_GRID_ROWS;
    const int total_mp = last_offsets[nf];
    if (cap >= 4096 || total_mp < 0 || (total_mp > 0 && (!last_kps || !last_mps || !last_desc))) {
        orbgpu_set_last_error("batched frame search: per-frame capacity must be below 4096", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    int max_mp = 0;
    for (int f = 0; f < nf; f++) {
        if (last_offsets[f + 1] < last_offsets[f]) return ORBGPU_ERR_BAD_ARG;
        max_mp = std::max(max_mp, last_offsets[f + 1] - last_offsets[f]);
    }
    orbgpu_batch_proj& P = g_bproj;
    P.last_upload.clear();  // this search reuses the scratch the projection search caches its uploads in
    if (!P.h_pinned) ORBGPU_CUDA_TRY(cudaMallocHost(&P.h_pinned, 64));
    if (P.h_cands_cap < nf) {
        if (P.h_cands) cudaFreeHost(P.h_cands);
        P.h_cands = nullptr;
        ORBGPU_CUDA_TRY(cudaMallocHost(&P.h_cands, sizeof(int) * nf));
        P.h_cands_cap = nf;
    }
    std::vector<BatchMotion> hm(nf);
    std::vector<BatchFrameInfo> hi(nf);
    for (int f = 0; f < nf; f++) {
        const orbgpu_frame_motion& m = motions[f];
        std::memcpy(hm[f].T, m.Tcw, sizeof(hm[f].T));
        hm[f].fx = m.fx;
        hm[f].fy = m.fy;
        hm[f].cx = m.cx;
        hm[f].cy = m.cy;
        hm[f].bf = m.bf;
        hm[f].maxX = (float)b->frame_w[f];
        hm[f].maxY = (float)b->frame_h[f];
        hm[f].level_mode = motion_level_mode(m, mono);
        const int w = b->frame_w[f], h = b->frame_h[f];
        hi[f].invW = static_cast<float>(ORBGPU_GRID_COLS) / static_cast<float>((float)w - 0.0f);
        hi[f].invH = static_cast<float>(ORBGPU_GRID_ROWS) / static_cast<float>((float)h - 0.0f);
        hi[f].n_cap = cap;
        for (int l = 0; l < 16; l++) hi[f].scale[l] = b->frame_scale[(size_t)f * 16 + l];
    }
    cudaStream_t st = b->stream;
    for (int attempt = 0; attempt < 3; attempt++) {
        const size_t need = sizeof(BatchFrameInfo) * nf + sizeof(BatchMotion) * nf +
                            sizeof(int) * ((size_t)nf * ncell * 2 + (size_t)nf * (ncell + 1) + (size_t)nf * cap * 2 +
                                           (nf + 1) + (size_t)std::max(1, total_mp) + nf + 16) +
                            sizeof(uint32_t) * (size_t)std::max(1, total_mp) * P.slot_cap + 16 * 256;
        if (need > P.bytes) {
            ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
            if (P.scratch) cudaFree(P.scratch);
            P.scratch = nullptr;
            ORBGPU_CUDA_TRY(dev_malloc(&P.scratch, need));
            P.bytes = need;
        }
        size_t off = 0;
        auto take = [&](size_t n) {
            off = (off + 255) & ~(size_t)255;
            uint8_t* p = P.scratch + off;
            off += n;
            return p;
        };
        BatchFrameInfo* info = (BatchFrameInfo*)take(sizeof(BatchFrameInfo) * nf);
        BatchMotion* mot = (BatchMotion*)take(sizeof(BatchMotion) * nf);
        int* cell_count = (int*)take(sizeof(int) * (size_t)nf * ncell);
        int* cursor = (int*)take(sizeof(int) * (size_t)nf * ncell);
        int* cell_start = (int*)take(sizeof(int) * (size_t)nf * (ncell + 1));
        int* key_cell = (int*)take(sizeof(int) * (size_t)nf * cap);
        int* cell_keys = (int*)take(sizeof(int) * (size_t)nf * cap);
        int* d_off = (int*)take(sizeof(int) * (nf + 1));
        int* slot_count = (int*)take(sizeof(int) * std::max(1, total_mp));
        int* status = (int*)take(sizeof(int) * 4);
        int* frame_cands = (int*)take(sizeof(int) * nf);
        uint32_t* slots = (uint32_t*)take(sizeof(uint32_t) * (size_t)std::max(1, total_mp) * P.slot_cap);
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(info, hi.data(), sizeof(BatchFrameInfo) * nf, cudaMemcpyHostToDevice, st));
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(mot, hm.data(), sizeof(BatchMotion) * nf, cudaMemcpyHostToDevice, st));
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(d_off, last_offsets, sizeof(int) * (nf + 1), cudaMemcpyHostToDevice, st));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(cell_count, 0, sizeof(int) * (size_t)nf * ncell, st));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int) * 4, st));
        ORBGPU_CUDA_TRY(cudaMemsetAsync(frame_cands, 0, sizeof(int) * nf, st));
        dim3 gk((cap + 255) / 256, nf);
        k_bgrid_count<<<gk, 256, 0, st>>>(kps, counts, cap, info, key_cell, cell_count);
        k_bgrid_scan<<<nf, 1024, 0, st>>>(cell_count, cell_start, cursor);
        k_bgrid_fill<<<gk, 256, 0, st>>>(counts, cap, key_cell, cursor, cell_keys);
        const int wpb = 8;
        if (max_mp > 0) {
            dim3 gc((max_mp + wpb - 1) / wpb, nf);
            k_bpf_candidates<<<gc, 32 * wpb, 0, st>>>(kps, desc, cap, info, cell_start, cell_keys, key_cell, mot, last_kps,
                                                      last_mps, last_desc, d_off, th, P.slot_cap, slots, slot_count,
                                                      status, frame_cands);
        }
        ORBGPU_CUDA_TRY(cudaGetLastError());
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(P.h_pinned, status, sizeof(int), cudaMemcpyDeviceToHost, st));
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(P.h_cands, frame_cands, sizeof(int) * nf, cudaMemcpyDeviceToHost, st));
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
        if (P.h_pinned[0] > P.slot_cap) {  // a window held more candidates than the slots: widen and redo
            P.slot_cap = ((P.h_pinned[0] + 63) / 64) * 64;
            continue;
        }
        int t_max = 0;
        for (int f = 0; f < nf; f++) t_max = std::max(t_max, P.h_cands[f]);
        const size_t fixed = sizeof(int) * ((size_t)2 * max_mp + 1 + 2 * (size_t)cap) + 2 * (size_t)max_mp + 64;
        size_t smem = fixed + sizeof(uint32_t) * (size_t)t_max;
        int t_cap = std::max(1, t_max);
        if (smem > 200 * 1024) {  // keys stay in global memory
            smem = fixed;
            t_cap = 0;
        }
        if (smem > 200 * 1024) {
            orbgpu_set_last_error("batched frame search: a frame's map points exceed shared memory", __FILE__, __LINE__);
            return ORBGPU_ERR_CAPACITY;
        }
        ORBGPU_CUDA_TRY(allow_max_dynamic_smem(k_bpf_resolve));
        k_bpf_resolve<<<nf, 1024, smem, st>>>(kps, cap, counts, last_kps, last_mps, d_off, P.slot_cap, slots, slot_count,
                                               check_ori, t_cap, match_out, nmatches, status);
        ORBGPU_CUDA_TRY(cudaGetLastError());
        ORBGPU_CUDA_TRY(cudaMemcpyAsync(P.h_pinned + 2, status + 1, sizeof(int) * 2, cudaMemcpyDeviceToHost, st));
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
        P.last_launches = 5;
        if (P.h_pinned[3] != 0) {
            orbgpu_set_last_error("batched frame search: resolution failed", __FILE__, __LINE__);
            return ORBGPU_ERR_CUDA;
        }
        return ORBGPU_OK;
    }
    return ORBGPU_ERR_CAPACITY;
}

// ---------------------------------------------------------------- batched stereo
// Frame::ComputeStereoMatches (src/Frame.cc:831-1082) for many (left, right)
// frame pairs of one batch extraction in one pass: the device functions of
// orbgpu_stereo.cuh over the pyramids resident in the batch's arena slots,
// one launch per step for all pairs (grid y = pair).
namespace orbgpu {

struct StereoPair {
    StereoLevels lv;
    int left, right;  // frame indices of the extraction
    int nRows;        // level-0 rows
    float bf, fx;
};

__global__ void k_bstereo_rows_count(const orbgpu_keypoint* kps, const int* counts, int cap, const StereoPair* pairs,
                                     int rows_stride, int* row_count) {
    const StereoPair& P = pairs[blockIdx.y];
    const int nR = min(counts[P.right], cap);
    int* rc = row_count + (size_t)blockIdx.y * rows_stride;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nR; i += gridDim.x * blockDim.x) {
        int lo, hi;
        if (!stereo_rows_of(kps[(size_t)P.right * cap + i], P.lv, P.nRows, lo, hi)) continue;
        for (int yi = lo; yi <= hi; yi++) atomicAdd(&rc[yi], 1);
    }
}

// One block per pair: row_start = exclusive prefix of the row counts
// (nRows + 1 entries), cursor = its copy.
__global__ void k_bstereo_scan(const int* row_count, const StereoPair* pairs, int rows_stride, int* row_start,
                               int* cursor) {
    __shared__ int s_scan[32];
    const int n = pairs[blockIdx.x].nRows + 1;
    const size_t o = (size_t)blockIdx.x * rows_stride;
    int carry = 0;
    for (int b0 = 0; b0 < n; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        const int v = i < n ? row_count[o + i] : 0;
        int tot;
        const int ex = block_exclusive_scan(v, s_scan, &tot);
        if (i < n) {
            row_start[o + i] = carry + ex;
            cursor[o + i] = carry + ex;
        }
        carry += tot;
    }
}

__global__ void k_bstereo_rows_fill(const orbgpu_keypoint* kps, const int* counts, int cap, const StereoPair* pairs,
                                    int rows_stride, int* cursor, int* row_keys, size_t key_stride) {
    const StereoPair& P = pairs[blockIdx.y];
    const int nR = min(counts[P.right], cap);
    int* cur = cursor + (size_t)blockIdx.y * rows_stride;
    int* keys = row_keys + blockIdx.y * key_stride;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nR; i += gridDim.x * blockDim.x) {
        int lo, hi;
        if (!stereo_rows_of(kps[(size_t)P.right * cap + i], P.lv, P.nRows, lo, hi)) continue;
        for (int yi = lo; yi <= hi; yi++) keys[atomicAdd(&cur[yi], 1)] = i;
    }
}

__global__ void k_bstereo_match(const orbgpu_keypoint* kps, const uint8_t* desc, const int* counts, int cap,
                                const StereoPair* pairs, int rows_stride, const int* row_start, const int* row_keys,
                                size_t key_stride, float* uright, float* depth, int* sad, int* status) {
    const StereoPair& P = pairs[blockIdx.y];
    const int iL = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (iL >= min(counts[P.left], cap)) return;
    const size_t p = blockIdx.y, l0 = (size_t)P.left * cap, r0 = (size_t)P.right * cap;
    stereo_match_warp(iL, kps + l0, desc + 32 * l0, kps + r0, desc + 32 * r0, P.lv, P.nRows,
                      row_start + p * rows_stride, row_keys + p * key_stride, P.bf, P.fx, uright + p * cap,
                      depth + p * cap, sad + p * cap, status);
}

__global__ void k_bstereo_median(const int* counts, int cap, const StereoPair* pairs, const int* sad, float* uright,
                                 float* depth, int* sort_buf, int sort_cap) {
    const StereoPair& P = pairs[blockIdx.x];
    const size_t p = blockIdx.x;
    stereo_median_block(min(counts[P.left], cap), sad + p * cap, uright + p * cap, depth + p * cap,
                        sort_buf + p * sort_cap, sort_cap, nullptr);
}

}  // namespace orbgpu

extern "C" int orbgpu_batch_compute_stereo_matches(orbgpu_batch* b, const orbgpu_keypoint* kps, const uint8_t* desc,
                                                   const int* counts, int npairs, const int* left_frame,
                                                   const int* right_frame, const float* bf, const float* fx,
                                                   float* uright, float* depth) {
    if (!b || b->nframes <= 0 || !kps || !desc || !counts || npairs < 0 || npairs > b->nframes ||
        (npairs > 0 && (!left_frame || !right_frame || !bf || !fx || !uright || !depth))) {
        orbgpu_set_last_error("invalid batched stereo arguments", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    if (npairs == 0) return ORBGPU_OK;
    const int cap = b->frame_cap, nl = b->nlevels;
    std::vector<StereoPair> hp(npairs);
    int max_rows = 1;
    float maxscale = 1.0f;
    for (int p = 0; p < npairs; p++) {
        const int lf = left_frame[p], rf = right_frame[p];
        if (lf < 0 || rf < 0 || lf >= b->nframes || rf >= b->nframes || !(bf[p] > 0.f) || !(fx[p] > 0.f)) {
            orbgpu_set_last_error("batched stereo: frame index or camera out of range", __FILE__, __LINE__);
            return ORBGPU_ERR_BAD_ARG;
        }
        const FramePlan* L = b->cur[lf];
        const FramePlan* R = b->cur[rf];
        if (L->w != R->w || L->h != R->h) {
            orbgpu_set_last_error("batched stereo: left and right frames differ in size", __FILE__, __LINE__);
            return ORBGPU_ERR_BAD_ARG;
        }
        StereoPair& P = hp[p];
        std::memset(&P, 0, sizeof(P));
        for (int l = 0; l < nl; l++) {
            P.lv.left[l] = b->arena + (size_t)lf * b->slot_bytes + L->layout.lv[l].pyr;
            P.lv.right[l] = b->arena + (size_t)rf * b->slot_bytes + R->layout.lv[l].pyr;
            P.lv.w[l] = L->geom[l].w;
            P.lv.h[l] = L->geom[l].h;
            P.lv.pitch[l] = L->geom[l].pitch;
            P.lv.scale[l] = L->tables.scale[l];
            P.lv.inv_scale[l] = 1.0f / L->tables.scale[l];
            maxscale = std::max(maxscale, P.lv.scale[l]);
        }
        P.lv.nlevels = nl;
        P.left = lf;
        P.right = rf;
        P.nRows = L->geom[0].h;
        P.bf = bf[p];
        P.fx = fx[p];
        max_rows = std::max(max_rows, P.nRows);
    }
    const int rows_stride = max_rows + 2;
    const int rows_per_key = 2 * (int)std::ceil(2.0f * maxscale) + 4;
    const size_t key_stride = (size_t)cap * rows_per_key;
    int sort_cap = 1;
    while (sort_cap < cap) sort_cap <<= 1;
    cudaStream_t st = b->stream;
    const size_t need = sizeof(StereoPair) * npairs + 3 * sizeof(int) * (size_t)npairs * rows_stride +
                        sizeof(int) * npairs * key_stride + sizeof(int) * (size_t)npairs * (cap + sort_cap) +
                        16 * 256;
    if (need > b->st_bytes) {
        ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
        if (b->st_scratch) cudaFree(b->st_scratch);
        b->st_scratch = nullptr;
        b->st_bytes = 0;
        ORBGPU_CUDA_TRY(dev_malloc(&b->st_scratch, need));
        b->st_bytes = need;
    }
    if (!b->st_pinned) ORBGPU_CUDA_TRY(cudaMallocHost(&b->st_pinned, 16));
    size_t off = 0;
    auto take = [&](size_t n) {
        off = (off + 255) & ~(size_t)255;
        uint8_t* q = b->st_scratch + off;
        off += n;
        return q;
    };
    StereoPair* d_pairs = (StereoPair*)take(sizeof(StereoPair) * npairs);
    int* row_count = (int*)take(sizeof(int) * (size_t)npairs * rows_stride);
    int* row_start = (int*)take(sizeof(int) * (size_t)npairs * rows_stride);
    int* cursor = (int*)take(sizeof(int) * (size_t)npairs * rows_stride);
    int* row_keys = (int*)take(sizeof(int) * npairs * key_stride);
    int* sad = (int*)take(sizeof(int) * (size_t)npairs * cap);
    int* sort_buf = (int*)take(sizeof(int) * (size_t)npairs * sort_cap);
    int* status = (int*)take(sizeof(int) * 4);
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(d_pairs, hp.data(), sizeof(StereoPair) * npairs, cudaMemcpyHostToDevice, st));
    ORBGPU_CUDA_TRY(cudaMemsetAsync(row_count, 0, sizeof(int) * (size_t)npairs * rows_stride, st));
    ORBGPU_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int) * 4, st));
    const dim3 gk((cap + 255) / 256, npairs);
    k_bstereo_rows_count<<<gk, 256, 0, st>>>(kps, counts, cap, d_pairs, rows_stride, row_count);
    k_bstereo_scan<<<npairs, 1024, 0, st>>>(row_count, d_pairs, rows_stride, row_start, cursor);
    k_bstereo_rows_fill<<<gk, 256, 0, st>>>(kps, counts, cap, d_pairs, rows_stride, cursor, row_keys, key_stride);
    const int wpb = 8;
    k_bstereo_match<<<dim3((cap + wpb - 1) / wpb, npairs), 32 * wpb, 0, st>>>(
        kps, desc, counts, cap, d_pairs, rows_stride, row_start, row_keys, key_stride, uright, depth, sad, status);
    k_bstereo_median<<<npairs, 1024, 0, st>>>(counts, cap, d_pairs, sad, uright, depth, sort_buf, sort_cap);
    ORBGPU_CUDA_TRY(cudaGetLastError());
    ORBGPU_CUDA_TRY(cudaMemcpyAsync(b->st_pinned, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    ORBGPU_CUDA_TRY(cudaStreamSynchronize(st));
    if (b->st_pinned[0]) {
        orbgpu_set_last_error("batched stereo: patch outside its level", __FILE__, __LINE__);
        return ORBGPU_ERR_BAD_ARG;
    }
    return ORBGPU_OK;
}

