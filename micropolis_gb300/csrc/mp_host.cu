// C ABI host layer (include/mp_core.h): patch store, frame orchestration of
// the plain per-pass path and of the batched path (one persistent launch per
// stage, the whole frame replayed as a CUDA graph), capacity growth on
// overflow, statistics and the headless framebuffer.
//
// Reference counterparts: Reyes::Renderer / RendererCL
// (src/Reyes/Renderer.h:29-45, src/Reyes/RendererCL.cpp:21-260), PatchIndex
// (src/Reyes/PatchIndex.cpp:57-146), Framebuffer (src/Reyes/Framebuffer.cpp),
// Projection (src/base/Projection.cpp:23-50).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/mp_core.h"
#include "mp_internal.h"

using namespace mp;

namespace {

struct Mesh {
    float4* cp = nullptr;
    int n_patches = 0;
    int type = 0;
    size_t n_points = 0;
};

template <typename T>
struct DevBuf {
    T* p = nullptr;
    long long n = 0;
};

}  // namespace

struct mp_ctx {
    mp_options opt{};
    std::string err;
    int device = 0;
    cudaStream_t own = nullptr, stream = nullptr;
    std::unordered_map<uint64_t, Mesh> meshes;

    bool in_frame = false;
    bool frame_valid = false;
    FrameDev fr{};
    std::vector<DrawDev> draws;       // draws of the current / last frame
    std::vector<float*> grad_ptr;     // per draw adjoint buffers

    // device state
    unsigned long long* ctrl = nullptr;
    unsigned long long* h_ctrl = nullptr;      // pinned readback
    DrawDev* d_draws = nullptr;
    DrawDev* h_draws = nullptr;                // pinned staging
    int* d_root_prefix = nullptr;
    int* h_root_prefix = nullptr;
    int draws_cap = 0;
    Queue q{};
    SubPatches sub{};                 // bound-and-split output, in emission order
    SubPatches sorted{};              // the same in canonical order (batched path, two launches)
    SortBuffers sb{};
    int sort_passes = 0;              // radix passes captured for this frame
    BigQuad* big = nullptr;
    long long big_cap = 0;
    float* mshade = nullptr;          // diffuse factor per micropolygon (batched path)
    long long mshade_cap = 0;
    Framebuffer fb{};

    // plain path
    Queue stack{};
    float4* pad_range = nullptr;
    uint2* pad_meta = nullptr;
    unsigned char* dec = nullptr;
    unsigned long long* keys = nullptr;
    unsigned long long* scan_state = nullptr;
    float4* pos_grid = nullptr;
    int2* pxl_grid = nullptr;
    float* depth_grid = nullptr;
    float4* color_grid = nullptr;
    int4* block_index = nullptr;
    long long pass_cap = 0;

    // graph of the batched frame
    cudaGraphExec_t graph = nullptr;
    int graph_draws = -1;
    long long graph_roots = -1;
    const void* graph_key[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // set by every reallocation of a buffer the graph's kernels use: a new
    // allocation may land at the freed one's address, so the pointers above
    // cannot tell that the captured sizes and pointers are stale
    bool graph_stale = false;

    int bns_grid = 0, raster_grid = 0, frame_grid = 0, sort_grid = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool stage_timing = false;
    void* staging = nullptr;          // pinned upload buffer (xyz of pageable sources)
    size_t staging_bytes = 0;
    float* xyz_dev = nullptr;         // uploaded xyz before widening to (x, y, z, 1)
    size_t xyz_cap = 0;               // floats
    cudaEvent_t sev[8] = {};
    mp_stats stats{};
    long long plain_bounds = 0, plain_passes = 0, plain_out = 0, plain_kernels = 0;
    long long plain_max_stack = 0;
    // stage events of the last frame (stage timing on): name, start, end in ns from the frame start
    struct TraceEvent {
        const char* name;
        long long start, end;
    };
    std::vector<TraceEvent> trace;
    unsigned char* image = nullptr;   // device buffer of mp_read_image
    long long image_bytes = 0;
    float* d_amp = nullptr;           // displacement amplitude multiplier read by the displacing kernels
    // asynchronous read-back: a device copy of one layer, sent to the host on its own stream
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_staged = nullptr, ev_copied = nullptr;
    cudaEvent_t ev_upload = nullptr;  // end of the last host-to-device copy of patch data
    float4* stage_color = nullptr;
    int* stage_depth = nullptr;
    bool readback_pending = false;
};

namespace {

mp_status fail(mp_ctx* c, mp_status st, const std::string& msg) {
    if (c) c->err = msg;
    return st;
}

mp_status cuda_fail(mp_ctx* c, cudaError_t e, const char* where) {
    cudaGetLastError();
    if (e == cudaErrorMemoryAllocation)
        return fail(c, MP_ERR_OUT_OF_MEMORY, std::string(where) + ": " + cudaGetErrorString(e));
    return fail(c, MP_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(expr)                                              \
    do {                                                      \
        cudaError_t e_ = (expr);                              \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #expr); \
    } while (0)

template <typename T>
cudaError_t dalloc(T** p, long long n) {
    *p = nullptr;
    if (n <= 0) n = 1;
    return cudaMalloc((void**)p, sizeof(T) * (size_t)n);
}

void dfree(void* p) {
    if (p) cudaFree(p);
}

// glm::perspective<float>(fovy, aspect, near, far), right-handed, depth -1..1,
// column-major (src/base/Projection.cpp:37-40).
void perspective(float fovy_rad, float aspect, float zn, float zf, float* m) {
    float th = std::tan(fovy_rad / 2.0f);
    std::memset(m, 0, 16 * sizeof(float));
    m[0] = 1.0f / (aspect * th);
    m[5] = 1.0f / th;
    m[10] = -(zf + zn) / (zf - zn);
    m[11] = -1.0f;
    m[14] = -(2.0f * zf * zn) / (zf - zn);
}

// first-frame guesses; both grow (and the frame is rendered again) on overflow
long long auto_queue_cap(long long roots) { return std::min(std::max(1LL << 22, roots * 32), 1LL << 28); }
long long auto_sub_cap(long long roots) { return std::min(std::max(1LL << 21, roots * 64), 1LL << 26); }

void free_sorted(mp_ctx* c) {
    dfree(c->sorted.range);
    dfree(c->sorted.meta);
    c->sorted = SubPatches{};
    for (int k = 0; k < 2; ++k) {
        dfree(c->sb.keys[k]);
        dfree(c->sb.vals[k]);
    }
    dfree(c->sb.hist);
    dfree(c->sb.counts);
    dfree(c->sb.group_counts);
    c->sb = SortBuffers{};
}

mp_status grow_queue(mp_ctx* c, long long need) {
    if (need <= c->q.capacity) return MP_OK;
    c->graph_stale = true;
    long long cap = std::max(need, c->q.capacity * 2);
    cudaFree(c->q.range);
    cudaFree(c->q.meta);
    cudaFree(c->q.seq);
    cudaFree(c->q.pts);
    cudaFree(c->q.path);
    c->q = Queue{};
    CK(dalloc(&c->q.range, cap));
    CK(dalloc(&c->q.meta, cap));
    CK(dalloc(&c->q.seq, cap));
    CK(dalloc(&c->q.pts, cap * kPtsPerSlot));
    CK(dalloc(&c->q.path, cap));
    CK(cudaMemsetAsync(c->q.seq, 0, sizeof(unsigned) * (size_t)cap, c->stream));
    c->q.capacity = cap;
    return MP_OK;
}

mp_status grow_sub(mp_ctx* c, long long need, bool keep) {
    const long long id_limit = (long long)(0xffffffffull / ((unsigned long long)c->fr.PS * c->fr.PS));
    if (need > id_limit) return fail(c, MP_ERR_OVERFLOW, "frame exceeds the 32-bit micropolygon id range");
    if (need <= c->sub.capacity) return MP_OK;
    c->graph_stale = true;
    long long cap = std::min(std::max(need, c->sub.capacity * 2), id_limit);
    SubPatches n{};
    CK(dalloc(&n.range, cap));
    CK(dalloc(&n.meta, cap));
    CK(dalloc(&n.seq, cap));
    CK(dalloc(&n.path, cap));
    CK(cudaMemsetAsync(n.seq, 0, sizeof(unsigned) * (size_t)cap, c->stream));
    n.capacity = cap;
    if (keep && c->sub.capacity > 0) {
        CK(cudaMemcpyAsync(n.range, c->sub.range, sizeof(float4) * (size_t)c->sub.capacity, cudaMemcpyDeviceToDevice,
                           c->stream));
        CK(cudaMemcpyAsync(n.meta, c->sub.meta, sizeof(int2) * (size_t)c->sub.capacity, cudaMemcpyDeviceToDevice,
                           c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    cudaFree(c->sub.range);
    cudaFree(c->sub.meta);
    cudaFree(c->sub.seq);
    cudaFree(c->sub.path);
    c->sub = n;
    // the canonical list and the sort's scratch follow the emitted list's capacity
    free_sorted(c);
    SubPatches o{};
    CK(dalloc(&o.range, cap));
    CK(dalloc(&o.meta, cap));
    o.capacity = cap;
    c->sorted = o;
    SortBuffers b{};
    b.capacity = cap;
    b.tiles = sort_tiles(cap);
    b.groups = (b.tiles + kSortGroup - 1) / kSortGroup;
    c->sb = b;
    for (int k = 0; k < 2; ++k) {
        CK(dalloc(&c->sb.keys[k], cap));
        CK(dalloc(&c->sb.vals[k], cap));
    }
    CK(dalloc(&c->sb.hist, 2 * kSortPasses * 256));
    CK(dalloc(&c->sb.counts, c->sb.tiles * 256));
    CK(dalloc(&c->sb.group_counts, kSortPasses * c->sb.groups * 256));
    CK(cudaMemsetAsync(c->sb.hist, 0, sizeof(unsigned) * 2 * kSortPasses * 256, c->stream));
    return MP_OK;
}

mp_status grow_big(mp_ctx* c, long long need) {
    if (need <= c->big_cap) return MP_OK;
    c->graph_stale = true;
    long long cap = std::max(need, c->big_cap * 2);
    cudaFree(c->big);
    c->big = nullptr;
    CK(dalloc(&c->big, cap));
    c->big_cap = cap;
    return MP_OK;
}

mp_status ensure_mshade(mp_ctx* c) {
    const long long need = c->sub.capacity * c->fr.PS * c->fr.PS;
    if (need <= c->mshade_cap) return MP_OK;
    c->graph_stale = true;
    dfree(c->mshade);
    c->mshade = nullptr;
    c->mshade_cap = 0;
    CK(dalloc(&c->mshade, need));
    c->mshade_cap = need;
    return MP_OK;
}

mp_status ensure_draws(mp_ctx* c, int n) {
    if (n <= c->draws_cap) return MP_OK;
    c->graph_stale = true;
    int cap = std::max(n, std::max(4, c->draws_cap * 2));
    // earlier draws of a plain frame may still be read by queued kernels: keep them
    CK(cudaStreamSynchronize(c->stream));
    DrawDev* nd = nullptr;
    CK(dalloc(&nd, cap));
    if (c->d_draws && c->draws_cap > 0)
        CK(cudaMemcpy(nd, c->d_draws, sizeof(DrawDev) * (size_t)c->draws_cap, cudaMemcpyDeviceToDevice));
    cudaFree(c->d_draws);
    cudaFree(c->d_root_prefix);
    cudaFreeHost(c->h_draws);
    cudaFreeHost(c->h_root_prefix);
    c->d_draws = nd;
    c->d_root_prefix = nullptr;
    c->h_draws = nullptr;
    c->h_root_prefix = nullptr;
    CK(dalloc(&c->d_root_prefix, cap + 1));
    CK(cudaMallocHost((void**)&c->h_draws, sizeof(DrawDev) * (size_t)cap));
    CK(cudaMallocHost((void**)&c->h_root_prefix, sizeof(int) * (size_t)(cap + 1)));
    c->draws_cap = cap;
    return MP_OK;
}

void invalidate_graph(mp_ctx* c) {
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    c->graph_draws = -1;
}

mp_status check_status(mp_ctx* c, unsigned long long st) {
    switch ((int)st) {
        case kOk: return MP_OK;
        case kErrOverflow: return fail(c, MP_ERR_OVERFLOW, "capacity exceeded");
        case kErrTimeout: return fail(c, MP_ERR_TIMEOUT, "bounded device wait expired");
        default: return fail(c, MP_ERR_CUDA, "device status " + std::to_string(st));
    }
}

unsigned long long hc(const mp_ctx* c, int w) { return c->h_ctrl[w * kCtrlStride]; }

mp_status read_ctrl(mp_ctx* c) {
    CK(cudaMemcpyAsync(c->h_ctrl, c->ctrl, sizeof(unsigned long long) * kNumCtrl * kCtrlStride,
                       cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return MP_OK;
}

// ---------------------------------------------------------------------------
// plain per-pass path for one draw (src/Reyes/RendererCL.cpp:170-260 with the
// BOUNDED bound&split of src/Reyes/BoundNSplitCLBounded.cpp:170-214)

mp_status ensure_plain(mp_ctx* c, long long need_stack) {
    const long long P = c->opt.reyes_patches_per_pass;
    if (c->pass_cap < P) {
        dfree(c->pad_range); dfree(c->pad_meta); dfree(c->dec); dfree(c->keys); dfree(c->scan_state);
        dfree(c->pos_grid); dfree(c->pxl_grid); dfree(c->depth_grid); dfree(c->color_grid); dfree(c->block_index);
        const long long G2 = (long long)(c->fr.PS + 1) * (c->fr.PS + 1), Q = (long long)c->fr.PS * c->fr.PS;
        CK(dalloc(&c->pad_range, P));
        CK(dalloc(&c->pad_meta, P));
        CK(dalloc(&c->dec, P));
        CK(dalloc(&c->keys, P));
        CK(dalloc(&c->scan_state, scan_state_words(P)));
        CK(dalloc(&c->pos_grid, P * G2));
        CK(dalloc(&c->pxl_grid, P * G2));
        CK(dalloc(&c->depth_grid, P * G2));
        CK(dalloc(&c->color_grid, P * Q));
        CK(dalloc(&c->block_index, P * (Q / 64)));
        c->pass_cap = P;
    }
    if (need_stack > c->stack.capacity) {
        long long cap = std::max(need_stack, c->stack.capacity * 2);
        Queue n{};
        CK(dalloc(&n.range, cap));
        CK(dalloc(&n.meta, cap));
        n.capacity = cap;
        if (c->stack.capacity > 0) {
            CK(cudaMemcpyAsync(n.range, c->stack.range, sizeof(float4) * (size_t)c->stack.capacity,
                               cudaMemcpyDeviceToDevice, c->stream));
            CK(cudaMemcpyAsync(n.meta, c->stack.meta, sizeof(uint2) * (size_t)c->stack.capacity,
                               cudaMemcpyDeviceToDevice, c->stream));
            CK(cudaStreamSynchronize(c->stream));
        }
        dfree(c->stack.range);
        dfree(c->stack.meta);
        c->stack = n;
    }
    return MP_OK;
}

mp_status plain_draw(mp_ctx* c, int draw_index) {
    const DrawDev& d = c->draws[(size_t)draw_index];
    const long long P = c->opt.reyes_patches_per_pass;
    // upload this draw's constants
    CK(cudaMemcpyAsync(c->d_draws + draw_index, &c->draws[(size_t)draw_index], sizeof(DrawDev),
                       cudaMemcpyHostToDevice, c->stream));
    mp_status st = ensure_plain(c, (long long)d.n_patches + 2 * P * (c->opt.max_split_depth + 2));
    if (st) return st;
    launch_bns_init_stack(c->stack, draw_index, d.n_patches, c->stream);
    c->plain_kernels += 1;
    long long h = d.n_patches;
    while (h > 0) {
        long long b = std::min(h, P);
        h -= b;
        if (h + 2 * b > c->stack.capacity) {
            st = ensure_plain(c, h + 2 * b);
            if (st) return st;
        }
        if (c->plain_out + b > c->sub.capacity) {
            st = grow_sub(c, c->plain_out + b, true);
            if (st) return st;
        }
        c->plain_max_stack = std::max(c->plain_max_stack, h + b);
        if (c->stage_timing) CK(cudaEventRecord(c->sev[0], c->stream));
        launch_bns_pass(c->d_draws, c->fr, c->stack, h, (int)b, c->pad_range, c->pad_meta, c->dec, c->keys,
                        c->scan_state, c->sub, c->plain_out, c->ctrl, c->opt.spin_limit, c->stream);
        CK(cudaGetLastError());
        c->plain_kernels += 3;   // bound, scan, move
        if (c->stage_timing) CK(cudaEventRecord(c->sev[1], c->stream));
        st = read_ctrl(c);
        if (c->stage_timing) {
            float ms = 0, t0 = 0;
            cudaEventElapsedTime(&ms, c->sev[0], c->sev[1]);
            cudaEventElapsedTime(&t0, c->ev0, c->sev[0]);
            c->stats.stage_ms[1] += ms;
            c->trace.push_back({"bound & split", (long long)(t0 * 1e6), (long long)((t0 + ms) * 1e6)});
        }
        if (st) return st;
        if (hc(c, kStatus)) return check_status(c, hc(c, kStatus));
        unsigned long long tot = hc(c, kScanTotal);
        long long draws_n = (long long)(tot & 0x7fffffffull), splits = (long long)(tot >> 31);
        h += 2 * splits;
        c->plain_bounds += b;
        c->plain_passes += 1;
        if (draws_n > 0) {
            int n = (int)draws_n;
            const bool tm = c->stage_timing;
            if (tm) CK(cudaEventRecord(c->sev[2], c->stream));
            launch_dice_grid(c->d_draws, c->fr, c->sub, c->plain_out, n, c->pos_grid, c->pxl_grid, c->depth_grid,
                             c->stream);
            if (tm) CK(cudaEventRecord(c->sev[3], c->stream));
            launch_shade_grid(c->d_draws, c->fr, c->sub, c->plain_out, n, c->pos_grid, c->pxl_grid, c->block_index,
                              c->color_grid, c->stream);
            if (tm) CK(cudaEventRecord(c->sev[4], c->stream));
            launch_sample_grid(c->d_draws, c->fr, c->sub, c->plain_out, n, c->block_index, c->pxl_grid,
                               c->depth_grid, c->fb, c->big, c->big_cap, c->ctrl, c->stream);
            if (tm) CK(cudaEventRecord(c->sev[5], c->stream));
            launch_raster_big(c->d_draws, c->fr, c->fb, c->big, c->big_cap, c->ctrl, c->stream);
            CK(cudaMemsetAsync(c->ctrl + kBigCount * kCtrlStride, 0, sizeof(unsigned long long), c->stream));
            if (tm) CK(cudaEventRecord(c->sev[6], c->stream));
            launch_pass_resolve(c->fr, c->fb, c->plain_out, n, c->color_grid, c->stream);
            c->plain_kernels += 5;   // dice, shade, sample, exact slow raster, pass resolve
            if (tm) CK(cudaEventRecord(c->sev[7], c->stream));
            CK(cudaGetLastError());
            if (tm) {
                CK(cudaEventSynchronize(c->sev[7]));
                float ms = 0;
                const int slot[5] = {2, 4, 5, 3, 6};  // dice, shade, sample, slow raster, pass resolve
                // command names of the reference's trace (tools/trace_summary.py maps these)
                static const char* const names[5] = {"dice", "shade", "sample", "sample", "sample"};
                for (int k = 0; k < 5; ++k) {
                    float t0 = 0;
                    cudaEventElapsedTime(&ms, c->sev[2 + k], c->sev[3 + k]);
                    cudaEventElapsedTime(&t0, c->ev0, c->sev[2 + k]);
                    c->stats.stage_ms[slot[k]] += ms;
                    c->trace.push_back({names[k], (long long)(t0 * 1e6), (long long)((t0 + ms) * 1e6)});
                }
            }
            c->plain_out += n;
        }
    }
    return MP_OK;
}

// ---------------------------------------------------------------------------
// batched path: the whole frame as one graph

// The overlapped frame kernel carries the CPU bound criterion only.
bool overlapped(const mp_ctx* c) { return c->opt.overlap && c->fr.criterion == MP_BOUND_CPU; }

int bns_blocks(const mp_ctx* c) {
    if (c->opt.bns_blocks > 0) return std::min(c->opt.bns_blocks, c->frame_grid);
    return std::max(1, c->frame_grid / 3);
}

// The sub-patch list the frame's micropolygon ids index: the canonical list
// on the batched path in separate launches, else the list as emitted.
const SubPatches& final_list(const mp_ctx* c) {
    return c->opt.path == MP_PATH_BATCHED && !overlapped(c) ? c->sorted : c->sub;
}

// Kernel launches of one batched frame.
long long batched_kernels(const mp_ctx* c) {
    // clear+reset, (bound-and-split, canonical sort, dice+raster | overlapped), slow raster, resolve
    if (overlapped(c)) return 4;
    return 6;
}

void launch_sort(mp_ctx* c) {
    launch_canonical_sort(c->d_root_prefix, c->sub, c->sorted, c->sb, c->ctrl, c->opt.spin_limit, c->sort_passes,
                          c->sort_grid, c->stream);
}

// Stages of a batched frame in launch order: the mp_stats.stage_ms slot
// and the trace name of each.  Names are the reference's command names,
// which its tools/trace_summary.py maps: bound-and-split is "bound & split";
// the canonical-order sort, a radix sort built on prefix sums, takes the
// name of the reference's prefix-sum command, "accumulate" (both count as
// subdivision there); the fused dice+shade+raster launch is "dice", the
// exact slow raster "sample", the colour resolve "shade".
struct StageMark {
    int slot;
    const char* name;
};
constexpr int kBatchedStages = 6;
constexpr StageMark kStageMarks[kBatchedStages] = {{0, "clear framebuffer"}, {1, "bound & split"}, {5, "accumulate"},
                                                   {2, "dice"},              {3, "sample"},        {4, "shade"}};

// Event sev[k] marks the end of stage k - 1 (sev[0] the start).  Inside a
// stream capture the record becomes an event node of the graph.
void mark(mp_ctx* c, int k, bool capturing) {
    if (capturing)
        cudaEventRecordWithFlags(c->sev[k], c->stream, cudaEventRecordExternal);
    else
        cudaEventRecord(c->sev[k], c->stream);
}

// The device work of one batched frame, from the upload of the draw
// constants to the read-back of the control words, with an event after each
// stage: bound-and-split, canonical order and rasterization as separate
// launches, or (option `overlap`) bound-and-split and rasterization as one
// overlapped launch over the list in emission order.
void enqueue_frame(mp_ctx* c, int n, long long roots, bool capturing) {
    cudaMemcpyAsync(c->d_draws, c->h_draws, sizeof(DrawDev) * (size_t)n, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->d_root_prefix, c->h_root_prefix, sizeof(int) * (size_t)(n + 1), cudaMemcpyHostToDevice,
                    c->stream);
    mark(c, 0, capturing);
    launch_clear(c->fb, c->fr, 0, c->stream, c->ctrl, roots);
    mark(c, 1, capturing);
    if (overlapped(c)) {
        // one launch, reported as dice+raster; bound-and-split and sort show 0
        mark(c, 2, capturing);
        mark(c, 3, capturing);
        launch_frame_kernel(c->d_draws, c->d_root_prefix, n, c->fr, c->q, c->sub, c->fb, c->mshade, c->big, c->big_cap,
                            c->ctrl, c->opt.spin_limit, c->frame_grid, bns_blocks(c), c->opt.dice_group, c->stream);
    } else {
        launch_bns_persistent(c->d_draws, c->d_root_prefix, n, c->fr, c->q, c->sub, c->ctrl, c->bns_grid,
                              c->opt.spin_limit, c->stream);
        mark(c, 2, capturing);
        launch_sort(c);
        mark(c, 3, capturing);
        launch_raster_fused(c->d_draws, c->fr, c->sorted, c->fb, c->mshade, c->big, c->big_cap, c->ctrl,
                            c->raster_grid, c->opt.dice_group, c->stream);
    }
    mark(c, 4, capturing);
    launch_raster_big(c->d_draws, c->fr, c->fb, c->big, c->big_cap, c->ctrl, c->stream);
    mark(c, 5, capturing);
    launch_resolve(c->d_draws, c->fr, final_list(c), c->fb, c->mshade, c->stream);
    mark(c, 6, capturing);
    cudaMemcpyAsync(c->h_ctrl, c->ctrl, sizeof(unsigned long long) * kNumCtrl * kCtrlStride, cudaMemcpyDeviceToHost,
                    c->stream);
}

// Stage times and trace lines of the last batched frame (its events have completed).
void read_stage_events(mp_ctx* c) {
    c->trace.clear();
    for (double& v : c->stats.stage_ms) v = 0;
    float t = 0;
    for (int k = 0; k < kBatchedStages; ++k) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, c->sev[k], c->sev[k + 1]) != cudaSuccess) ms = 0;
        c->stats.stage_ms[kStageMarks[k].slot] = ms;
        if (!(overlapped(c) && (k == 1 || k == 2)))
            c->trace.push_back({kStageMarks[k].name, (long long)(t * 1e6), (long long)((t + ms) * 1e6)});
        t += ms;
    }
    cudaGetLastError();
}

mp_status capture_frame(mp_ctx* c, int n, long long roots) {
    invalidate_graph(c);
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_frame(c, n, roots, true);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
    c->graph_draws = n;
    c->graph_roots = roots;
    c->graph_stale = false;
    c->graph_key[0] = c->q.range;
    c->graph_key[1] = c->sub.range;
    c->graph_key[2] = c->big;
    c->graph_key[3] = c->d_draws;
    c->graph_key[4] = c->mshade;
    c->graph_key[5] = c->sorted.range;
    return MP_OK;
}

mp_status batched_frame(mp_ctx* c) {
    const int n = (int)c->draws.size();
    mp_status st = ensure_draws(c, n);
    if (st) return st;
    long long roots = 0;
    c->h_root_prefix[0] = 0;
    for (int i = 0; i < n; ++i) {
        c->h_draws[i] = c->draws[(size_t)i];
        c->h_draws[i].grad_cp = (size_t)i < c->grad_ptr.size() ? c->grad_ptr[(size_t)i] : nullptr;
        roots += c->draws[(size_t)i].n_patches;
        c->h_root_prefix[i + 1] = (int)roots;
    }
    if (roots >= (1LL << 31)) return fail(c, MP_ERR_INVALID_ARG, "more than 2^31 patches in one frame");
    long long qcap = c->opt.queue_capacity > 0 ? c->opt.queue_capacity : auto_queue_cap(roots);
    long long scap = c->opt.subpatch_capacity > 0 ? c->opt.subpatch_capacity : auto_sub_cap(roots);
    if ((st = grow_queue(c, qcap)) || (st = grow_sub(c, scap, false)) || (st = grow_big(c, 1 << 16)) ||
        (st = ensure_mshade(c)))
        return st;
    const int passes = canonical_sort_passes(c->opt.max_split_depth, roots);
    if (passes != c->sort_passes) {
        c->sort_passes = passes;
        c->graph_stale = true;
    }
    for (int attempt = 0; attempt < 8; ++attempt) {
        if (c->stage_timing) {
            // the graph's launches issued one by one (same events)
            CK(cudaEventRecord(c->ev0, c->stream));
            enqueue_frame(c, n, roots, false);
            CK(cudaEventRecord(c->ev1, c->stream));
            CK(cudaStreamSynchronize(c->stream));
            CK(cudaGetLastError());
        } else {
            if (!c->graph || c->graph_stale || c->graph_draws != n || c->graph_roots != roots ||
                c->graph_key[0] != c->q.range || c->graph_key[1] != c->sub.range || c->graph_key[2] != c->big ||
                c->graph_key[3] != c->d_draws || c->graph_key[4] != c->mshade || c->graph_key[5] != c->sorted.range) {
                st = capture_frame(c, n, roots);
                if (st) return st;
            }
            CK(cudaEventRecord(c->ev0, c->stream));
            CK(cudaGraphLaunch(c->graph, c->stream));
            CK(cudaEventRecord(c->ev1, c->stream));
            CK(cudaStreamSynchronize(c->stream));
        }
        read_stage_events(c);
        unsigned long long status = hc(c, kStatus);
        if (status != kErrOverflow) {
            if (status) return check_status(c, status);
            break;
        }
        // regrow what overflowed and render the frame again
        long long pushed = (long long)(hc(c, kQTail) >> 32) - roots;
        long long outc = (long long)hc(c, kOutCount);
        long long bigc = (long long)hc(c, kBigCount);
        if (pushed > c->q.capacity && (st = grow_queue(c, pushed + pushed / 2))) return st;
        if (outc > c->sub.capacity && ((st = grow_sub(c, outc + outc / 4, false)) || (st = ensure_mshade(c))))
            return st;
        if (bigc > c->big_cap && (st = grow_big(c, bigc * 2))) return st;
        if (attempt == 7) {
            char msg[256];
            std::snprintf(msg, sizeof(msg),
                          "capacity still exceeded after regrowth (queue %lld/%lld, sub-patches %lld/%lld, "
                          "slow quads %lld/%lld)",
                          pushed, c->q.capacity, outc, c->sub.capacity, bigc, c->big_cap);
            return fail(c, MP_ERR_OVERFLOW, msg);
        }
    }
    return MP_OK;
}

mp_status fill_draw(mp_ctx* c, const Mesh& m, const float* mv, const mp_projection* proj, const float* color,
                    int view, DrawDev& d) {
    if (!proj) return fail(c, MP_ERR_INVALID_ARG, "projection is NULL");
    if (proj->viewport[0] != c->opt.window_size[0] || proj->viewport[1] != c->opt.window_size[1])
        return fail(c, MP_ERR_INVALID_ARG, "projection viewport must equal window_size");
    if (view < 0 || view >= c->opt.batch_views) return fail(c, MP_ERR_INVALID_ARG, "view out of range");
    if (!(proj->near_plane > 0) || !(proj->fovy_deg > 0)) return fail(c, MP_ERR_INVALID_ARG, "bad projection");
    std::memset(&d, 0, sizeof(d));
    d.cp = m.cp;
    d.n_patches = m.n_patches;
    d.type = m.type;
    d.view = view;
    std::memcpy(d.mv, mv, sizeof(d.mv));
    const int W = proj->viewport[0], H = proj->viewport[1];
    const float fovy = proj->fovy_deg;
    const float aspect = float(W) / H;
    perspective((float)(fovy * M_PI / 180), aspect, proj->near_plane, 10000.0f, d.proj);
    for (int i = 0; i < 4; ++i) d.color[i] = color ? color[i] : 1.0f;
    // src/base/Projection.cpp:23-35
    float fy = 1.0f / (float)std::tan(fovy * M_PI / 360);
    float fx = fy / aspect;
    d.vpx = W / 2.0f;
    d.vpy = H / 2.0f;
    d.fx = fx * d.vpx;
    d.fy = fy * d.vpy;
    d.near_plane = proj->near_plane;
    d.near_eps = (float)((double)proj->near_plane * 0.1);
    d.cull_ribbon = c->opt.cull_ribbon;
    d.vx = W;
    d.vy = H;
    return MP_OK;
}

void untile(const float* src, const int* dsrc, float* dst, int* ddst, int W, int H) {
    const int gx = W / 8;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            long long t = ((long long)(x / 8 + gx * (y / 8)) << 6) + (x & 7) + ((y & 7) << 3);
            long long o = (long long)y * W + x;
            if (dst) std::memcpy(dst + 4 * o, src + 4 * t, 4 * sizeof(float));
            if (ddst) ddst[o] = dsrc[t];
        }
}

}  // namespace

// ===========================================================================
// C ABI

extern "C" {

void mp_options_default(mp_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->window_size[0] = 1600;   // reyes.options:2
    o->window_size[1] = 1200;
    o->reyes_patch_size = 8;    // :14
    o->bound_n_split_limit = 8; // :17
    o->reyes_patches_per_pass = 100000;  // :44
    o->cull_ribbon = 32;        // :20
    o->max_split_depth = 23;    // :40
    o->bound_sample_rate = 3;   // :37
    o->subpixel_bits = 6;       // :50
    o->framebuffer_tile_size = 8;  // :47
    o->backface_culling = 1;    // :31
    o->displacement = 0;        // :67
    o->displacement_amplitude = 1.0f;
    o->clear_color[0] = 0.1f;   // :11
    o->clear_color[1] = 0.1f;
    o->clear_color[2] = 0.7f;
    o->clear_color[3] = 0.0f;
    o->batch_views = 1;
    o->path = MP_PATH_BATCHED;
    o->spin_limit = 1 << 20;
}

mp_status mp_create(const mp_options* opts, mp_ctx** out) {
    if (!out) return MP_ERR_INVALID_ARG;
    *out = nullptr;
    mp_options o;
    if (opts) o = *opts; else mp_options_default(&o);
    const int W = o.window_size[0], H = o.window_size[1];
    if (W <= 0 || H <= 0 || W % 8 || H % 8 || W > 4096 || H > 4096) return MP_ERR_INVALID_ARG;
    if (o.reyes_patch_size != 8 && o.reyes_patch_size != 16) return MP_ERR_INVALID_ARG;
    if (o.subpixel_bits < 1 || o.subpixel_bits > 8 || ((long long)std::max(W, H) << o.subpixel_bits) > (1LL << 18))
        return MP_ERR_INVALID_ARG;
    if (o.bound_sample_rate != 3 || o.framebuffer_tile_size != 8) return MP_ERR_INVALID_ARG;
    if (o.max_split_depth < 0 || o.max_split_depth > 254) return MP_ERR_INVALID_ARG;
    if (o.reyes_patches_per_pass < 1 || o.batch_views < 1 || o.batch_views > 65536) return MP_ERR_INVALID_ARG;
    if (o.path != MP_PATH_PLAIN && o.path != MP_PATH_BATCHED) return MP_ERR_INVALID_ARG;
    if (o.spin_limit <= 0) o.spin_limit = 1 << 20;
    if (o.bound_criterion != MP_BOUND_CPU && o.bound_criterion != MP_BOUND_GPU) return MP_ERR_INVALID_ARG;
    if (o.raster_tile == 0) o.raster_tile = 8;
    if (o.raster_tile != 8 && o.raster_tile != 16 && o.raster_tile != 32) return MP_ERR_INVALID_ARG;
    if (o.dice_group == 0) o.dice_group = o.reyes_patch_size == 16 ? 6 : 11;
    if (o.reyes_patch_size == 8 && o.dice_group != 8 && o.dice_group != 11 && o.dice_group != 16 &&
        o.dice_group != 22)
        return MP_ERR_INVALID_ARG;
    if (o.reyes_patch_size == 16 && o.dice_group != 2 && o.dice_group != 3 && o.dice_group != 4 &&
        o.dice_group != 6)
        return MP_ERR_INVALID_ARG;
    mp_ctx* c = new mp_ctx();
    c->opt = o;
    cudaError_t e = cudaGetDevice(&c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return MP_ERR_CUDA;
    }
    c->stream = c->own;
    FrameDev& fr = c->fr;
    fr.W = W;
    fr.H = H;
    fr.PS = o.reyes_patch_size;
    fr.shift = o.subpixel_bits;
    fr.limit = o.bound_n_split_limit;
    fr.max_depth = o.max_split_depth;
    fr.backface = o.backface_culling ? 1 : 0;
    fr.displacement = o.displacement ? 1 : 0;
    fr.fdisp[0] = 0.04f * o.displacement_amplitude;
    fr.fdisp[1] = 0.02f * o.displacement_amplitude;
    fr.fdisp[2] = 0.01f * o.displacement_amplitude;
    // src/Reyes/Framebuffer.cpp:65-68
    fr.clear[0] = powf(o.clear_color[0], 2.2f);
    fr.clear[1] = powf(o.clear_color[1], 2.2f);
    fr.clear[2] = powf(o.clear_color[2], 2.2f);
    fr.clear[3] = 1000.0f;
    fr.gx = W / 8;
    fr.gy = H / 8;
    mp_status st = MP_OK;
    auto ck = [&](cudaError_t err, const char* w) {
        if (err != cudaSuccess && st == MP_OK) st = cuda_fail(c, err, w);
    };
    ck(dalloc(&c->ctrl, (long long)kNumCtrl * kCtrlStride), "ctrl");
    ck(dalloc(&c->d_amp, 1), "amplitude");
    ck(cudaMemcpyAsync(c->d_amp, &o.displacement_amplitude, sizeof(float), cudaMemcpyHostToDevice, c->stream),
       "amplitude");
    fr.amp_dev = c->d_amp;
    ck(cudaMemsetAsync(c->ctrl, 0, sizeof(unsigned long long) * kNumCtrl * kCtrlStride, c->stream), "ctrl memset");
    ck(cudaMallocHost((void**)&c->h_ctrl, sizeof(unsigned long long) * kNumCtrl * kCtrlStride), "h_ctrl");
    c->fb.pixels = (long long)W * H;
    c->fb.views = o.batch_views;
    // the key buffer is sized for the largest key tile (32 px) so the tile can change per frame
    c->fb.key_pixels = (long long)((W + 31) / 32 * 32) * ((H + 31) / 32 * 32);
    fr.kshift = o.raster_tile == 32 ? 5 : o.raster_tile == 16 ? 4 : 3;
    fr.kgx = (W + (1 << fr.kshift) - 1) >> fr.kshift;
    fr.criterion = o.bound_criterion;
    ck(dalloc(&c->fb.keys, c->fb.key_pixels * c->fb.views), "fb keys");
    ck(dalloc(&c->fb.color, c->fb.pixels * c->fb.views), "fb color");
    ck(dalloc(&c->fb.depth, c->fb.pixels * c->fb.views), "fb depth");
    ck(cudaEventCreate(&c->ev0), "event");
    ck(cudaEventCreate(&c->ev1), "event");
    for (auto& e : c->sev) ck(cudaEventCreate(&e), "event");
    if (st == MP_OK) st = ensure_draws(c, 4);
    if (st == MP_OK) st = grow_big(c, 1 << 16);
    if (st == MP_OK) {
        c->bns_grid = bns_persistent_grid(fr.criterion);
        c->raster_grid = raster_fused_grid(fr.PS, o.dice_group);
        c->frame_grid = frame_kernel_grid(fr.PS, o.dice_group);
        c->sort_grid = canonical_sort_grid();
        launch_clear(c->fb, c->fr, 1, c->stream);
        ck(cudaStreamSynchronize(c->stream), "init");
    }
    if (st != MP_OK) {
        mp_destroy(c);
        return st;
    }
    *out = c;
    return MP_OK;
}

void mp_destroy(mp_ctx* c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->copy_stream) {
        cudaStreamSynchronize(c->copy_stream);
        cudaStreamDestroy(c->copy_stream);
    }
    if (c->ev_staged) cudaEventDestroy(c->ev_staged);
    if (c->ev_upload) cudaEventDestroy(c->ev_upload);
    if (c->ev_copied) cudaEventDestroy(c->ev_copied);
    dfree(c->stage_color);
    dfree(c->stage_depth);
    invalidate_graph(c);
    for (auto& kv : c->meshes) dfree(kv.second.cp);
    dfree(c->ctrl);
    dfree(c->d_amp);
    if (c->h_ctrl) cudaFreeHost(c->h_ctrl);
    if (c->staging) cudaFreeHost(c->staging);
    dfree(c->xyz_dev);
    dfree(c->d_draws);
    dfree(c->d_root_prefix);
    if (c->h_draws) cudaFreeHost(c->h_draws);
    if (c->h_root_prefix) cudaFreeHost(c->h_root_prefix);
    dfree(c->q.range); dfree(c->q.meta); dfree(c->q.seq); dfree(c->q.pts); dfree(c->q.path);
    dfree(c->sub.range); dfree(c->sub.meta); dfree(c->sub.seq); dfree(c->sub.path);
    free_sorted(c);
    dfree(c->big);
    dfree(c->mshade);
    dfree(c->fb.keys); dfree(c->fb.color); dfree(c->fb.depth);
    dfree(c->stack.range); dfree(c->stack.meta);
    dfree(c->pad_range); dfree(c->pad_meta); dfree(c->dec); dfree(c->keys); dfree(c->scan_state);
    dfree(c->pos_grid); dfree(c->pxl_grid); dfree(c->depth_grid); dfree(c->color_grid); dfree(c->block_index);
    dfree(c->image);
    for (auto& e : c->sev)
        if (e) cudaEventDestroy(e);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
}

const char* mp_last_error(const mp_ctx* c) { return c ? c->err.c_str() : "null context"; }

mp_status mp_set_stream(mp_ctx* c, void* stream) {
    if (!c) return MP_ERR_INVALID_ARG;
    if (c->in_frame) return fail(c, MP_ERR_STATE, "cannot change stream inside a frame");
    cudaStream_t s = stream ? (cudaStream_t)stream : c->own;
    if (s != c->stream) invalidate_graph(c);
    c->stream = s;
    return MP_OK;
}

mp_status mp_are_patches_loaded(mp_ctx* c, uint64_t handle, int32_t* loaded) {
    if (!c || !loaded) return MP_ERR_INVALID_ARG;
    *loaded = c->meshes.count(handle) ? 1 : 0;
    return MP_OK;
}

static mp_status load_common(mp_ctx* c, uint64_t handle, const void* src, size_t n_points, mp_patch_type type,
                             bool device) {
    if (!c) return MP_ERR_INVALID_ARG;
    // Scene::draw loads on first use inside a frame (src/micropolis/Scene.cpp:186-188);
    // only replacing a handle that this frame may already reference is refused
    if (c->in_frame && c->meshes.count(handle) && !c->draws.empty())
        return fail(c, MP_ERR_STATE, "reloading a handle after this frame's first draw");
    if (type != MP_BEZIER && type != MP_GREGORY) return fail(c, MP_ERR_INVALID_ARG, "bad patch type");
    const size_t per = type == MP_BEZIER ? 16 : 20;
    if (n_points % per) return fail(c, MP_ERR_INVALID_ARG, "point count is not a whole number of patches");
    if (n_points / per >= (1u << 31)) return fail(c, MP_ERR_INVALID_ARG, "too many patches");
    if (n_points && !src) return fail(c, MP_ERR_INVALID_ARG, "null patch data");
    Mesh m;
    auto it = c->meshes.find(handle);
    if (it != c->meshes.end() && it->second.n_points == n_points && it->second.type == type) {
        m = it->second;  // same size: reuse the device buffer
    } else {
        if (it != c->meshes.end()) {
            CK(cudaStreamSynchronize(c->stream));
            dfree(it->second.cp);
            c->meshes.erase(it);
        }
        m.n_patches = (int)(n_points / per);
        m.type = type;
        m.n_points = n_points;
        CK(dalloc(&m.cp, (long long)n_points));
    }
    if (n_points) {
        if (device) {
            CK(cudaMemcpyAsync(m.cp, src, sizeof(float4) * n_points, cudaMemcpyDeviceToDevice, c->stream));
            if (!c->in_frame) CK(cudaStreamSynchronize(c->stream));
        } else {
            // src/Reyes/PatchIndex.cpp:83-98: upload the vec3 data and widen it
            // to (x, y, z, 1) on the device.  Page-locked sources are copied
            // directly; others go through a pinned staging buffer reused
            // across loads.
            const size_t bytes = sizeof(float) * 3 * n_points;
            if (c->xyz_cap < 3 * n_points) {
                CK(cudaStreamSynchronize(c->stream));
                dfree(c->xyz_dev);
                c->xyz_dev = nullptr;
                c->xyz_cap = 0;
                CK(dalloc(&c->xyz_dev, (long long)(3 * n_points)));
                c->xyz_cap = 3 * n_points;
            }
            cudaPointerAttributes attr{};
            const bool pinned = cudaPointerGetAttributes(&attr, src) == cudaSuccess && attr.type == cudaMemoryTypeHost;
            cudaGetLastError();  // a pageable pointer is not an error
            const void* h = src;
            if (!pinned) {
                if (c->staging_bytes < bytes) {
                    CK(cudaStreamSynchronize(c->stream));
                    if (c->staging) cudaFreeHost(c->staging);
                    c->staging = nullptr;
                    c->staging_bytes = 0;
                    CK(cudaMallocHost(&c->staging, bytes));
                    c->staging_bytes = bytes;
                } else {
                    CK(cudaStreamSynchronize(c->stream));  // the previous upload has left the staging buffer
                }
                std::memcpy(c->staging, src, bytes);
                h = c->staging;
            }
            if (!c->ev_upload) CK(cudaEventCreateWithFlags(&c->ev_upload, cudaEventDisableTiming));
            CK(cudaMemcpyAsync(c->xyz_dev, h, bytes, cudaMemcpyHostToDevice, c->stream));
            CK(cudaEventRecord(c->ev_upload, c->stream));
            launch_widen_points(c->xyz_dev, m.cp, (long long)n_points, c->stream);
            CK(cudaGetLastError());
            // The call returns once the source has been read (the caller's
            // page-locked buffer is read asynchronously; outside a frame the
            // load is blocking like the reference's); the widening runs in
            // stream order before any frame that reads the patches.
            if (pinned || !c->in_frame) CK(cudaEventSynchronize(c->ev_upload));
        }
    }
    c->meshes[handle] = m;
    return MP_OK;
}

mp_status mp_load_patches(mp_ctx* c, uint64_t handle, const float* xyz, size_t n_points, mp_patch_type type) {
    return load_common(c, handle, xyz, n_points, type, false);
}

mp_status mp_load_patches_device(mp_ctx* c, uint64_t handle, const void* dev_xyz1, size_t n_points,
                                 mp_patch_type type) {
    return load_common(c, handle, dev_xyz1, n_points, type, true);
}

mp_status mp_set_displacement_amplitude(mp_ctx* c, float amp) {
    if (!c || !std::isfinite(amp)) return MP_ERR_INVALID_ARG;
    if (c->in_frame) return fail(c, MP_ERR_STATE, "amplitude change inside a frame");
    c->opt.displacement_amplitude = amp;
    c->fr.fdisp[0] = 0.04f * amp;
    c->fr.fdisp[1] = 0.02f * amp;
    c->fr.fdisp[2] = 0.01f * amp;
    // the kernels read the multiplier from device memory: a stream-ordered
    // write, no new graph (a pageable source is staged before the call returns)
    CK(cudaMemcpyAsync(c->d_amp, &amp, sizeof(float), cudaMemcpyHostToDevice, c->stream));
    return MP_OK;
}

mp_status mp_set_displacement_amplitude_device(mp_ctx* c, const void* amp_dev) {
    if (!c || !amp_dev) return MP_ERR_INVALID_ARG;
    if (c->in_frame) return fail(c, MP_ERR_STATE, "amplitude change inside a frame");
    CK(cudaMemcpyAsync(c->d_amp, amp_dev, sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    return MP_OK;
}

mp_status mp_update_patches_device(mp_ctx* c, uint64_t handle, const void* dev_xyz1) {
    if (!c || !dev_xyz1) return MP_ERR_INVALID_ARG;
    auto it = c->meshes.find(handle);
    if (it == c->meshes.end()) return fail(c, MP_ERR_NOT_LOADED, "handle not loaded");
    CK(cudaMemcpyAsync(it->second.cp, dev_xyz1, sizeof(float4) * it->second.n_points, cudaMemcpyDeviceToDevice,
                       c->stream));
    return MP_OK;
}

mp_status mp_delete_patches(mp_ctx* c, uint64_t handle) {
    if (!c) return MP_ERR_INVALID_ARG;
    if (c->in_frame) return fail(c, MP_ERR_STATE, "delete_patches inside a frame");
    auto it = c->meshes.find(handle);
    if (it == c->meshes.end()) return fail(c, MP_ERR_NOT_LOADED, "handle not loaded");
    cudaStreamSynchronize(c->stream);
    dfree(it->second.cp);
    c->meshes.erase(it);
    invalidate_graph(c);
    c->frame_valid = false;
    return MP_OK;
}

mp_status mp_prepare(mp_ctx* c) {
    if (!c) return MP_ERR_INVALID_ARG;
    if (c->in_frame) return fail(c, MP_ERR_STATE, "prepare called twice");
    c->in_frame = true;
    c->frame_valid = false;
    c->draws.clear();
    c->plain_bounds = c->plain_passes = c->plain_out = 0;
    c->plain_kernels = 0;
    c->plain_max_stack = 0;
    c->trace.clear();
    for (double& v : c->stats.stage_ms) v = 0;
    if (c->opt.path == MP_PATH_PLAIN) {
        CK(cudaEventRecord(c->ev0, c->stream));
        launch_clear(c->fb, c->fr, 1, c->stream, c->ctrl, 0);
        c->plain_kernels += 1;
        CK(cudaGetLastError());
    }
    return MP_OK;
}

mp_status mp_draw_patches_view(mp_ctx* c, uint64_t handle, const float mv[16], const mp_projection* proj,
                               const float color[4], int32_t view) {
    if (!c || !mv) return MP_ERR_INVALID_ARG;
    if (!c->in_frame) return fail(c, MP_ERR_STATE, "draw_patches outside prepare/finish");
    auto it = c->meshes.find(handle);
    if (it == c->meshes.end()) return fail(c, MP_ERR_NOT_LOADED, "handle not loaded");
    if (c->draws.size() >= (1u << 24)) return fail(c, MP_ERR_INVALID_ARG, "too many draws in one frame");
    DrawDev d;
    mp_status st = fill_draw(c, it->second, mv, proj, color, view, d);
    if (st) return st;
    c->draws.push_back(d);
    if (c->opt.path == MP_PATH_PLAIN) {
        st = ensure_draws(c, (int)c->draws.size());
        if (st) return st;
        if (d.n_patches > 0) return plain_draw(c, (int)c->draws.size() - 1);
    }
    return MP_OK;
}

mp_status mp_draw_views(mp_ctx* c, int32_t n, const mp_view* views) {
    if (!c || n < 0 || (n > 0 && !views)) return MP_ERR_INVALID_ARG;
    for (int32_t i = 0; i < n; ++i) {
        const mp_view& v = views[i];
        mp_status st = mp_draw_patches_view(c, v.handle, v.modelview, &v.proj, v.color, v.view);
        if (st) return st;
    }
    return MP_OK;
}

mp_status mp_draw_patches(mp_ctx* c, uint64_t handle, const float mv[16], const mp_projection* proj,
                          const float color[4]) {
    return mp_draw_patches_view(c, handle, mv, proj, color, 0);
}

mp_status mp_finish(mp_ctx* c) {
    if (!c) return MP_ERR_INVALID_ARG;
    if (!c->in_frame) return fail(c, MP_ERR_STATE, "finish without prepare");
    c->in_frame = false;
    mp_status st = MP_OK;
    if (c->opt.path == MP_PATH_BATCHED) {
        st = batched_frame(c);
        if (st) return st;
        c->stats.subpatches = std::min((long long)hc(c, kOutCount), c->sub.capacity);
        c->stats.bounds = (long long)(hc(c, kQTail) >> 32);
        c->stats.passes = 1;
        c->stats.kernels = batched_kernels(c);
    } else {
        CK(cudaEventRecord(c->ev1, c->stream));
        st = read_ctrl(c);
        if (st) return st;
        if (hc(c, kStatus)) return check_status(c, hc(c, kStatus));
        c->stats.subpatches = c->plain_out;
        c->stats.bounds = c->plain_bounds;
        c->stats.passes = c->plain_passes;
        c->stats.kernels = c->plain_kernels;
        if (c->stage_timing) {
            float ms = 0;
            cudaEventElapsedTime(&ms, c->ev0, c->ev1);
            double sum = 0;
            for (int k = 0; k < 7; ++k) sum += c->stats.stage_ms[k];
            c->stats.stage_ms[7] = ms - sum;
        }
    }
    c->stats.micropolygons = c->stats.subpatches * c->fr.PS * c->fr.PS;
    c->stats.fragments = (long long)hc(c, kFragments);
    c->stats.big_quads = (long long)hc(c, kBigTotal);
    float ms = 0;
    if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) c->stats.gpu_ms = ms;
    cudaGetLastError();
    c->frame_valid = true;
    return MP_OK;
}

mp_status mp_set_stage_timing(mp_ctx* c, int32_t on) {
    if (!c) return MP_ERR_INVALID_ARG;
    if (c->in_frame) return fail(c, MP_ERR_STATE, "stage timing change inside a frame");
    c->stage_timing = on != 0;
    return MP_OK;
}

// Appends printf-formatted text at *pos; false once the buffer is full.
bool put(char* buf, size_t cap, size_t* pos, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    const int n = std::vsnprintf(buf + *pos, cap - *pos, fmt, ap);
    va_end(ap);
    if (n < 0 || (size_t)n >= cap - *pos) {
        buf[*pos] = 0;
        return false;
    }
    *pos += (size_t)n;
    return true;
}

mp_status mp_dump_trace(mp_ctx* c, char* buf, size_t cap) {
    if (!c || !buf || cap == 0) return MP_ERR_INVALID_ARG;
    buf[0] = 0;
    size_t pos = 0;
    const char* queue = c->opt.path == MP_PATH_PLAIN ? "plain" : "batched";
    if (!c->frame_valid) return fail(c, MP_ERR_STATE, "no finished frame");
    if (c->trace.empty())
        return fail(c, MP_ERR_STATE,
                    "the plain path times its commands only with stage timing on (mp_set_stage_timing)");
    long long prev_end = 0;
    for (size_t i = 0; i < c->trace.size(); ++i) {
        const auto& e = c->trace[i];
        // each command depends on the one before it on the stream, so it
        // starts no earlier than that one ends (event times are rounded to
        // the nanosecond independently)
        const long long start = std::max(e.start, prev_end), end = std::max(e.end, start);
        prev_end = end;
        bool ok = i == 0 ? put(buf, cap, &pos, "%s@%s:%lld:%lld:%lld:%lld:%zu:\n", e.name, queue, start, start,
                               start, end, i)
                         : put(buf, cap, &pos, "%s@%s:%lld:%lld:%lld:%lld:%zu:%zu\n", e.name, queue, start, start,
                               start, end, i, i - 1);
        if (!ok) return MP_ERR_OVERFLOW;
    }
    return MP_OK;
}

mp_status mp_dump_stats(mp_ctx* c, char* buf, size_t cap) {
    if (!c || !buf || cap == 0) return MP_ERR_INVALID_ARG;
    buf[0] = 0;
    // device memory by use (the reference's opencl_memory_by_use)
    long long cp = 0, input = 0;
    for (const auto& m : c->meshes) cp += (long long)m.second.n_points * (long long)sizeof(float4);
    for (const auto& d : c->draws) input += d.n_patches;
    const long long G2 = (long long)(c->fr.PS + 1) * (c->fr.PS + 1), Q = (long long)c->fr.PS * c->fr.PS;
    const struct {
        const char* use;
        long long bytes;
    } mem[] = {
        {"control points", cp},
        {"work queue", c->q.capacity * (long long)(sizeof(float4) * (1 + kPtsPerSlot) + sizeof(uint2) +
                                                   2 * sizeof(unsigned))},
        {"sub-patch list", c->sub.capacity * (long long)(sizeof(float4) + sizeof(int2) + 2 * sizeof(unsigned))},
        {"canonical sub-patch list", c->sorted.capacity * (long long)(sizeof(float4) + sizeof(int2))},
        {"canonical order sort", c->sb.capacity * 2 * (long long)(sizeof(unsigned long long) + sizeof(unsigned)) +
                                     (c->sb.tiles + kSortPasses * c->sb.groups) * 256 * (long long)sizeof(unsigned)},
        {"diffuse factors", c->mshade_cap * (long long)sizeof(float)},
        {"framebuffer", c->fb.key_pixels * c->fb.views * 8 + c->fb.pixels * c->fb.views * 20},
        {"exact slow raster quads", c->big_cap * (long long)sizeof(BigQuad)},
        {"bound and split stack", c->stack.capacity * (long long)(sizeof(float4) + sizeof(uint2))},
        {"pass grids", c->pass_cap * (G2 * (16 + 8 + 4) + Q * 16 + (Q / 64) * 16 + 16 + 8 + 1 + 8)},
        {"image", c->image_bytes},
    };
    long long total = 0;
    for (const auto& m : mem) total += m.bytes;
    size_t pos = 0;
    bool ok = put(buf, cap, &pos, "opencl_mem = %lld;\n", total);
    for (const auto& m : mem)
        if (m.bytes > 0) ok = ok && put(buf, cap, &pos, "opencl_mem@%s = %lld;\n", m.use, m.bytes);
    const long long max_patches = c->opt.path == MP_PATH_PLAIN
                                      ? c->plain_max_stack
                                      : (long long)(hc(c, kQTail) >> 32) - (long long)hc(c, kRoots);
    ok = ok && put(buf, cap, &pos, "opengl_mem = 0;\n");
    ok = ok && put(buf, cap, &pos, "max_patches = %lld;\n", max_patches);
    ok = ok && put(buf, cap, &pos, "patches_per_frame = %lld;\n", (long long)c->stats.subpatches);
    ok = ok && put(buf, cap, &pos, "processed_patches_per_frame = %lld;\n", (long long)c->stats.bounds);
    ok = ok && put(buf, cap, &pos, "pass_count = %lld;\n", (long long)c->stats.passes);
    ok = ok && put(buf, cap, &pos, "total_input_patches = %lld;\n", input);
    ok = ok && put(buf, cap, &pos, "bound_n_split_balance = ;");
    return ok ? MP_OK : MP_ERR_OVERFLOW;
}

mp_status mp_read_image(mp_ctx* c, int32_t view, uint8_t* rgb) {
    if (!c || !rgb || view < 0 || view >= c->fb.views) return MP_ERR_INVALID_ARG;
    const long long n = (long long)c->fr.W * c->fr.H * 3;
    if (c->image_bytes < n) {
        dfree(c->image);
        c->image = nullptr;
        c->image_bytes = 0;
        CK(dalloc(&c->image, n));
        c->image_bytes = n;
    }
    launch_image(c->fb.color + view * c->fb.pixels, c->fr, c->image, c->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(rgb, c->image, (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return MP_OK;
}

mp_status mp_framebuffer(mp_ctx* c, void** color_dev, void** depth_dev, int32_t* width, int32_t* height,
                         int32_t* views) {
    if (!c) return MP_ERR_INVALID_ARG;
    if (color_dev) *color_dev = c->fb.color;
    if (depth_dev) *depth_dev = c->fb.depth;
    if (width) *width = c->fr.W;
    if (height) *height = c->fr.H;
    if (views) *views = c->fb.views;
    return MP_OK;
}

mp_status mp_read_framebuffer(mp_ctx* c, int32_t view, float* color, int32_t* depth, int32_t linear) {
    if (!c || view < 0 || view >= c->fb.views) return MP_ERR_INVALID_ARG;
    const long long n = c->fb.pixels;
    std::vector<float> tc;
    std::vector<int> td;
    float* cdst = color;
    int* ddst = depth;
    if (linear) {
        if (color) { tc.resize((size_t)n * 4); cdst = tc.data(); }
        if (depth) { td.resize((size_t)n); ddst = td.data(); }
    }
    if (cdst) CK(cudaMemcpyAsync(cdst, c->fb.color + view * n, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    if (ddst) CK(cudaMemcpyAsync(ddst, c->fb.depth + view * n, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (linear) untile(cdst, ddst, color, depth, c->fr.W, c->fr.H);
    return MP_OK;
}

mp_status mp_read_framebuffer_async(mp_ctx* c, int32_t view, float* color, int32_t* depth) {
    if (!c || view < 0 || view >= c->fb.views || (!color && !depth)) return MP_ERR_INVALID_ARG;
    if (!c->frame_valid) return fail(c, MP_ERR_STATE, "no finished frame");
    if (c->in_frame) return fail(c, MP_ERR_STATE, "read-back inside a frame");
    const long long n = c->fb.pixels;
    if (!c->copy_stream) {
        // first use: the staging layer, a copy stream and its events
        CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&c->ev_staged, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c->ev_copied, cudaEventDisableTiming));
        CK(dalloc(&c->stage_color, n));
        CK(dalloc(&c->stage_depth, n));
    }
    // the staging layer is free once the previous read-back has left it
    if (c->readback_pending) CK(cudaStreamWaitEvent(c->stream, c->ev_copied, 0));
    if (color)
        CK(cudaMemcpyAsync(c->stage_color, c->fb.color + view * n, sizeof(float4) * (size_t)n,
                           cudaMemcpyDeviceToDevice, c->stream));
    if (depth)
        CK(cudaMemcpyAsync(c->stage_depth, c->fb.depth + view * n, sizeof(int) * (size_t)n,
                           cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaEventRecord(c->ev_staged, c->stream));
    CK(cudaStreamWaitEvent(c->copy_stream, c->ev_staged, 0));
    if (color)
        CK(cudaMemcpyAsync(color, c->stage_color, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToHost,
                           c->copy_stream));
    if (depth)
        CK(cudaMemcpyAsync(depth, c->stage_depth, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->copy_stream));
    CK(cudaEventRecord(c->ev_copied, c->copy_stream));
    c->readback_pending = true;
    return MP_OK;
}

mp_status mp_wait_read_framebuffer(mp_ctx* c) {
    if (!c) return MP_ERR_INVALID_ARG;
    if (!c->readback_pending) return MP_OK;
    CK(cudaEventSynchronize(c->ev_copied));
    c->readback_pending = false;
    return MP_OK;
}

mp_status mp_copy_framebuffer_device(mp_ctx* c, int32_t view, void* color_dev, void* depth_dev) {
    if (!c || view < 0 || view >= c->fb.views) return MP_ERR_INVALID_ARG;
    const long long n = c->fb.pixels;
    if (color_dev)
        CK(cudaMemcpyAsync(color_dev, c->fb.color + view * n, sizeof(float4) * (size_t)n, cudaMemcpyDeviceToDevice,
                           c->stream));
    if (depth_dev)
        CK(cudaMemcpyAsync(depth_dev, c->fb.depth + view * n, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice,
                           c->stream));
    return MP_OK;
}

mp_status mp_read_visibility(mp_ctx* c, int32_t view, int64_t* ids) {
    if (!c || !ids || view < 0 || view >= c->fb.views) return MP_ERR_INVALID_ARG;
    if (!c->frame_valid) return fail(c, MP_ERR_STATE, "no finished frame");
    const long long nk = c->fb.key_pixels;
    std::vector<unsigned long long> k((size_t)nk);
    CK(cudaMemcpyAsync(k.data(), c->fb.keys + view * nk, sizeof(unsigned long long) * (size_t)nk,
                       cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const int W = c->fr.W, H = c->fr.H, ks = c->fr.kshift, m = (1 << ks) - 1;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const long long o = ((long long)(x / 8 + c->fr.gx * (y / 8)) << 6) + (x & 7) + ((y & 7) << 3);
            const long long ki = ((long long)((x >> ks) + c->fr.kgx * (y >> ks)) << (2 * ks)) + (x & m) + ((y & m) << ks);
            const unsigned long long key = k[(size_t)ki];
            ids[o] = key == kClearKey ? -1 : (int64_t)(key & 0xffffffffull);
        }
    return MP_OK;
}

mp_status mp_subpatches(mp_ctx* c, int64_t* count, int32_t* draw, int32_t* pid, float* range, int64_t cap) {
    if (!c) return MP_ERR_INVALID_ARG;
    if (!c->frame_valid) return fail(c, MP_ERR_STATE, "no finished frame");
    long long n = c->stats.subpatches;
    if (count) *count = n;
    long long k = std::min<long long>(n, cap);
    if (k <= 0) return MP_OK;
    std::vector<float4> r((size_t)k);
    std::vector<int2> m((size_t)k);
    const SubPatches& list = final_list(c);
    CK(cudaMemcpyAsync(r.data(), list.range, sizeof(float4) * (size_t)k, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(m.data(), list.meta, sizeof(int2) * (size_t)k, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    for (long long i = 0; i < k; ++i) {
        if (draw) draw[i] = m[(size_t)i].y;
        if (pid) pid[i] = m[(size_t)i].x;
        if (range) {
            range[4 * i] = r[(size_t)i].x;
            range[4 * i + 1] = r[(size_t)i].y;
            range[4 * i + 2] = r[(size_t)i].z;
            range[4 * i + 3] = r[(size_t)i].w;
        }
    }
    return MP_OK;
}

mp_status mp_stats_get(mp_ctx* c, mp_stats* s) {
    if (!c || !s) return MP_ERR_INVALID_ARG;
    *s = c->stats;
    return MP_OK;
}

mp_status mp_dice_subpatches(mp_ctx* c, int32_t draw, int64_t n, const int32_t* pid, const float* range, float* pos,
                             int32_t* pxl, float* depth) {
    if (!c || n < 0 || (n && (!pid || !range))) return MP_ERR_INVALID_ARG;
    if (!c->frame_valid || draw < 0 || draw >= (int)c->draws.size()) return fail(c, MP_ERR_STATE, "no such draw");
    if (n == 0) return MP_OK;
    for (long long i = 0; i < n; ++i)
        if (pid[i] < 0 || pid[i] >= c->draws[(size_t)draw].n_patches)
            return fail(c, MP_ERR_INVALID_ARG, "patch id out of range");
    const long long G2 = (long long)(c->fr.PS + 1) * (c->fr.PS + 1);
    SubPatches tmp{};
    float4* dpos = nullptr;
    int2* dpxl = nullptr;
    float* ddep = nullptr;
    std::vector<float4> r((size_t)n);
    std::vector<int2> m((size_t)n);
    for (long long i = 0; i < n; ++i) {
        r[(size_t)i] = make_float4(range[4 * i], range[4 * i + 1], range[4 * i + 2], range[4 * i + 3]);
        m[(size_t)i] = make_int2(pid[i], draw);
    }
    mp_status st = MP_OK;
    auto run = [&]() -> mp_status {
        CK(dalloc(&tmp.range, n));
        CK(dalloc(&tmp.meta, n));
        tmp.capacity = n;
        CK(dalloc(&dpos, n * G2));
        CK(dalloc(&dpxl, n * G2));
        CK(dalloc(&ddep, n * G2));
        CK(cudaMemcpyAsync(c->d_draws, c->draws.data(), sizeof(DrawDev) * c->draws.size(), cudaMemcpyHostToDevice,
                           c->stream));
        CK(cudaMemcpyAsync(tmp.range, r.data(), sizeof(float4) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(tmp.meta, m.data(), sizeof(int2) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
        launch_dice_debug(c->d_draws, c->fr, tmp, (int)n, dpos, dpxl, ddep, c->stream);
        CK(cudaGetLastError());
        if (pos) CK(cudaMemcpyAsync(pos, dpos, sizeof(float4) * (size_t)(n * G2), cudaMemcpyDeviceToHost, c->stream));
        if (pxl) CK(cudaMemcpyAsync(pxl, dpxl, sizeof(int2) * (size_t)(n * G2), cudaMemcpyDeviceToHost, c->stream));
        if (depth) CK(cudaMemcpyAsync(depth, ddep, sizeof(float) * (size_t)(n * G2), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        return MP_OK;
    };
    st = run();
    dfree(tmp.range); dfree(tmp.meta); dfree(dpos); dfree(dpxl); dfree(ddep);
    c->graph_key[3] = nullptr;  // draws buffer content changed: recapture the graph next frame
    return st;
}

mp_status mp_set_grad_buffer(mp_ctx* c, int32_t draw, void* grad_dev) {
    if (!c || draw < 0) return MP_ERR_INVALID_ARG;
    if ((size_t)draw >= c->grad_ptr.size()) c->grad_ptr.resize((size_t)draw + 1, nullptr);
    c->grad_ptr[(size_t)draw] = (float*)grad_dev;
    return MP_OK;
}

mp_status mp_backward(mp_ctx* c, int32_t view, const void* grad_color_dev, void* grad_amp_dev) {
    if (!c || !grad_color_dev) return MP_ERR_INVALID_ARG;
    if (!c->frame_valid || c->opt.path != MP_PATH_BATCHED) return fail(c, MP_ERR_STATE, "backward needs a batched frame");
    if (view < 0 || view >= c->fb.views) return fail(c, MP_ERR_INVALID_ARG, "view out of range");
    const int n = (int)c->draws.size();
    for (int i = 0; i < n; ++i) {
        c->h_draws[i] = c->draws[(size_t)i];
        c->h_draws[i].grad_cp = (size_t)i < c->grad_ptr.size() ? c->grad_ptr[(size_t)i] : nullptr;
    }
    CK(cudaMemcpyAsync(c->d_draws, c->h_draws, sizeof(DrawDev) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    launch_adjoint(c->d_draws, c->fr, final_list(c), c->fb, (const float4*)grad_color_dev, (float*)grad_amp_dev, view,
                   c->stream);
    CK(cudaGetLastError());
    return MP_OK;
}

mp_status mp_inclusive_scan(mp_ctx* c, const int32_t* in, int32_t* out, int64_t n) {
    if (!c || n < 0 || (n && (!in || !out))) return MP_ERR_INVALID_ARG;
    if (n == 0) return MP_OK;
    int *din = nullptr, *dout = nullptr;
    unsigned long long* state = nullptr;
    mp_status st = MP_OK;
    auto run = [&]() -> mp_status {
        CK(dalloc(&din, n));
        CK(dalloc(&dout, n));
        CK(dalloc(&state, scan_state_words(n) + 2 * n));
        CK(cudaMemcpyAsync(din, in, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
        launch_inclusive_scan_i32(din, dout, n, state, c->ctrl, c->opt.spin_limit, c->stream);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(out, dout, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
        mp_status s2 = read_ctrl(c);
        if (s2) return s2;
        if (hc(c, kStatus)) return check_status(c, hc(c, kStatus));
        return MP_OK;
    };
    st = run();
    dfree(din); dfree(dout); dfree(state);
    return st;
}

mp_status mp_atomic_bench(mp_ctx* c, int64_t n_slots, int64_t n_ops, int32_t pattern, double* rate) {
    if (!c || n_slots < 64 || n_ops <= 0 || !rate) return MP_ERR_INVALID_ARG;
    unsigned long long* buf = nullptr;
    mp_status st = MP_OK;
    auto run = [&]() -> mp_status {
        CK(dalloc(&buf, n_slots));
        CK(cudaMemsetAsync(buf, 0xff, sizeof(unsigned long long) * (size_t)n_slots, c->stream));
        launch_atomic_bench(buf, n_slots, n_ops, pattern, c->stream);  // warm-up
        CK(cudaEventRecord(c->ev0, c->stream));
        launch_atomic_bench(buf, n_slots, n_ops, pattern, c->stream);
        CK(cudaEventRecord(c->ev1, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        CK(cudaGetLastError());
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        *rate = (double)n_ops / (ms * 1e-3);
        return MP_OK;
    };
    st = run();
    dfree(buf);
    return st;
}

}  // extern "C"
