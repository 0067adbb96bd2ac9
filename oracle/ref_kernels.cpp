// The reference's own dice / shade / sample / clear kernels (kernels/*.cl,
// rewritten by clshim/rewrite.py into _ref/kernels/ and compiled as C++ over
// clshim/cl_shim.h) run on the CPU with the launch geometry of
// src/Reyes/RendererCL.cpp:203-260, after the reference's CPU bound-and-split
// (ref_pin.cpp).  TEST INFRASTRUCTURE ONLY: it pins the oracle's kernel
// restatement to the reference's kernel source.
//
// Work-items run as fibers (ucontext): one work-group at a time per host
// thread, each work-item a fiber that switches back to the scheduler at a
// barrier; work-group local memory is `static thread_local` (rewrite.py).
// Work-groups are spread over host threads.
#include <ucontext.h>

#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

#include "clshim/cl_shim.h"

// The reference's compile-time constants (RendererCL.cpp:73-87 and
// BoundNSplitCLBounded.cpp:61-62), run-time here.
struct RefkConfig {
    int patch_size = 8, tile_size = 8, pxl_shift = 6, backface = 1, displacement = 0;
    int2 grid_size, vp_min_px, vp_max_px, vp_size_px, fb_size;
    float cull_ribbon = 32.0f;
    int max_split_depth = 22;
};
static RefkConfig g_cfg;
#define PATCH_SIZE (g_cfg.patch_size)
#define TILE_SIZE (g_cfg.tile_size)
#define GRID_SIZE (g_cfg.grid_size)
#define VIEWPORT_MIN_PIXEL (g_cfg.vp_min_px)
#define VIEWPORT_MAX_PIXEL (g_cfg.vp_max_px)
#define VIEWPORT_SIZE_PIXEL (g_cfg.vp_size_px)
#define FRAMEBUFFER_SIZE (g_cfg.fb_size)
#define BACKFACE_CULLING (g_cfg.backface)
#define PXLCOORD_SHIFT (g_cfg.pxl_shift)
#define DISPLACEMENT (g_cfg.displacement)
#define CULL_RIBBON (g_cfg.cull_ribbon)
#define MAX_SPLIT_DEPTH (g_cfg.max_split_depth)
#define BOUND_SAMPLE_RATE 3   // reyes.options bound_sample_rate (src/Reyes/config.xml:92)

// ---------------------------------------------------------------------------
// fiber runtime

namespace {

constexpr int kMaxItems = 256;
constexpr size_t kStack = 64 * 1024;

struct Item {
    size_t gid[3], lid[3], grp[3];
    ucontext_t ctx;
    int state;   // 0 runnable, 1 at a barrier, 2 finished
};

struct Fibers {
    Item items[kMaxItems];
    std::vector<char> stacks;
    ucontext_t sched;
    int n = 0, cur = 0;
    const std::function<void()>* body = nullptr;
    Fibers() : stacks((size_t)kMaxItems * kStack) {}
};

thread_local Fibers* tf = nullptr;

void trampoline() {
    (*tf->body)();
    tf->items[tf->cur].state = 2;
}

// Runs work-group `grp` of a launch with local size loc over `body`.
void run_group(const std::function<void()>& body, const size_t grp[3], const size_t loc[3]) {
    Fibers& f = *tf;
    f.body = &body;
    f.n = (int)(loc[0] * loc[1] * loc[2]);
    int k = 0;
    for (size_t z = 0; z < loc[2]; ++z)
        for (size_t y = 0; y < loc[1]; ++y)
            for (size_t x = 0; x < loc[0]; ++x, ++k) {
                Item& it = f.items[k];
                it.lid[0] = x; it.lid[1] = y; it.lid[2] = z;
                for (int d = 0; d < 3; ++d) it.grp[d] = grp[d];
                it.gid[0] = grp[0] * loc[0] + x;
                it.gid[1] = grp[1] * loc[1] + y;
                it.gid[2] = grp[2] * loc[2] + z;
                getcontext(&it.ctx);
                it.ctx.uc_stack.ss_sp = f.stacks.data() + (size_t)k * kStack;
                it.ctx.uc_stack.ss_size = kStack;
                it.ctx.uc_link = &f.sched;
                makecontext(&it.ctx, trampoline, 0);
                it.state = 0;
            }
    while (true) {
        bool live = false;
        for (int i = 0; i < f.n; ++i) {
            if (f.items[i].state == 2) continue;
            f.items[i].state = 0;
            f.cur = i;
            swapcontext(&f.sched, &f.items[i].ctx);
            if (f.items[i].state != 2) live = true;
        }
        if (!live) break;   // every work-item finished; else all wait at a barrier: resume them
    }
}

// A launch: global size glb, local size loc, work-groups over `threads` host threads.
void launch(const std::function<void()>& body, const size_t glb[3], const size_t loc[3], int threads) {
    const size_t ng[3] = {glb[0] / loc[0], glb[1] / loc[1], glb[2] / loc[2]};
    const size_t total = ng[0] * ng[1] * ng[2];
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        Fibers f;
        tf = &f;
        size_t g;
        while ((g = next.fetch_add(1)) < total) {
            const size_t grp[3] = {g % ng[0], (g / ng[0]) % ng[1], g / (ng[0] * ng[1])};
            run_group(body, grp, loc);
        }
        tf = nullptr;
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
}

}  // namespace

size_t get_global_id(int d) { return tf->items[tf->cur].gid[d]; }
size_t get_local_id(int d) { return tf->items[tf->cur].lid[d]; }
size_t get_group_id(int d) { return tf->items[tf->cur].grp[d]; }
void barrier(int) {
    Item& it = tf->items[tf->cur];
    it.state = 1;
    swapcontext(&it.ctx, &tf->sched);
}

// ---------------------------------------------------------------------------
// the reference's kernels

#include "_ref/kernels/utility.h"
namespace refk_reyes {
#include "_ref/kernels/reyes.inc"
}
namespace refk_fb {
#include "_ref/kernels/framebuffer.inc"
}
namespace refk_bezier {
#define eval_patch eval_bezier_patch
#include "_ref/kernels/dice.inc"
#undef eval_patch
}
namespace refk_gregory {
#define eval_patch eval_gregory_patch
#include "_ref/kernels/dice.inc"
#undef eval_patch
}
namespace refk_bound_bezier {
#define eval_patch eval_bezier_patch
#include "_ref/kernels/bound_n_split.h"
#undef eval_patch
}
namespace refk_bound_gregory {
#define eval_patch eval_gregory_patch
#include "_ref/kernels/bound_n_split.h"
#undef eval_patch
}

// ---------------------------------------------------------------------------
// frame driver

extern "C" {
long refpin_bound_n_split(const float* cp_in, int n_patches, int type, const float* mv16, float fovy,
                          float near_plane, int w, int h, float ribbon, float limit, int max_split_depth, int* pid,
                          float* range, long cap);
void refpin_projection_matrix(float fovy, float near_plane, int w, int h, float* out16);
void refpin_screen_params(float fovy, float near_plane, int w, int h, float* f2, float* vp2);

// The reference's GPU bound-and-split for one draw: bound() of
// kernels/bound_n_split.h:42-100 per range, with the projection record of
// init_projection_buffer (BoundNSplitCLBounded.cpp:108-121), the split of
// the move kernel (kernels/bound_n_split_multipass.cl:103-128: children at
// depth + 1 around c = (rmin + rmax) * 0.5f) and DRAW ranges emitted, over a
// LIFO stack.  The emitted set does not depend on the order of visits.
// Writes at most cap records; returns the count, or -1 past 2^26 ranges.
long refk_bound_n_split_gpu(const float* cp_in, int n_patches, int type, const float* mv16, float fovy,
                            float near_plane, int w, int h, float ribbon, float limit, int max_split_depth, int* pid,
                            float* range, long cap) {
    g_cfg.cull_ribbon = ribbon;
    g_cfg.max_split_depth = max_split_depth;
    const int per = type == 0 ? 16 : 20;
    std::vector<float4> patch((size_t)n_patches * per);
    for (size_t k = 0; k < patch.size(); ++k)
        patch[k] = float4(cp_in[3 * k], cp_in[3 * k + 1], cp_in[3 * k + 2], 1.0f);
    float proj16[16], f2[2], vp2[2];
    refpin_projection_matrix(fovy, near_plane, w, h, proj16);
    refpin_screen_params(fovy, near_plane, w, h, f2, vp2);
    projection P;
    for (int c = 0; c < 4; ++c) P.proj.m[c] = float4(proj16[4 * c], proj16[4 * c + 1], proj16[4 * c + 2], proj16[4 * c + 3]);
    P.screen_matrix.m[0] = float2(vp2[0], 0.0f);
    P.screen_matrix.m[1] = float2(0.0f, vp2[1]);
    P.fovy = fovy;
    P.f = float2(f2[0], f2[1]);
    P.near = near_plane;
    P.far = 1000.0f;   // Projection::far() (src/base/Projection.h:49)
    P.screen_size = int2(w, h);
    matrix4 mv;
    for (int c = 0; c < 4; ++c) mv.m[c] = float4(mv16[4 * c], mv16[4 * c + 1], mv16[4 * c + 2], mv16[4 * c + 3]);
    struct R { int pid; uchar depth; float2 mn, mx; };
    std::vector<R> stack;
    for (int i = n_patches - 1; i >= 0; --i) stack.push_back(R{i, 0, float2(0, 0), float2(1, 1)});
    long n = 0, visits = 0;
    while (!stack.empty()) {
        R r = stack.back();
        stack.pop_back();
        if (++visits > (1L << 26)) return -1;
        const uchar flag = type == 0
            ? refk_bound_bezier::bound(patch.data(), r.pid, r.mn, r.mx, r.depth, &mv, &P, limit)
            : refk_bound_gregory::bound(patch.data(), r.pid, r.mn, r.mx, r.depth, &mv, &P, limit);
        if (flag & 1) {
            if (n < cap) {
                pid[n] = r.pid;
                range[4 * n] = r.mn.x; range[4 * n + 1] = r.mn.y;
                range[4 * n + 2] = r.mx.x; range[4 * n + 3] = r.mx.y;
            }
            ++n;
        } else if (flag & 2) {
            const float2 c = (r.mn + r.mx) * 0.5f;
            R a{r.pid, (uchar)(r.depth + 1), r.mn, r.mx}, b{r.pid, (uchar)(r.depth + 1), r.mn, r.mx};
            if (flag & 4) { a.mx = float2(c.x, r.mx.y); b.mn = float2(c.x, r.mn.y); }
            else { a.mx = float2(r.mx.x, c.y); b.mn = float2(r.mn.x, c.y); }
            stack.push_back(b);
            stack.push_back(a);
        }
    }
    return n;
}

// The reference's dice and shade kernels over `count` sub-patches of one
// draw in one pass (RendererCL.cpp:203-238): the position, pixel and depth
// grids ((PS+1)^2 per sub-patch), the colour grid (PS^2 per sub-patch, left
// untouched where shade returns early for an empty block) and the block
// bounds (int4 per 8x8 block).
void refk_dice_shade(int W, int H, float fovy, float near_plane, int patch_size, int subpixel_bits, int backface,
                     int displacement, const float* cp_in, int n_patches, int type, const float* mv16,
                     const float* color, int count, const int* pids, const float* ranges, float* pos_out,
                     int* pxl_out, float* dep_out, float* col_out, int* block_out, int threads) {
    g_cfg.patch_size = patch_size;
    g_cfg.pxl_shift = subpixel_bits;
    g_cfg.backface = backface;
    g_cfg.displacement = displacement;
    g_cfg.fb_size = int2(W, H);
    g_cfg.grid_size = int2((W + 7) / 8, (H + 7) / 8);
    g_cfg.vp_min_px = int2(0, 0);
    g_cfg.vp_max_px = int2(W, H);
    g_cfg.vp_size_px = int2(W, H);
    const int per = type == 0 ? 16 : 20;
    std::vector<float4> patch((size_t)n_patches * per);
    for (size_t k = 0; k < patch.size(); ++k)
        patch[k] = float4(cp_in[3 * k], cp_in[3 * k + 1], cp_in[3 * k + 2], 1.0f);
    float proj16[16];
    refpin_projection_matrix(fovy, near_plane, W, H, proj16);
    float16 proj, mv;
    for (int k = 0; k < 16; ++k) {
        proj.s[k] = proj16[k];
        mv.s[k] = mv16[k];
    }
    std::vector<float2> mins((size_t)count), maxs((size_t)count);
    for (int s = 0; s < count; ++s) {
        mins[(size_t)s] = float2(ranges[4 * s], ranges[4 * s + 1]);
        maxs[(size_t)s] = float2(ranges[4 * s + 2], ranges[4 * s + 3]);
    }
    float4* pos = reinterpret_cast<float4*>(pos_out);
    int2* pxl = reinterpret_cast<int2*>(pxl_out);
    float4* col = reinterpret_cast<float4*>(col_out);
    int4* blocks = reinterpret_cast<int4*>(block_out);
    const float4 dc(color[0], color[1], color[2], color[3]);
    const int gw = 8;
    {
        const size_t glb[3] = {(size_t)(patch_size + gw), (size_t)(patch_size + gw), (size_t)count};
        const size_t loc[3] = {(size_t)gw, (size_t)gw, 1};
        std::function<void()> body = [&]() {
            if (type == 0)
                refk_bezier::dice(patch.data(), pids, mins.data(), maxs.data(), pos, pxl, dep_out, mv, proj);
            else
                refk_gregory::dice(patch.data(), pids, mins.data(), maxs.data(), pos, pxl, dep_out, mv, proj);
        };
        launch(body, glb, loc, threads);
    }
    {
        const size_t glb[3] = {(size_t)patch_size, (size_t)patch_size, (size_t)count}, loc[3] = {8, 8, 1};
        std::function<void()> body = [&]() { refk_reyes::shade(pos, pxl, blocks, col, dc); };
        launch(body, glb, loc, threads);
    }
}

// One frame as RendererCL draws it: clear (kernels/framebuffer.cl and the
// depth fill of RendererCL.cpp:115-135), then per draw the reference's CPU
// bound-and-split and, per pass of at most patches_per_pass sub-patches,
// dice / shade / sample (RendererCL.cpp:203-260).  color: tiled float4
// (W*H*4), depth: tiled int (W*H).  Returns the number of sub-patches.
long refk_render(int W, int H, float fovy, float near_plane, float cull_ribbon, float limit, int max_split_depth,
                 int patches_per_pass, int patch_size, int subpixel_bits, int backface, int displacement,
                 const float* clear_color, int n_draws, const float* const* cps, const int* n_patches,
                 const int* types, const float* mvs, const float* colors, float* color_out, int* depth_out,
                 int threads) {
    g_cfg.patch_size = patch_size;
    g_cfg.tile_size = 8;
    g_cfg.pxl_shift = subpixel_bits;
    g_cfg.backface = backface;
    g_cfg.displacement = displacement;
    g_cfg.fb_size = int2(W, H);
    g_cfg.grid_size = int2((W + 7) / 8, (H + 7) / 8);
    g_cfg.vp_min_px = int2(0, 0);
    g_cfg.vp_max_px = int2(W, H);
    g_cfg.vp_size_px = int2(W, H);
    const long npx = (long)W * H;
    float4* fb = reinterpret_cast<float4*>(color_out);
    // clear (src/Reyes/Framebuffer.cpp:63-72)
    {
        float4 c(powf(clear_color[0], 2.2f), powf(clear_color[1], 2.2f), powf(clear_color[2], 2.2f), 1000.0f);
        const size_t glb[3] = {(size_t)npx, 1, 1}, loc[3] = {64, 1, 1};
        std::function<void()> body = [&]() { refk_fb::clear(fb, c); };
        launch(body, glb, loc, threads);
    }
    for (long i = 0; i < npx; ++i) depth_out[i] = 0x7fffffff;
    std::vector<int> tile_locks((size_t)(W / 8) * (H / 8) + 1, 1);
    float proj16[16];
    refpin_projection_matrix(fovy, near_plane, W, H, proj16);
    float16 proj;
    for (int k = 0; k < 16; ++k) proj.s[k] = proj16[k];
    const int G = patch_size + 1, Q = patch_size * patch_size, B = (patch_size / 8) * (patch_size / 8);
    const int gw = 8;   // dice_group_width (reyes.options)
    long total = 0;
    for (int d = 0; d < n_draws; ++d) {
        const int per = types[d] == 0 ? 16 : 20;
        const long cap = 1 << 24;
        std::vector<int> pid((size_t)cap);
        std::vector<float> rng((size_t)cap * 4);
        long n = refpin_bound_n_split(cps[d], n_patches[d], types[d], mvs + 16 * d, fovy, near_plane, W, H,
                                      cull_ribbon, limit, max_split_depth, pid.data(), rng.data(), cap);
        if (n > cap) return -1;
        total += n;
        std::vector<float4> patch((size_t)n_patches[d] * per);
        for (size_t k = 0; k < patch.size(); ++k)
            patch[k] = float4(cps[d][3 * k], cps[d][3 * k + 1], cps[d][3 * k + 2], 1.0f);
        float16 mv;
        for (int k = 0; k < 16; ++k) mv.s[k] = mvs[16 * d + k];
        const float4 dc(colors[4 * d], colors[4 * d + 1], colors[4 * d + 2], colors[4 * d + 3]);
        for (long first = 0; first < n; first += patches_per_pass) {
            const int cnt = (int)std::min<long>(patches_per_pass, n - first);
            std::vector<int> pids(pid.begin() + first, pid.begin() + first + cnt);
            std::vector<float2> mins((size_t)cnt), maxs((size_t)cnt);
            for (int s = 0; s < cnt; ++s) {
                mins[(size_t)s] = float2(rng[4 * (first + s)], rng[4 * (first + s) + 1]);
                maxs[(size_t)s] = float2(rng[4 * (first + s) + 2], rng[4 * (first + s) + 3]);
            }
            std::vector<float4> pos((size_t)cnt * G * G);
            std::vector<int2> pxl((size_t)cnt * G * G);
            std::vector<float> dep((size_t)cnt * G * G);
            std::vector<int4> blocks((size_t)cnt * B);
            std::vector<float4> col((size_t)cnt * Q);
            {
                const size_t glb[3] = {(size_t)(patch_size + gw), (size_t)(patch_size + gw), (size_t)cnt};
                const size_t loc[3] = {(size_t)gw, (size_t)gw, 1};
                std::function<void()> body = [&]() {
                    if (types[d] == 0)
                        refk_bezier::dice(patch.data(), pids.data(), mins.data(), maxs.data(), pos.data(), pxl.data(),
                                          dep.data(), mv, proj);
                    else
                        refk_gregory::dice(patch.data(), pids.data(), mins.data(), maxs.data(), pos.data(),
                                           pxl.data(), dep.data(), mv, proj);
                };
                launch(body, glb, loc, threads);
            }
            {
                const size_t glb[3] = {(size_t)patch_size, (size_t)patch_size, (size_t)cnt}, loc[3] = {8, 8, 1};
                std::function<void()> body = [&]() {
                    refk_reyes::shade(pos.data(), pxl.data(), blocks.data(), col.data(), dc);
                };
                launch(body, glb, loc, threads);
            }
            {
                const size_t glb[3] = {8, 8, (size_t)cnt * B}, loc[3] = {8, 8, 1};
                std::function<void()> body = [&]() {
                    refk_reyes::sample(blocks.data(), pxl.data(), col.data(), dep.data(), tile_locks.data(), fb,
                                       depth_out);
                };
                launch(body, glb, loc, threads);
            }
        }
    }
    return total;
}

}  // extern "C"
