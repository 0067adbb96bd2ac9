/*
 * CPU oracle for the REYES hot path: TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
 * may load this library, and only as the checker or as the timed CPU
 * baseline.  The product path (micropolis_gb300, libmpcore.so) never calls
 * into it.
 *
 * It restates, in plain C++ compiled with -O2 -ffp-contract=off:
 *   - the reference's CPU bound-and-split (src/Reyes/BoundNSplitCLCPU.cpp,
 *     src/base/Projection.cpp, src/base/Patch.cpp, src/base/utility.h);
 *   - the reference's dice / shade / sample / clear kernels (kernels/dice.cl,
 *     kernels/reyes.cl, kernels/utility.h, kernels/framebuffer.cl) with one
 *     fixed choice for every rounding the OpenCL build flags leave open;
 *   - an FP64 Bernstein dicer and an FP64 image-loss gradient (the reference
 *     has no gradient code; this one differentiates the restated dicer).
 *
 * Pinning: the bound-and-split arithmetic is checked bit-for-bit against the
 * reference's own src/base/Patch.cpp and src/base/Projection.cpp compiled
 * from the reference tree (oracle/build_ref.sh) over a glm stand-in that
 * fixes glm 0.9.9's scalar operation order.  The kernel restatement has no
 * reference-side golden vectors (no OpenCL runtime exists on either machine):
 * its parity is unpinned beyond the restatement itself.
 */
#pragma once
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One draw call: a mesh of patches, its modelview and object colour. */
typedef struct {
    const float* cp;     /* xyz control points, 16 (Bezier) or 20 (Gregory) per patch */
    int32_t n_patches;
    int32_t type;        /* 0 = Bezier, 1 = Gregory */
    float mv[16];        /* column-major modelview, as glm stores mat4 */
    float color[4];      /* object colour (diffuse) */
} or_draw;

/* Frame-wide options, named as in the reference's reyes.options. */
typedef struct {
    int32_t width, height;          /* window_size */
    float fovy_deg, near_plane;     /* Projection(fovy, near, viewport) */
    float bound_n_split_limit;
    float cull_ribbon;
    int32_t max_split_depth;
    int32_t reyes_patches_per_pass;
    int32_t reyes_patch_size;
    int32_t subpixel_bits;
    int32_t backface_culling;
    int32_t displacement;
    float displacement_amplitude;   /* multiplies the 0.04/0.02/0.01 amplitudes */
    float clear_color[4];
    int32_t bound_criterion;        /* 0: CPU criterion (BoundNSplitCLCPU.cpp), 1: GPU criterion
                                       (kernels/bound_n_split.h), restated with R1-R6 */
} or_params;

/* CPU bound-and-split of one draw.  Writes the emitted sub-patches in the
 * reference's emission order (pid, then range as min.x, min.y, max.x, max.y)
 * and returns how many there are (may exceed cap: only cap are written).
 * n_bounds receives the number of bound evaluations (visited ranges). */
int64_t or_bound_n_split(const or_params* p, const or_draw* d,
                         int32_t* pid, float* range, int64_t cap, int64_t* n_bounds);

/* Every draw's sub-patches in the canonical order: ascending key
 * (root << 32 | split path), root = the draw's first root + patch id (draws
 * in order), the split path's bit 31 - d set when the sub-patch is the high
 * half of its depth-d ancestor's split.  Writes up to cap records (any output
 * may be NULL) and returns how many there are. */
int64_t or_canonical_subpatches(const or_params* p, const or_draw* draws, int32_t n_draws,
                                int32_t* draw, int32_t* pid, float* range, uint64_t* key, int64_t cap);

/* Full frame: clear, bound-and-split every draw, then dice, shade and
 * sample the sub-patches in the canonical order, numbering micropolygons
 * s * PS^2 + nu + nv * PS for canonical sub-patch s; at equal depth the
 * first writer (the smallest number) is kept.  color: tiled float4
 * framebuffer (W*H*4), depth: tiled int32 depth buffer (W*H).  stats (may be
 * NULL) receives [sub-patches, micropolygons, fragments, bounds]. */
int or_render(const or_params* p, const or_draw* draws, int32_t n_draws,
              float* color, int32_t* depth, int64_t* stats);
/* Same, and win (may be NULL) receives the winning number of every tiled
 * pixel, or -1. */
int or_render_win(const or_params* p, const or_draw* draws, int32_t n_draws,
                  float* color, int32_t* depth, int64_t* win, int64_t* stats);

/* Same, but from an explicit sub-patch list (draw index, pid, range), so that
 * the kernel restatement can be checked on a given set.  win (may be NULL)
 * receives, per tiled pixel, the winning sub-patch list index * PS^2 + quad
 * (nu + nv*PS), or -1. */
int or_render_subpatches(const or_params* p, const or_draw* draws, int32_t n_draws,
                         int64_t n_sub, const int32_t* sub_draw, const int32_t* sub_pid,
                         const float* sub_range, float* color, int32_t* depth,
                         int64_t* win, int64_t* stats);
/* Same, with the list's sub-patch s numbered first_index + s (a slice of a
 * longer list: slices merged by the smallest (depth, number) per pixel give
 * the frame of the whole list). */
int or_render_subpatches_at(const or_params* p, const or_draw* draws, int32_t n_draws, int64_t n_sub,
                            int64_t first_index, const int32_t* sub_draw, const int32_t* sub_pid,
                            const float* sub_range, float* color, int32_t* depth, int64_t* win,
                            int64_t* stats);

/* Restated dice of one sub-patch: (PS+1)^2 vertices, index nu + nv*(PS+1).
 * pos: float4 eye-space (after displacement), pxl: int2, depth: float. */
void or_dice(const or_params* p, const or_draw* d, int32_t pid, const float range[4],
             float* pos, int32_t* pxl, float* depth);

/* FP64 Bernstein dice of the same vertices (eye space, after displacement). */
void or_shade_quads(const or_params* p, const or_draw* d, int32_t pid, const float range[4], float* color);
void or_dice_fp64(const or_params* p, const or_draw* d, int32_t pid, const float range[4],
                  double* pos3);

/* FP64 loss sum_px sum_ch (c - t)^2 with visibility fixed by `win`
 * (per tiled pixel: sub-patch index * PS^2 + quad, or -1 = background).
 * cp overrides d->cp for every draw's patches (same layout), amp is the
 * displacement amplitude multiplier.  grad_cp (may be NULL) receives the
 * analytic FP64 gradient per control-point coordinate of draw 0, grad_amp
 * (may be NULL) the gradient w.r.t. amp. */
double or_loss_fp64(const or_params* p, const or_draw* d,
                    int64_t n_sub, const int32_t* sub_pid, const float* sub_range,
                    const int64_t* win, const float* target, const double* cp, double amp,
                    double* grad_cp, double* grad_amp);

/* Sine / cosine used by the displacement: Cody-Waite reduction by pi/2 and
 * Taylor polynomials, evaluated with fused multiply-adds. */
float or_sinf(float x);
float or_cosf(float x);

/* Reference self-test input: the inclusive prefix sum checked by the
 * reference's test_CL_prefix_sum (srand(43), values rand()%8+1). */
void or_inclusive_scan(const int32_t* in, int32_t* out, int64_t n);

#ifdef __cplusplus
}
#endif
