// Device-side math of the REYES core, shared by the bound-and-split,
// dice/raster, resolve and adjoint kernels.
//
// Every floating-point operation whose rounding decides a result is written
// with an explicit rounding intrinsic, and the whole library is compiled with
// -fmad=false so nothing else is fused behind our back:
//   * bound-and-split (src/Reyes/BoundNSplitCLCPU.cpp:249-336,
//     src/base/Projection.cpp:57-106, src/base/Patch.cpp:107-210): no fused
//     operations at all, so the emitted sub-patch set is bit-identical to the
//     reference's CPU bound-and-split;
//   * dice / shade / sample (kernels/dice.cl, kernels/reyes.cl,
//     kernels/utility.h): the rounding choices allowed by the reference's
//     -cl-mad-enable -cl-fast-relaxed-math build are fixed as
//       R1 a*b + c is one fma; dot() fuses its first product,
//          fma(w, w', fma(z, z', fma(x, x', y*y'))); the barycentric dot and
//          vector sums a*A + b*B (Gregory blends, colour) fuse the later one,
//          fma(b, B, a*A); cross(): a*b - c*d = fma(-c, d, a*b)
//       R2 a division x / y is x * RN(1 / y) (the reciprocal correctly rounded,
//          as -cl-fast-relaxed-math permits); sqrt correctly rounded
//       R3 max(x, 0) ignores NaN (fmaxf)
//       R4 float->int truncates and saturates, NaN -> 0 (cvt.rzi.s32.f32)
//       R5 int arithmetic wraps modulo 2^32
//       R6 native_sin = mp_sinf (Cody-Waite reduction modulo pi, odd Taylor polynomial)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mp {

constexpr int kMaxPS = 16;

// Per-draw constants (one draw = one mesh drawn with one modelview into one
// framebuffer layer), resident in device memory.
struct DrawDev {
    const float4* cp;      // control points (x, y, z, 1), 16 or 20 per patch
    float* grad_cp;        // adjoint output, xyz per control point (nullptr = none)
    int n_patches;
    int type;              // 0 Bezier, 1 Gregory
    int view;              // framebuffer layer
    int pad0;
    float mv[16];          // column-major modelview (glm layout)
    float proj[16];        // glm::perspective(fovy, aspect, near, 10000), column-major
    float color[4];        // object colour
    // Projection::bound (src/base/Projection.cpp:23-35)
    float fx, fy, vpx, vpy;
    float near_plane, cull_ribbon;
    int vx, vy;
    // GPU criterion: eps = near * 0.1 of kernels/bound_n_split.h:57, the
    // product taken in double as the OpenCL source's double literal makes it
    float near_eps;
    int pad1[3];
};

// Frame-wide constants.
struct FrameDev {
    int W, H;              // framebuffer size (all layers)
    int PS;                // reyes_patch_size (8 or 16)
    int shift;             // subpixel_bits
    float limit;           // bound_n_split_limit
    int max_depth;         // max_split_depth
    int backface;          // backface_culling
    int displacement;      // displacement on/off
    float fdisp[3];        // 0.04, 0.02, 0.01 times the amplitude multiplier (load_amplitude)
    const float* amp_dev;  // the amplitude multiplier in device memory (nullptr: fdisp as given)
    float clear[4];        // clear colour (powf(c, 2.2), alpha 1000)
    int gx, gy;            // 8-pixel tile grid of the output framebuffer
    int n_draws;
    int kshift;            // depth|id key buffer tile: 1 << kshift pixels (8, 16 or 32)
    int kgx;               // key tiles per row
    int criterion;         // mp_bound_criterion
};

// Depth|id key stored per pixel: (idepth << 32) | mp_id.  The clear key keeps
// the reference's cleared depth 0x7fffffff (src/Reyes/RendererCL.cpp:123-126).
constexpr unsigned long long kClearKey = 0x7fffffffffffffffULL;

// ---------------------------------------------------------------------------
// Bound-and-split arithmetic: plain IEEE, no fused operations.

struct F3 { float x, y, z; };

__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdiv_rn(a, b); }

// Packed pairs (the FFMA2 / FMUL2 / FADD2 instructions of sm_100 and later):
// each component rounds as ffma / fmul / fadd, one instruction issue for two.
// The dice arithmetic packs the x/y and z/w components of one evaluation.
// They are kept out of the bound-and-split arithmetic, which must not fuse:
// there a packed product feeding a packed sum gave a different sub-patch set
// than the scalar _rn operations (a contraction the -fmad=false build does
// not rule out for the packed forms).  In the dice arithmetic a packed
// product only feeds a multiply, the multiplicand of a fused multiply-add, or
// (the viewport transform) an exact scaling by 0.5, where a contraction
// could not change a bit.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fadd2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 dup2(float a) { return make_float2(a, a); }
// src/base/utility.h:86-94
__device__ __forceinline__ float minimum(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float maximum(float a, float b) { return a > b ? a : b; }

// src/base/Patch.cpp:107-113
struct SplineW { float a, b, c, d; };
__device__ __forceinline__ SplineW spline_weights(float t) {
    float s = fsub(1.0f, t);
    SplineW w;
    w.a = fmul(fmul(s, s), s);
    w.b = fmul(fmul(fmul(3.0f, s), s), t);
    w.c = fmul(fmul(fmul(3.0f, s), t), t);
    w.d = fmul(fmul(t, t), t);
    return w;
}
__device__ __forceinline__ float spline1(const SplineW& w, float p0, float p1, float p2, float p3) {
    return fadd(fadd(fadd(fmul(w.a, p0), fmul(w.b, p1)), fmul(w.c, p2)), fmul(w.d, p3));
}
__device__ __forceinline__ F3 spline3(const SplineW& w, const F3& p0, const F3& p1, const F3& p2,
                                      const F3& p3) {
    return F3{spline1(w, p0.x, p1.x, p2.x, p3.x), spline1(w, p0.y, p1.y, p2.y, p3.y),
              spline1(w, p0.z, p1.z, p2.z, p3.z)};
}
__device__ __forceinline__ F3 ld3(const float4* p) {
    float4 v = __ldg(p);
    return F3{v.x, v.y, v.z};
}

// glm 0.9.9 mat4 * vec4(p, 1): (m0*x + m1*y) + (m2*z + m3*1), per component.
__device__ __forceinline__ F3 mv_point(const float* m, const F3& p) {
    F3 r;
    r.x = fadd(fadd(fmul(m[0], p.x), fmul(m[4], p.y)), fadd(fmul(m[8], p.z), fmul(m[12], 1.0f)));
    r.y = fadd(fadd(fmul(m[1], p.x), fmul(m[5], p.y)), fadd(fmul(m[9], p.z), fmul(m[13], 1.0f)));
    r.z = fadd(fadd(fmul(m[2], p.x), fmul(m[6], p.y)), fadd(fmul(m[10], p.z), fmul(m[14], 1.0f)));
    return r;
}

// glm::distance: sqrt((dx*dx + dy*dy) + dz*dz)
__device__ __forceinline__ float distance3(const F3& a, const F3& b) {
    float dx = fsub(b.x, a.x), dy = fsub(b.y, a.y), dz = fsub(b.z, a.z);
    return __fsqrt_rn(fadd(fadd(fmul(dx, dx), fmul(dy, dy)), fmul(dz, dz)));
}

// Gregory patch (src/base/Patch.cpp:186-210), evaluated at (u, v) after the swap.
__device__ __forceinline__ F3 blend3(float a, const F3& A, float b, const F3& B, float den) {
    return F3{fdiv(fadd(fmul(a, A.x), fmul(b, B.x)), den), fdiv(fadd(fmul(a, A.y), fmul(b, B.y)), den),
              fdiv(fadd(fmul(a, A.z), fmul(b, B.z)), den)};
}
// Not inlined: the nine calls of bound_range share one copy of the code,
// which keeps the bound-and-split loop inside the instruction cache.
static __device__ __noinline__ F3 eval_gregory_cpu(const float4* pd, float u_in, float v_in) {
    float u = v_in, v = u_in;  // std::swap(u, v)
    F3 F0 = blend3(u, ld3(pd + 12), v, ld3(pd + 16), fadd(u, v));
    F3 F1 = blend3(fsub(1.0f, u), ld3(pd + 17), v, ld3(pd + 13), fadd(fsub(1.0f, u), v));
    // F2 = ((1-u)*fm[2] + (1-v)*fp[2]) / (2-u-v): the CPU blend swaps the roles
    // of fp and fm relative to the kernel version (kernels/utility.h:171)
    F3 F2 = blend3(fsub(1.0f, u), ld3(pd + 18), fsub(1.0f, v), ld3(pd + 14), fsub(fsub(2.0f, u), v));
    F3 F3v = blend3(u, ld3(pd + 19), fsub(1.0f, v), ld3(pd + 15), fsub(fadd(1.0f, u), v));
    SplineW wu = spline_weights(u);
    F3 P0 = spline3(wu, ld3(pd + 0), ld3(pd + 8), ld3(pd + 7), ld3(pd + 3));
    F3 P1 = spline3(wu, ld3(pd + 4), F0, F3v, ld3(pd + 11));
    F3 P2 = spline3(wu, ld3(pd + 9), F1, F2, ld3(pd + 6));
    F3 P3 = spline3(wu, ld3(pd + 1), ld3(pd + 5), ld3(pd + 10), ld3(pd + 2));
    return spline3(spline_weights(v), P0, P1, P2, P3);
}

// The range bound of src/Reyes/BoundNSplitCLCPU.cpp:249-336: 3x3 samples at
// min + (max - min) * i * 0.5, eye-space bbox, and the largest summed sample
// distance along x (vlen) and along y (hlen).  For Bezier patches the four
// row splines in t = u are shared by the three samples with the same u; each
// sample still performs exactly the reference's operations.
struct RangeBound {
    F3 bmin, bmax;
    float vlen, hlen;
};

__device__ __forceinline__ void bbox_add(RangeBound& b, const F3& p) {
    b.bmin.x = minimum(p.x, b.bmin.x);
    b.bmin.y = minimum(p.y, b.bmin.y);
    b.bmin.z = minimum(p.z, b.bmin.z);
    b.bmax.x = maximum(p.x, b.bmax.x);
    b.bmax.y = maximum(p.y, b.bmax.y);
    b.bmax.z = maximum(p.z, b.bmax.z);
}

// The 9 samples are visited column by column (iv outer, iu inner, the
// column loop not unrolled) so that only one column and the previous one are
// live and the code stays small.  Every value is formed by
// the reference's operations in the reference's order: the column sum v_iv is
// (0 + d01) + d12, the row sums h_iu accumulate across columns in the same
// order, vlen/hlen take maximum() in index order 0, 1, 2, and the bbox
// (minimum/maximum that skip NaN) does not depend on the visiting order.
// Eye-space points of the samples (iu, iv), iu = 0..2, of one column iv of
// the 3x3 grid; only the samples whose bit is set in `need` are evaluated.
__device__ __forceinline__ void bound_column(const DrawDev& d, int pid, float4 r, int iv, F3 cur[3],
                                             unsigned need = 7u) {
    float sv[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) sv[i] = fadd(r.x, fmul(fmul(fsub(r.z, r.x), (float)i), 0.5f));
    const float su_iv = fadd(r.y, fmul(fmul(fsub(r.w, r.y), (float)iv), 0.5f));
    if (d.type == 0) {
        // eval_patch(P, t = u, s = v): rows P[i][0..3] in t, then the column in s
        const float4* P = d.cp + (size_t)pid * 16;
        SplineW wt = spline_weights(su_iv);
        F3 row[4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
            row[i] = spline3(wt, ld3(P + 4 * i + 0), ld3(P + 4 * i + 1), ld3(P + 4 * i + 2), ld3(P + 4 * i + 3));
#pragma unroll
        for (int iu = 0; iu < 3; ++iu)
            if (need & (1u << iu))
                cur[iu] = mv_point(d.mv, spline3(spline_weights(sv[iu]), row[0], row[1], row[2], row[3]));
    } else {
        const float4* P = d.cp + (size_t)pid * 20;
#pragma unroll
        for (int iu = 0; iu < 3; ++iu)
            if (need & (1u << iu)) cur[iu] = mv_point(d.mv, eval_gregory_cpu(P, su_iv, sv[iu]));
    }
}

// column iv's summed distance: v = (0 + d(ps[0][iv], ps[1][iv])) + d(ps[1][iv], ps[2][iv])
__device__ __forceinline__ float column_length(const F3 cur[3]) {
    return fadd(fadd(0.0f, distance3(cur[0], cur[1])), distance3(cur[1], cur[2]));
}

__device__ __forceinline__ RangeBound bound_range(const DrawDev& d, int pid, float4 r) {
    RangeBound b;
    const float inf = __int_as_float(0x7f800000);
    b.bmin = F3{inf, inf, inf};
    b.bmax = F3{-inf, -inf, -inf};
    b.vlen = 0.0f;
    float hsum[3] = {0.0f, 0.0f, 0.0f};
    F3 prev[3];
#pragma unroll 1
    for (int iv = 0; iv < 3; ++iv) {
        F3 cur[3];
        bound_column(d, pid, r, iv, cur);
#pragma unroll
        for (int iu = 0; iu < 3; ++iu) bbox_add(b, cur[iu]);
        b.vlen = maximum(column_length(cur), b.vlen);
        if (iv > 0) {
#pragma unroll
            for (int iu = 0; iu < 3; ++iu) hsum[iu] = fadd(hsum[iu], distance3(prev[iu], cur[iu]));
        }
#pragma unroll
        for (int iu = 0; iu < 3; ++iu) prev[iu] = cur[iu];
    }
    b.hlen = 0.0f;
#pragma unroll
    for (int iu = 0; iu < 3; ++iu) b.hlen = maximum(hsum[iu], b.hlen);
    return b;
}

// src/base/Projection.cpp:57-106.  Returns true when culled, else the screen size.
__device__ __forceinline__ bool projection_cull(const DrawDev& d, const RangeBound& b, float& sx, float& sy) {
    float n = -b.bmax.z;
    float f = -b.bmin.z;
    if (f < d.near_plane) return true;
    n = maximum(d.near_plane, n);
    float mnx = fadd(fmul(fdiv(b.bmin.x, b.bmin.x < 0 ? n : f), d.fx), d.vpx);
    float mny = fadd(fmul(fdiv(b.bmin.y, b.bmin.y < 0 ? n : f), d.fy), d.vpy);
    float mxx = fadd(fmul(fdiv(b.bmax.x, b.bmax.x > 0 ? n : f), d.fx), d.vpx);
    float mxy = fadd(fmul(fdiv(b.bmax.y, b.bmax.y > 0 ? n : f), d.fy), d.vpy);
    if (mnx > fadd((float)(d.vx - 1), d.cull_ribbon) || mxx < -d.cull_ribbon ||
        mny > fadd((float)(d.vy - 1), d.cull_ribbon) || mxy < -d.cull_ribbon)
        return true;
    sx = fsub(mxx, mnx);
    sy = fsub(mxy, mny);
    return false;
}

enum BnsDecision { kCull = 0, kDraw = 1, kSplitY = 2, kSplitX = 3, kDrop = 4 };

// src/Reyes/BoundNSplitCLCPU.cpp:117-148: cull, draw when in front of the eye
// and smaller than the limit, drop past the depth cap, otherwise split the
// direction with the longer sampled length (vlen < hlen halves y).
__device__ __forceinline__ int bns_decide_bound(const DrawDev& d, const FrameDev& fr, const RangeBound& b, int depth) {
    float sx, sy;
    if (projection_cull(d, b, sx, sy)) return kCull;
    if (b.bmin.z < 0 && sx < fr.limit && sy < fr.limit) return kDraw;
    if (depth > fr.max_depth) return kDrop;
    return (b.vlen < b.hlen) ? kSplitY : kSplitX;
}


// Children of a split (BoundNSplitCLCPU.cpp:231-245): low half, high half.
__device__ __forceinline__ void split_children(float4 r, int dec, float4& c0, float4& c1) {
    if (dec == kSplitY) {
        float cy = fmul(fadd(r.y, r.w), 0.5f);
        c0 = make_float4(r.x, r.y, r.z, cy);
        c1 = make_float4(r.x, cy, r.z, r.w);
    } else {
        float cx = fmul(fadd(r.x, r.z), 0.5f);
        c0 = make_float4(r.x, r.y, cx, r.w);
        c1 = make_float4(cx, r.y, r.z, r.w);
    }
}

// ---------------------------------------------------------------------------
// Kernel restatement arithmetic (R1-R6).

__device__ __forceinline__ float ffma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
// R2: x / y in the kernel restatement
__device__ __forceinline__ float frcp(float y) { return __frcp_rn(y); }
__device__ __forceinline__ float kdiv(float x, float y) { return fmul(x, frcp(y)); }


// Cosine for the adjoint's derivatives: Cody-Waite reduction with pi/2 =
// P1 + P2 + P3 (three floats from the exact value of pi) and Taylor
// polynomials (degree 9 / 10) on |r| <= pi/4, with fused multiply-adds.
__device__ __forceinline__ void sincos_reduced(float x, float& sr, float& cr, int& q) {
    float k = rintf(fmul(x, 0x1.45f306p-1f));
    float r = ffma(-k, 0x1.921fb6p+0f, x);
    r = ffma(-k, -0x1.777a5cp-25f, r);
    r = ffma(-k, -0x1.ee59dap-50f, r);
    float kq = fsub(k, fmul(4.0f, floorf(fmul(k, 0.25f))));
    q = (int)kq;
    float r2 = fmul(r, r);
    float ps = ffma(r2, 0x1.71de3ap-19f, -0x1.a01a02p-13f);
    ps = ffma(r2, ps, 0x1.111112p-7f);
    ps = ffma(r2, ps, -0x1.555556p-3f);
    sr = ffma(fmul(r, r2), ps, r);
    float pc = ffma(r2, -0x1.27e4fcp-22f, 0x1.a01a02p-16f);
    pc = ffma(r2, pc, -0x1.6c16c2p-10f);
    pc = ffma(r2, pc, 0x1.555556p-5f);
    pc = ffma(r2, pc, -0x1.0p-1f);
    cr = ffma(r2, pc, 1.0f);
}
// R6 native_sin: reduction by pi = PI1 + PI2 + PI3 (the pi/2 split doubled,
// exactly) to |r| <= pi/2, the odd Taylor polynomial of degree 13, the sign
// of (-1)^k; one polynomial instead of the two of sincos_reduced.
__device__ __forceinline__ float mp_sinf(float x) {
    if (!isfinite(x)) return fsub(x, x);
    const float k = rintf(fmul(x, 0x1.45f306p-2f));
    float r = ffma(-k, 0x1.921fb6p+1f, x);
    r = ffma(-k, -0x1.777a5cp-24f, r);
    r = ffma(-k, -0x1.ee59dap-49f, r);
    const float r2 = fmul(r, r);
    float p = ffma(r2, 0x1.612462p-33f, -0x1.ae6456p-26f);
    p = ffma(r2, p, 0x1.71de3ap-19f);
    p = ffma(r2, p, -0x1.a01a02p-13f);
    p = ffma(r2, p, 0x1.111112p-7f);
    p = ffma(r2, p, -0x1.555556p-3f);
    const float sn = ffma(fmul(r, r2), p, r);
    const float odd = fsub(k, fmul(2.0f, floorf(fmul(k, 0.5f))));
    return odd != 0.0f ? -sn : sn;
}
__device__ __forceinline__ float mp_cosf(float x) {
    if (!isfinite(x)) return fsub(x, x);
    float s, c;
    int q;
    sincos_reduced(x, s, c, q);
    q &= 3;
    return q == 0 ? c : q == 1 ? -s : q == 2 ? -c : s;
}

__device__ __forceinline__ float sel_nan(float x) { return isnan(x) ? 0.0f : x; }

// kernels/utility.h:121-152 -- p += (v_i * c_j) * P[4i + j], i-major; P.w = 1.
// Row weights v_i (in t.x) and column weights c_j (in t.y) of
// kernels/utility.h:127-145: v = s^3, 3 s^2 t, 3 s t^2, t^3 with the
// source's left-to-right products.
__device__ __forceinline__ float4 row_weights(float tx) {
    float sx = fsub(1.0f, tx);
    return make_float4(fmul(fmul(sx, sx), sx), fmul(fmul(fmul(3.0f, sx), sx), tx), fmul(fmul(fmul(3.0f, sx), tx), tx),
                       fmul(fmul(tx, tx), tx));
}
__device__ __forceinline__ float4 col_weights(float ty) {
    float sy = fsub(1.0f, ty);
    return make_float4(fmul(fmul(sy, sy), sy), fmul(fmul(fmul(3.0f, ty), sy), sy), fmul(fmul(fmul(3.0f, ty), ty), sy),
                       fmul(fmul(ty, ty), ty));
}
// p += (v_i * c_j) * Q_{4i+j}, i-major, one fma per component (R1); the
// x/y and z/w chains run as packed pairs.
template <typename Pts>
__device__ __forceinline__ float4 accumulate16(const Pts& Q, float4 vw4, float4 cw4) {
    const float2 vw[4] = {dup2(vw4.x), dup2(vw4.y), dup2(vw4.z), dup2(vw4.w)};
    const float2 cw[4] = {dup2(cw4.x), dup2(cw4.y), dup2(cw4.z), dup2(cw4.w)};
    float2 pxy = make_float2(0.f, 0.f), pzw = make_float2(0.f, 0.f);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float2 w = fmul2(vw[i], cw[j]);
            const float4 c = Q[4 * i + j];
            pxy = ffma2(w, make_float2(c.x, c.y), pxy);
            pzw = ffma2(w, make_float2(c.z, c.w), pzw);
        }
    return make_float4(pxy.x, pxy.y, pzw.x, pzw.y);
}
__device__ __forceinline__ float4 eval_bezier_dice_w(const float4* P, float4 vw, float4 cw) {
    return accumulate16(P, vw, cw);
}
__device__ __forceinline__ float4 eval_bezier_dice(const float4* P, float tx, float ty) {
    return eval_bezier_dice_w(P, row_weights(tx), col_weights(ty));
}

__device__ __forceinline__ float4 blend4(float a, float4 A, float b, float4 B, float den) {
    const float2 r = dup2(frcp(den)), a2 = dup2(a), b2 = dup2(b);
    const float2 xy = fmul2(ffma2(b2, make_float2(B.x, B.y), fmul2(a2, make_float2(A.x, A.y))), r);
    const float2 zw = fmul2(ffma2(b2, make_float2(B.z, B.w), fmul2(a2, make_float2(A.z, A.w))), r);
    return make_float4(sel_nan(xy.x), sel_nan(xy.y), sel_nan(zw.x), sel_nan(zw.y));
}

// kernels/utility.h:155-206 -- Gregory patch with NaN face blends zeroed.
__device__ __forceinline__ float4 eval_gregory_dice_w(const float4* P, float tx, float ty, float4 vw, float4 cw) {
    float u = tx, v = ty;
    float4 F0 = blend4(u, P[12], v, P[16], fadd(u, v));
    float4 F1 = blend4(fsub(1.0f, u), P[17], v, P[13], fadd(fsub(1.0f, u), v));
    float4 F2 = blend4(fsub(1.0f, u), P[14], fsub(1.0f, v), P[18], fsub(fsub(2.0f, u), v));
    float4 F3 = blend4(u, P[19], fsub(1.0f, v), P[15], fsub(fadd(1.0f, u), v));
    const float4 pts[16] = {P[0], P[4], P[9], P[1], P[8], F0, F1, P[5], P[7], F3, F2, P[10], P[3], P[11], P[6], P[2]};
    return accumulate16(pts, vw, cw);
}
__device__ __forceinline__ float4 eval_gregory_dice(const float4* P, float tx, float ty) {
    return eval_gregory_dice_w(P, tx, ty, row_weights(tx), col_weights(ty));
}

// kernels/utility.h:174-180: each row a dot(), fma(w, w', fma(z, z',
// fma(x, x', y*y'))) (R1); rows 0/1 and 2/3 as packed pairs (the
// column-major m holds each pair of rows side by side).
__device__ __forceinline__ float4 mul_m44v4(const float* m, float4 v) {
    const float2 x = dup2(v.x), y = dup2(v.y), z = dup2(v.z), w = dup2(v.w);
    float2 r01 = fmul2(make_float2(m[4], m[5]), y);
    float2 r23 = fmul2(make_float2(m[6], m[7]), y);
    r01 = ffma2(make_float2(m[0], m[1]), x, r01);
    r23 = ffma2(make_float2(m[2], m[3]), x, r23);
    r01 = ffma2(make_float2(m[8], m[9]), z, r01);
    r23 = ffma2(make_float2(m[10], m[11]), z, r23);
    r01 = ffma2(make_float2(m[12], m[13]), w, r01);
    r23 = ffma2(make_float2(m[14], m[15]), w, r23);
    return make_float4(r01.x, r01.y, r23.x, r23.y);
}

// The displacement amplitudes of a frame: kernels/dice.cl:52-54's 0.04,
// 0.02 and 0.01 times the multiplier held in device memory, so that a caller
// can change it between frames from device data.  Kernels that displace call
// this once on their copy of the frame constants.
__device__ __forceinline__ void load_amplitude(FrameDev& fr) {
    if (fr.amp_dev && fr.displacement) {
        const float a = *(volatile const float*)fr.amp_dev;
        fr.fdisp[0] = fmul(0.04f, a);
        fr.fdisp[1] = fmul(0.02f, a);
        fr.fdisp[2] = fmul(0.01f, a);
    }
}

// kernels/dice.cl:51-67 -- eye-space displacement, updated coordinates used
// immediately; fd are the three amplitudes.
__device__ __forceinline__ float4 displace(float4 pos, const float* fd) {
    const float k[3] = {5.0f, 7.0f, 11.0f};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        pos.x = ffma(mp_sinf(fmul(fmul(pos.y, k[i]), 2.0f)), fd[i], pos.x);
        pos.y = ffma(mp_sinf(fmul(fmul(pos.x, k[i]), 2.0f)), fd[i], pos.y);
        pos.z = ffma(fmul(mp_sinf(fmul(fmul(pos.y, k[i]), 2.0f)), mp_sinf(fmul(fmul(pos.x, 3.0f), 2.0f))), fd[i],
                     pos.z);
    }
    return pos;
}

// Eye-space position of dice vertex (nu, nv) of a sub-patch (kernels/dice.cl:44-67).
// nu / PS is exact (PS is a power of two), so it is formed as nu * (1 / PS).
// Parameter of dice vertex index n along one side: mix(rmin, rmax, n / PS).
__device__ __forceinline__ float dice_param(float rmin, float rmax, int n, const FrameDev& fr) {
    const float inv = fr.PS == 16 ? 0.0625f : 0.125f;  // RN(1 / PS), exact for PS in {8, 16}
    return ffma(fsub(rmax, rmin), fmul((float)n, inv), rmin);
}
// Eye position from precomputed parameters and weights of one vertex.
__device__ __forceinline__ float4 dice_eye_w(int type, const float* mv, const FrameDev& fr, const float4* P, float tx,
                                             float ty, float4 vw, float4 cw) {
    float4 o = (type == 0) ? eval_bezier_dice_w(P, vw, cw) : eval_gregory_dice_w(P, tx, ty, vw, cw);
    float4 pos = mul_m44v4(mv, o);
    if (fr.displacement) pos = displace(pos, fr.fdisp);
    return pos;
}
__device__ __forceinline__ float4 dice_eye_m(int type, const float* mv, const FrameDev& fr, const float4* P,
                                             float4 r, int nu, int nv) {
    const float tx = dice_param(r.x, r.z, nu, fr), ty = dice_param(r.y, r.w, nv, fr);
    return dice_eye_w(type, mv, fr, P, tx, ty, row_weights(tx), col_weights(ty));
}
__device__ __forceinline__ float4 dice_eye(const DrawDev& d, const FrameDev& fr, const float4* P, float4 r,
                                           int nu, int nv) {
    return dice_eye_m(d.type, d.mv, fr, P, r, nu, nv);
}

// Projection to fixed-point pixel coordinates and NDC depth (kernels/dice.cl:69-79).
__device__ __forceinline__ void project_vertex_m(const float* proj, const FrameDev& fr, float4 pos, int& px,
                                                 int& py, float& depth) {
    float4 p = mul_m44v4(proj, pos);
    int vsx = fr.W << fr.shift, vsy = fr.H << fr.shift;
    const float rw = frcp(p.w);
    // (p.xy / p.w * VIEWPORT_SIZE) / 2 + VIEWPORT_SIZE / 2, x and y packed
    float2 e = fmul2(make_float2(p.x, p.y), dup2(rw));
    e = fmul2(e, make_float2((float)vsx, (float)vsy));
    e = fmul2(e, dup2(0.5f));
    e = fadd2(e, make_float2((float)(vsx / 2), (float)(vsy / 2)));
    px = __float2int_rz(e.x);
    py = __float2int_rz(e.y);
    depth = fmul(p.z, rw);
}
// project_vertex_m for a glm::perspective matrix, whose only nonzero
// entries are m0, m5, m10, m14 and m11 = -1 (the host builds every draw's
// projection so).  For a finite position with eye z != 0 the general product
// reduces exactly: each zero term adds a zero to a rounded product, which
// changes at most the sign of a zero result, and the viewport transform
// (+ W/2, + H/2) and the depth clamp do not see that sign; p.w = -z.  Any
// other position takes the general product.
__device__ __forceinline__ void project_vertex_persp(const float* proj, const FrameDev& fr, float4 pos, int& px,
                                                     int& py, float& depth) {
    const float mag = fadd(fadd(fabsf(pos.x), fabsf(pos.y)), fadd(fabsf(pos.z), fabsf(pos.w)));
    if (!(mag < __int_as_float(0x7f800000)) || pos.z == 0.0f) {
        project_vertex_m(proj, fr, pos, px, py, depth);
        return;
    }
    const int vsx = fr.W << fr.shift, vsy = fr.H << fr.shift;
    const float2 pxy = fmul2(make_float2(proj[0], proj[5]), make_float2(pos.x, pos.y));
    const float pz = ffma(proj[14], pos.w, fmul(proj[10], pos.z));
    const float rw = frcp(-pos.z);
    float2 e = fmul2(pxy, dup2(rw));
    e = fmul2(e, make_float2((float)vsx, (float)vsy));
    e = fmul2(e, dup2(0.5f));
    e = fadd2(e, make_float2((float)(vsx / 2), (float)(vsy / 2)));
    px = __float2int_rz(e.x);
    py = __float2int_rz(e.y);
    depth = fmul(pz, rw);
}
__device__ __forceinline__ void project_vertex(const DrawDev& d, const FrameDev& fr, float4 pos, int& px, int& py,
                                               float& depth) {
    project_vertex_m(d.proj, fr, pos, px, py, depth);
}

struct V3 { float x, y, z; };
// dot(): fma(z, z', fma(x, x', y*y')) (R1)
__device__ __forceinline__ float dot3(V3 a, V3 b) { return ffma(a.z, b.z, ffma(a.x, b.x, fmul(a.y, b.y))); }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
    return V3{ffma(-a.z, b.y, fmul(a.y, b.z)), ffma(-a.x, b.z, fmul(a.z, b.x)), ffma(-a.y, b.x, fmul(a.x, b.y))};
}
__device__ __forceinline__ V3 normalize3(V3 v) {
    const float r = frcp(__fsqrt_rn(dot3(v, v)));
    return V3{fmul(v.x, r), fmul(v.y, r), fmul(v.z, r)};
}

// kernels/reyes.cl:172-191 -- flat shading of a quad from its 4 eye positions
// (vertex order 0:(u,v) 1:(u+1,v) 2:(u,v+1) 3:(u+1,v+1)).  shade_m is the
// diffuse factor max(dot(n, l), 0); shade_color the colour
// ac*dc + m*dc + pow(..)*sc with sc = 0, whose last term is +0.
__device__ __forceinline__ V3 light_dir() { return normalize3(V3{4.0f, 3.0f, 8.0f}); }
__device__ __forceinline__ float shade_m_l(V3 l, float x0, float y0, float z0, float x1, float y1, float z1,
                                           float x2, float y2, float z2, float x3, float y3, float z3) {
    V3 du{fmul(fsub(fadd(fsub(x1, x0), x3), x2), 0.5f), fmul(fsub(fadd(fsub(y1, y0), y3), y2), 0.5f),
          fmul(fsub(fadd(fsub(z1, z0), z3), z2), 0.5f)};
    V3 dv{fmul(fsub(fadd(fsub(x2, x0), x3), x1), 0.5f), fmul(fsub(fadd(fsub(y2, y0), y3), y1), 0.5f),
          fmul(fsub(fadd(fsub(z2, z0), z3), z1), 0.5f)};
    V3 n = normalize3(cross3(dv, du));
    return fmaxf(dot3(n, l), 0.0f);
}
__device__ __forceinline__ float shade_m(float x0, float y0, float z0, float x1, float y1, float z1, float x2,
                                         float y2, float z2, float x3, float y3, float z3) {
    V3 du{fmul(fsub(fadd(fsub(x1, x0), x3), x2), 0.5f), fmul(fsub(fadd(fsub(y1, y0), y3), y2), 0.5f),
          fmul(fsub(fadd(fsub(z1, z0), z3), z2), 0.5f)};
    V3 dv{fmul(fsub(fadd(fsub(x2, x0), x3), x1), 0.5f), fmul(fsub(fadd(fsub(y2, y0), y3), y1), 0.5f),
          fmul(fsub(fadd(fsub(z2, z0), z3), z1), 0.5f)};
    V3 n = normalize3(cross3(dv, du));
    V3 l = normalize3(V3{4.0f, 3.0f, 8.0f});
    return fmaxf(dot3(n, l), 0.0f);
}
__device__ __forceinline__ float4 shade_color(float m, const float* dc) {
    return make_float4(fadd(ffma(m, dc[0], fmul(0.015f, dc[0])), 0.0f), fadd(ffma(m, dc[1], fmul(0.015f, dc[1])), 0.0f),
                       fadd(ffma(m, dc[2], fmul(0.015f, dc[2])), 0.0f), fadd(ffma(m, dc[3], fmul(1.0f, dc[3])), 0.0f));
}
__device__ __forceinline__ float4 shade_quad(const float4* pos, const float* dc) {
    return shade_color(shade_m(pos[0].x, pos[0].y, pos[0].z, pos[1].x, pos[1].y, pos[1].z, pos[2].x, pos[2].y,
                               pos[2].z, pos[3].x, pos[3].y, pos[3].z),
                       dc);
}

// kernels/reyes.cl:240-265 edge setup of one triangle (wrapping int32, R5).
struct Tri {
    int Dx[3], Dy[3], O[3], C[3];
    int Px[3], Py[3];
    float dv[3];
    float rdn;   // RN(1 / dn), dn = E_{e+1}(P_e), the same integer for e = 0, 1, 2
};
__device__ __forceinline__ int wmul(int a, int b) { return (int)((unsigned)a * (unsigned)b); }
__device__ __forceinline__ int wadd(int a, int b) { return (int)((unsigned)a + (unsigned)b); }
__device__ __forceinline__ int wsub(int a, int b) { return (int)((unsigned)a - (unsigned)b); }

__device__ __forceinline__ void tri_setup(Tri& t, int x0, int y0, float d0, int x1, int y1, float d1, int x2, int y2,
                                          float d2) {
    t.Px[0] = x0; t.Px[1] = x1; t.Px[2] = x2;
    t.Py[0] = y0; t.Py[1] = y1; t.Py[2] = y2;
    t.dv[0] = d0; t.dv[1] = d1; t.dv[2] = d2;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        int en = (e + 1) % 3;
        t.Dx[e] = wsub(t.Py[en], t.Py[e]);
        t.Dy[e] = wsub(t.Px[e], t.Px[en]);
    }
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        t.O[e] = wadd(wmul(t.Dx[e], t.Px[e]), wmul(t.Dy[e], t.Py[e]));
        t.C[e] = (t.Dx[e] > 0 || (t.Dx[e] == 0 && t.Dy[e] > 0)) ? -1 : 0;
    }
    // The barycentric denominator of kernels/reyes.cl:256-258 is edge e+1's
    // function at vertex e.  With D = P_{e+1} - P_e and F = P_{e+2} - P_e it
    // is D.y * F.x - D.x * F.y, minus twice the signed area, the same for all
    // three e; wrapped int32 arithmetic is a ring, so the identity holds
    // exactly and one reciprocal serves the three weights of every sample.
    const int dn = wsub(wadd(wmul(t.Dx[1], t.Px[0]), wmul(t.Dy[1], t.Py[0])), t.O[1]);
    t.rdn = frcp((float)dn);
}

// inside_triangle(): updates depth when the sample is inside and nearer.
__device__ __forceinline__ bool tri_test(const Tri& t, int tx, int ty, float& depth) {
    int V[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) V[e] = wsub(wadd(wmul(t.Dx[e], tx), wmul(t.Dy[e], ty)), t.O[e]);
    bool ok = V[0] > t.C[0] && V[1] > t.C[1] && V[2] > t.C[2];
    if (ok) {
        float w[3];
#pragma unroll
        for (int e = 0; e < 3; ++e) w[e] = fmul((float)V[(e + 1) % 3], t.rdn);
        float d = ffma(t.dv[2], w[2], ffma(t.dv[1], w[1], fmul(t.dv[0], w[0])));
        if (d < depth) depth = d;
    }
    return ok;
}

// idepth = (int)(clamp(depth / 200, 0, 1) * 0x7fffffff) (kernels/reyes.cl:364)
__device__ __forceinline__ unsigned idepth_of(float depth) {
    float c = fminf(fmaxf(fmul(depth, 0.005f), 0.0f), 1.0f);   // 0.005f == RN(1 / 200)
    return (unsigned)__float2int_rz(fmul(c, 2147483648.0f));
}

// Tiled framebuffer index (kernels/reyes.cl:37-45, 8-pixel tiles).
__device__ __forceinline__ long long fb_index(const FrameDev& fr, int x, int y) {
    int tx = x >> 3, ty = y >> 3;
    return ((long long)(tx + fr.gx * ty) << 6) + (x & 7) + ((y & 7) << 3);
}
// Pixel of output index i (inverse of fb_index).
__device__ __forceinline__ void fb_pixel(const FrameDev& fr, long long i, int& x, int& y) {
    const int t = (int)(i >> 6);
    x = ((t % fr.gx) << 3) + (int)(i & 7);
    y = ((t / fr.gx) << 3) + (int)((i >> 3) & 7);
}
// Index of pixel (x, y) in the depth|id key buffer, tiled by 1 << kshift
// pixels so that the atomics of one micropolygon neighbourhood share lines.
__device__ __forceinline__ long long key_index(const FrameDev& fr, int x, int y) {
    const int k = fr.kshift, m = (1 << k) - 1;
    return ((long long)((x >> k) + fr.kgx * (y >> k)) << (2 * k)) + (x & m) + ((y & m) << k);
}

// The reference's GPU bound criterion (kernels/bound_n_split.h:8-100), in the
// kernel arithmetic (R1-R6).  The nine screen positions pp[v][u] are consumed
// as they are produced: the sum along u of row v and the sum along v of
// column u accumulate in the reference's order, so only the previous column
// is kept.
__device__ __forceinline__ int bns_decide_gpu(const DrawDev& d, const FrameDev& fr, int pid, float4 r, int depth) {
    if (depth >= fr.max_depth - 1) return kCull;
    const float inf = __int_as_float(0x7f800000);
    float mnx = inf, mny = inf, mnz = inf, mxx = -inf, mxy = -inf, mxz = -inf;
    float2 prev[3];                                  // pp[v][u - 1]
    float hsum[3] = {0.0f, 0.0f, 0.0f};              // along u, per row v
    float vlen = 0.0f;
    const float4* P = d.cp + (size_t)pid * (d.type == 0 ? 16 : 20);
#pragma unroll 1
    for (int u = 0; u < 3; ++u) {
        float vsum = 0.0f;                           // along v, column u
        float2 above = make_float2(0.0f, 0.0f);      // pp[v - 1][u]
#pragma unroll
        for (int v = 0; v < 3; ++v) {
            // uv = mix(rmin, rmax, (u, v) * (1 / (RES - 1)))
            const float tx = ffma(fsub(r.z, r.x), fmul((float)u, 0.5f), r.x);
            const float ty = ffma(fsub(r.w, r.y), fmul((float)v, 0.5f), r.y);
            const float4 o = d.type == 0 ? eval_bezier_dice(P, tx, ty) : eval_gregory_dice(P, tx, ty);
            const float4 p = mul_m44v4(d.mv, o);
            mnx = fminf(mnx, p.x); mny = fminf(mny, p.y); mnz = fminf(mnz, p.z);
            mxx = fmaxf(mxx, p.x); mxy = fmaxf(mxy, p.y); mxz = fmaxf(mxz, p.z);
            const float4 q = mul_m44v4(d.proj, p);
            const float rw = frcp(q.w);
            const float x = fmul(q.x, rw), y = fmul(q.y, rw);
            // mul_cm2v2(screen_matrix = diag(vp), (x, y)): m0 * x + m1 * y per component
            const float2 s = make_float2(ffma(0.0f, y, fmul(d.vpx, x)), ffma(d.vpy, y, fmul(0.0f, x)));
            // distance(a, b) = sqrt(dot(a - b, a - b)), R1: fma(dx, dx, dy*dy)
            if (v > 0) {
                const float dx = fsub(above.x, s.x), dy = fsub(above.y, s.y);
                vsum = fadd(vsum, __fsqrt_rn(ffma(dx, dx, fmul(dy, dy))));
            }
            if (u > 0) {
                const float dx = fsub(prev[v].x, s.x), dy = fsub(prev[v].y, s.y);
                hsum[v] = fadd(hsum[v], __fsqrt_rn(ffma(dx, dx, fmul(dy, dy))));
            }
            above = s;
            prev[v] = s;
        }
        vlen = fmaxf(vsum, vlen);
    }
    // outside_frustum (kernels/bound_n_split.h:8-30)
    float n = -mxz;
    const float f = -mnz;
    if (f < d.near_plane || n > 1000.0f) return kCull;
    n = fmaxf(d.near_plane, n);
    // `x / n * f.x + screen_size.x * 0.5`: the 0.5 is a double literal, so the
    // product is rounded to float before a double addition of W/2, which is
    // exact, then rounded to float: one float multiply and one float add.
    const float sminx = fadd(fmul(kdiv(mnx, mnx < 0 ? n : f), d.fx), d.vpx);
    const float sminy = fadd(fmul(kdiv(mny, mny < 0 ? n : f), d.fy), d.vpy);
    const float smaxx = fadd(fmul(kdiv(mxx, mxx > 0 ? n : f), d.fx), d.vpx);
    const float smaxy = fadd(fmul(kdiv(mxy, mxy > 0 ? n : f), d.fy), d.vpy);
    if (sminx > fadd((float)(d.vx - 1), d.cull_ribbon) || smaxx < -d.cull_ribbon ||
        sminy > fadd((float)(d.vy - 1), d.cull_ribbon) || smaxy < -d.cull_ribbon)
        return kCull;
    // straddles the eye plane: split the shorter parametric side (VSPLIT halves x)
    if (mnz < d.near_eps && mxz > d.near_plane) return fsub(r.z, r.x) < fsub(r.w, r.y) ? kSplitX : kSplitY;
    float hlen = 0.0f;
#pragma unroll
    for (int v = 0; v < 3; ++v) hlen = fmaxf(hsum[v], hlen);
    if (hlen <= fr.limit && vlen <= fr.limit) return kDraw;
    return hlen > vlen ? kSplitX : kSplitY;
}

// ---------------------------------------------------------------------------
// Samples inherited from the parent range.  A child of a split shares two of
// its three sample lines with its parent: splitting x at cx, the low child's
// sample columns iu = 0, 2 lie at the parent's iu = 0, 1 and the high
// child's at the parent's iu = 1, 2 (likewise rows iv for a split of y).
// With dyadic ranges whose sides are multiples of 2^-24 (split depth <= 24)
// every sample parameter is formed exactly, so the shared samples are the
// same floats as the parent's and their evaluation would give the same
// points bit for bit; the child takes them from its queue record and
// evaluates only the three new ones.
constexpr int kInheritNone = 0, kInheritX = 1, kInheritY = 2;
constexpr int kInheritMaxDepth = 24;
constexpr int kPtsPerSlot = 5;   // float4 per queue record of inherited samples

// Points of a lane's current range in shared memory: point (iu, iv),
// component c at sp[((3 * iv + iu) * 3 + c) * st].
__device__ __forceinline__ int spi(int iu, int iv, int c, int st) { return ((3 * iv + iu) * 3 + c) * st; }

// bound_range with the samples that `flag` marks as inherited already in
// sp; evaluates the others, leaves all nine points in sp and returns the
// same bound as bound_range.
__device__ __forceinline__ RangeBound bound_range_inherit(const DrawDev& d, int pid, float4 r, int flag, float* sp,
                                                          int st) {
    RangeBound b;
    const float inf = __int_as_float(0x7f800000);
    b.bmin = F3{inf, inf, inf};
    b.bmax = F3{-inf, -inf, -inf};
    b.vlen = 0.0f;
    float hsum[3] = {0.0f, 0.0f, 0.0f};
    F3 prev[3];
#pragma unroll 1
    for (int iv = 0; iv < 3; ++iv) {
        const unsigned need = flag == kInheritX ? 2u : (flag == kInheritY && iv != 1) ? 0u : 7u;
        F3 cur[3];
#pragma unroll
        for (int iu = 0; iu < 3; ++iu)
            if (!(need & (1u << iu)))
                cur[iu] = F3{sp[spi(iu, iv, 0, st)], sp[spi(iu, iv, 1, st)], sp[spi(iu, iv, 2, st)]};
        if (need) bound_column(d, pid, r, iv, cur, need);
#pragma unroll
        for (int iu = 0; iu < 3; ++iu)
            if (need & (1u << iu)) {
                sp[spi(iu, iv, 0, st)] = cur[iu].x;
                sp[spi(iu, iv, 1, st)] = cur[iu].y;
                sp[spi(iu, iv, 2, st)] = cur[iu].z;
            }
#pragma unroll
        for (int iu = 0; iu < 3; ++iu) bbox_add(b, cur[iu]);
        b.vlen = maximum(column_length(cur), b.vlen);
        if (iv > 0) {
#pragma unroll
            for (int iu = 0; iu < 3; ++iu) hsum[iu] = fadd(hsum[iu], distance3(prev[iu], cur[iu]));
        }
#pragma unroll
        for (int iu = 0; iu < 3; ++iu) prev[iu] = cur[iu];
    }
    b.hlen = 0.0f;
#pragma unroll
    for (int iu = 0; iu < 3; ++iu) b.hlen = maximum(hsum[iu], b.hlen);
    return b;
}

// Queue record of inherited samples (kPtsPerSlot float4): six points, three
// floats each, in the order the flag implies -- kInheritX: (0, iv), (2, iv)
// for iv = 0..2; kInheritY: (iu, 0), (iu, 2) for iu = 0..2 -- and the flag
// in the last float.
__device__ __forceinline__ void inherited_slot(int flag, int k, int& iu, int& iv) {
    if (flag == kInheritX) {
        iu = k < 3 ? 0 : 2;
        iv = k % 3;
    } else {
        iu = k % 3;
        iv = k < 3 ? 0 : 2;
    }
}

// Reads a record into sp; returns its flag.
__device__ __forceinline__ int load_inherited(const float4* rec, float* sp, int st) {
    const int flag = __float_as_int(__ldcg(rec + kPtsPerSlot - 1).w);
    if (flag != kInheritX && flag != kInheritY) return kInheritNone;
    // float j of the record is component j % 3 of point j / 3
#pragma unroll
    for (int k = 0; k < kPtsPerSlot; ++k) {
        const float4 v = __ldcg(rec + k);
        const float f[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int j = 4 * k + e;
            if (j < 18) {
                int iu, iv;
                inherited_slot(flag, j / 3, iu, iv);
                sp[spi(iu, iv, j % 3, st)] = f[e];
            }
        }
    }
    return flag;
}

// Writes the record of child `half` (0 low, 1 high) of a range split by
// `dec`, from the parent's nine points in sp; kInheritNone past the depth
// where sample parameters stay exact.
__device__ __forceinline__ void store_inherited(float4* rec, int dec, int half, int child_depth, const float* sp,
                                                int st) {
    int flag = kInheritNone;
    if (child_depth <= kInheritMaxDepth && (dec == kSplitX || dec == kSplitY))
        flag = dec == kSplitX ? kInheritX : kInheritY;
    if (flag == kInheritNone) {
        rec[kPtsPerSlot - 1] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(kInheritNone));
        return;
    }
#pragma unroll
    for (int k = 0; k < kPtsPerSlot; ++k) {
        float f[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int j = 4 * k + e;
            if (j < 18) {
                int iu, iv;
                inherited_slot(flag, j / 3, iu, iv);
                // the child's line 0 / 2 is the parent's line half / half + 1
                if (flag == kInheritX) iu = half + (iu == 2 ? 1 : 0);
                else iv = half + (iv == 2 ? 1 : 0);
                f[e] = sp[spi(iu, iv, j % 3, st)];
            }
        }
        if (k == kPtsPerSlot - 1) f[3] = __int_as_float(flag);
        rec[k] = make_float4(f[0], f[1], f[2], f[3]);
    }
}

// The decision of one range.  CRIT: 0 the CPU criterion, 1 the GPU
// criterion, -1 chosen at run time from fr.criterion (one kernel for both).
template <int CRIT>
__device__ __forceinline__ int bns_decide(const DrawDev& d, const FrameDev& fr, int pid, float4 r, int depth) {
    if (CRIT == 1 || (CRIT < 0 && fr.criterion == 1)) return bns_decide_gpu(d, fr, pid, r, depth);
    return bns_decide_bound(d, fr, bound_range(d, pid, r), depth);
}
// The CPU criterion with inherited samples (sp as in bound_range_inherit).
__device__ __forceinline__ int bns_decide_inherit(const DrawDev& d, const FrameDev& fr, int pid, float4 r, int depth,
                                                  int flag, float* sp, int st) {
    return bns_decide_bound(d, fr, bound_range_inherit(d, pid, r, flag, sp, st), depth);
}

}  // namespace mp
