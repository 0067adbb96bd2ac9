// CPU oracle: TEST INFRASTRUCTURE ONLY (see oracle.h for who may call it).
//
// Build: g++ -O2 -ffp-contract=off -fno-fast-math -fPIC -shared (oracle/build.sh).
// -ffp-contract=off matters: the reference's CPU bound-and-split was built
// for x86 with -O2 -msse4 (SConstruct:41), which never fuses a multiply and
// an add, while GCC on aarch64 fuses by default.
//
// Arithmetic conventions of the kernel restatement.  The reference kernels
// are built with -cl-fast-relaxed-math -cl-mad-enable (src/CL/Program.cpp:118),
// which leaves rounding open.  This restatement fixes one admissible choice
// and the CUDA kernels follow the same one.  Where a sum of products leaves a
// choice, R1 takes the one gcc 13 makes when it compiles the kernel source
// itself with contraction on (oracle/ref_kernels.cpp, the pin in
// tests/test_refkernels_cpu.py, which reproduces this oracle's frames):
//   R1  an expression a*b + c (or c + a*b) is one fused multiply-add;
//       dot() (mul_m44v4's rows, shading, distance) fuses the first product:
//       dot(a, b) = fma(a.w, b.w, fma(a.z, b.z, fma(a.x, b.x, a.y*b.y)));
//       the barycentric dot of inside_triangle and the vector sums
//       a*A + b*B (Gregory blends, mul_cm2v2, mul_pm4v4 / mul_cm4v4, the
//       colour ac*dc + m*dc) fuse the later product: fma(b, B, a*A);
//       cross() components a*b - c*d are fma(-c, d, a*b);
//   R2  a division x / y is x * RN(1 / y), the reciprocal correctly rounded
//       (-cl-fast-relaxed-math permits it); square root is correctly rounded;
//   R3  max(x, 0) on floats ignores a NaN operand (fmaxf);
//   R4  float -> int conversion truncates, saturates at the int range and
//       maps NaN to 0 (the CUDA cvt.rzi.s32.f32 rule);
//   R5  int arithmetic wraps modulo 2^32;
//   R6  native_sin is or_sinf below (Cody-Waite reduction modulo pi + an odd
//       Taylor polynomial).
#include "oracle.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <limits>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Small vector types (the reference uses glm; these carry the same values).
struct V2 { float x, y; };
struct V3 { float x, y, z; };
struct V4 { float x, y, z, w; };

// src/base/utility.h:86-94 -- minimum/maximum keep the second operand when
// the first is NaN.
static inline float minimum(float a, float b) { return a < b ? a : b; }
static inline float maximum(float a, float b) { return a > b ? a : b; }

// src/base/utility.h:96-137 -- BBox starts at +/-inf, add_point uses minimum/maximum.
struct BBox {
    V3 min, max;
    void clear() {
        const float inf = std::numeric_limits<float>::infinity();
        min = {inf, inf, inf};
        max = {-inf, -inf, -inf};
    }
    void add_point(const V3& p) {
        min.x = minimum(p.x, min.x);
        min.y = minimum(p.y, min.y);
        min.z = minimum(p.z, min.z);
        max.x = maximum(p.x, max.x);
        max.y = maximum(p.y, max.y);
        max.z = maximum(p.z, max.z);
    }
};

// ---------------------------------------------------------------------------
// Bound-and-split arithmetic (no fused operations anywhere in this section).

// src/base/Patch.cpp:107-113 -- s^3 p0 + 3 s^2 t p1 + 3 s t^2 p2 + t^3 p3,
// scalar factors evaluated left to right, the sum left to right.
static inline V3 eval_spline(const V3& p0, const V3& p1, const V3& p2, const V3& p3, float t) {
    float s = 1 - t;
    float a = s * s * s;
    float b = 3 * s * s * t;
    float c = 3 * s * t * t;
    float d = t * t * t;
    V3 r;
    r.x = a * p0.x + b * p1.x + c * p2.x + d * p3.x;
    r.y = a * p0.y + b * p1.y + c * p2.y + d * p3.y;
    r.z = a * p0.z + b * p1.z + c * p2.z + d * p3.z;
    return r;
}

static inline V3 v3(const float* p) { return V3{p[0], p[1], p[2]}; }

// src/base/Patch.cpp:115-129 -- rows P[i][0..3] in t, then the column in s.
// P[i][j] is control point 4*i + j.
static V3 eval_patch(const float* cp, float t, float s) {
    V3 p[4];
    for (int i = 0; i < 4; ++i)
        p[i] = eval_spline(v3(cp + 3 * (4 * i + 0)), v3(cp + 3 * (4 * i + 1)),
                           v3(cp + 3 * (4 * i + 2)), v3(cp + 3 * (4 * i + 3)), t);
    return eval_spline(p[0], p[1], p[2], p[3], s);
}

static inline V3 add3(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 mul3(float s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
static inline V3 div3(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }

// src/base/Patch.cpp:186-210 -- Gregory patch; u and v are swapped first, the
// face points are blended with unguarded divisions (NaN at the corners).
static V3 eval_gregory_patch(const float* pd, float u, float v) {
    std::swap(u, v);
    const float* p = pd + 0 * 3;
    const float* ep = pd + 4 * 3;
    const float* em = pd + 8 * 3;
    const float* fp = pd + 12 * 3;
    const float* fm = pd + 16 * 3;
    V3 F0 = div3(add3(mul3(u, v3(fp + 0)), mul3(v, v3(fm + 0))), u + v);
    V3 F1 = div3(add3(mul3(1 - u, v3(fm + 3)), mul3(v, v3(fp + 3))), 1 - u + v);
    V3 F2 = div3(add3(mul3(1 - u, v3(fm + 6)), mul3(1 - v, v3(fp + 6))), 2 - u - v);
    V3 F3 = div3(add3(mul3(u, v3(fm + 9)), mul3(1 - v, v3(fp + 9))), 1 + u - v);
    V3 P[4];
    P[0] = eval_spline(v3(p + 0), v3(em + 0), v3(ep + 9), v3(p + 9), u);
    P[1] = eval_spline(v3(ep + 0), F0, F3, v3(em + 9), u);
    P[2] = eval_spline(v3(em + 3), F1, F2, v3(ep + 6), u);
    P[3] = eval_spline(v3(p + 3), v3(ep + 3), v3(em + 6), v3(p + 6), u);
    return eval_spline(P[0], P[1], P[2], P[3], v);
}

// glm 0.9.9 mat4 * vec4 (scalar path): (m0*x + m1*y) + (m2*z + m3*w), the
// columns m0..m3 scaled component-wise.  Used as vec3(mv * vec4(p, 1))
// (src/Reyes/BoundNSplitCLCPU.cpp:268,313).
static inline V3 mul_mv_point(const float* m, const V3& p) {
    V3 r;
    r.x = (m[0] * p.x + m[4] * p.y) + (m[8] * p.z + m[12] * 1.0f);
    r.y = (m[1] * p.x + m[5] * p.y) + (m[9] * p.z + m[13] * 1.0f);
    r.z = (m[2] * p.x + m[6] * p.y) + (m[10] * p.z + m[14] * 1.0f);
    return r;
}

// glm::distance(a, b) = sqrt(dot(b - a, b - a)), dot = (x*x + y*y) + z*z.
static inline float distance(const V3& a, const V3& b) {
    float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    return std::sqrt(dx * dx + dy * dy + dz * dz);
}

// src/base/Projection.cpp:23-35
struct Projection {
    float near_plane;
    int vx, vy;
    float fx, fy, vpx, vpy;
    float cull_ribbon;
    void init(float fovy, float hither, int w, int h, float ribbon) {
        near_plane = hither;
        vx = w;
        vy = h;
        float aspect = float(w) / h;
        fy = 1.0f / (float)std::tan(fovy * M_PI / 360);
        fx = fy / aspect;
        vpx = w / 2.0f;
        vpy = h / 2.0f;
        fx *= vpx;
        fy *= vpy;
        cull_ribbon = ribbon;
    }
    // src/base/Projection.cpp:57-106
    void bound(const BBox& bbox, V2& size, bool& cull) const {
        V2 mn, mx;
        float n = -bbox.max.z;
        float f = -bbox.min.z;
        if (f < near_plane) { cull = true; return; }
        n = maximum(near_plane, n);
        mn.x = (bbox.min.x < 0) ? bbox.min.x / n * fx + vpx : bbox.min.x / f * fx + vpx;
        mn.y = (bbox.min.y < 0) ? bbox.min.y / n * fy + vpy : bbox.min.y / f * fy + vpy;
        mx.x = (bbox.max.x > 0) ? bbox.max.x / n * fx + vpx : bbox.max.x / f * fx + vpx;
        mx.y = (bbox.max.y > 0) ? bbox.max.y / n * fy + vpy : bbox.max.y / f * fy + vpy;
        if (mn.x > vx - 1 + cull_ribbon || mx.x < -cull_ribbon ||
            mn.y > vy - 1 + cull_ribbon || mx.y < -cull_ribbon) {
            cull = true;
            return;
        }
        size = V2{mx.x - mn.x, mx.y - mn.y};
        cull = false;
    }
};

// src/Reyes/PatchRange.h:9-27
struct PatchRange {
    float minx, miny, maxx, maxy;
    int64_t depth;
    int64_t patch_id;
    // split path: bit 31 - d is 1 when the range is the high half of its
    // depth-d ancestor's split (not in the reference's record; it names the
    // range's place in the split tree for the canonical order below)
    uint32_t path;
};

// Path of the high half of a split of r (the low half keeps r's path).
static inline uint32_t high_path(const PatchRange& r) {
    return r.depth < 32 ? r.path | (0x80000000u >> r.depth) : r.path;
}

// src/Reyes/BoundNSplitCLCPU.cpp:249-336 -- 3x3 samples at
// min + (max-min)*i*0.5; v from range.x, u from range.y.
static void bound_range(const PatchRange& r, const float* cp, int type, const float* mv,
                        BBox& box, float& vlen, float& hlen) {
    const int RES = 3;
    V3 ps[RES][RES];
    box.clear();
    for (int iu = 0; iu < RES; ++iu) {
        for (int iv = 0; iv < RES; ++iv) {
            float v = r.minx + (r.maxx - r.minx) * (float)iu * (1.0f / (RES - 1));
            float u = r.miny + (r.maxy - r.miny) * (float)iv * (1.0f / (RES - 1));
            V3 pos = (type == 0) ? eval_patch(cp + 3 * 16 * r.patch_id, u, v)
                                 : eval_gregory_patch(cp + 3 * 20 * r.patch_id, u, v);
            V3 pt = mul_mv_point(mv, pos);
            box.add_point(pt);
            ps[iu][iv] = pt;
        }
    }
    vlen = 0;
    hlen = 0;
    for (int i = 0; i < RES; ++i) {
        float h = 0, v = 0;
        for (int j = 0; j < RES - 1; ++j) {
            v += distance(ps[j][i], ps[j + 1][i]);
            h += distance(ps[i][j], ps[i][j + 1]);
        }
        vlen = maximum(v, vlen);
        hlen = maximum(h, hlen);
    }
}

// The reference's GPU criterion (kernels/bound_n_split.h), defined with the
// kernel restatement below.
enum GpuBound { kGpuCull = 0, kGpuDraw = 1, kGpuHSplit = 2, kGpuVSplit = 6 };
static int bound_gpu(const or_params* P, const or_draw* d, const PatchRange& r);

// src/Reyes/BoundNSplitCLCPU.cpp:31-56 (init) and 75-159 (the LIFO loop).
// Batches of reyes_patches_per_pass only cut the emission sequence into
// passes; the sequence itself does not depend on the batch size.  With the
// GPU criterion the same loop applies kernels/bound_n_split.h's decision
// (the emitted set does not depend on the traversal order; VSPLIT halves x,
// HSPLIT halves y, kernels/bound_n_split_multipass.cl:111-125).
template <typename Emit>
static int64_t bound_n_split(const or_params* P, const or_draw* d, Emit emit) {
    Projection proj;
    proj.init(P->fovy_deg, P->near_plane, P->width, P->height, P->cull_ribbon);
    std::vector<PatchRange> stack((size_t)d->n_patches);
    for (int64_t i = 0; i < d->n_patches; ++i) stack[(size_t)i] = PatchRange{0, 0, 1, 1, 0, i, 0};
    const float s = P->bound_n_split_limit;
    int64_t bounds = 0;
    BBox box;
    float vlen, hlen;
    while (!stack.empty()) {
        PatchRange r = stack.back();
        stack.pop_back();
        if (P->bound_criterion == 1) {
            ++bounds;
            const int g = bound_gpu(P, d, r);
            if (g == kGpuDraw) {
                emit(r);
            } else if (g == kGpuHSplit) {
                float cy = (r.miny + r.maxy) * 0.5f;
                stack.push_back(PatchRange{r.minx, r.miny, r.maxx, cy, r.depth + 1, r.patch_id, r.path});
                stack.push_back(PatchRange{r.minx, cy, r.maxx, r.maxy, r.depth + 1, r.patch_id, high_path(r)});
            } else if (g == kGpuVSplit) {
                float cx = (r.minx + r.maxx) * 0.5f;
                stack.push_back(PatchRange{r.minx, r.miny, cx, r.maxy, r.depth + 1, r.patch_id, r.path});
                stack.push_back(PatchRange{cx, r.miny, r.maxx, r.maxy, r.depth + 1, r.patch_id, high_path(r)});
            }
            continue;
        }
        bound_range(r, d->cp, d->type, d->mv, box, vlen, hlen);
        ++bounds;
        V2 size;
        bool cull;
        proj.bound(box, size, cull);
        if (cull) continue;
        if (box.min.z < 0 && size.x < s && size.y < s) {
            emit(r);
        } else if (r.depth > (int64_t)P->max_split_depth) {
            // depth cap: the range is dropped
        } else if (vlen < hlen) {
            // vsplit_range (:231-237): halve y, push low half then high half
            float cy = (r.miny + r.maxy) * 0.5f;
            stack.push_back(PatchRange{r.minx, r.miny, r.maxx, cy, r.depth + 1, r.patch_id, r.path});
            stack.push_back(PatchRange{r.minx, cy, r.maxx, r.maxy, r.depth + 1, r.patch_id, high_path(r)});
        } else {
            // hsplit_range (:239-245): halve x
            float cx = (r.minx + r.maxx) * 0.5f;
            stack.push_back(PatchRange{r.minx, r.miny, cx, r.maxy, r.depth + 1, r.patch_id, r.path});
            stack.push_back(PatchRange{cx, r.miny, r.maxx, r.maxy, r.depth + 1, r.patch_id, high_path(r)});
        }
    }
    return bounds;
}

// ---------------------------------------------------------------------------
// Kernel restatement helpers (conventions R1-R6 in the file header).

static inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }

// R4
static inline int32_t f2i_rz_sat(float x) {
    if (std::isnan(x)) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
}

static inline float fmaxnan(float a, float b) { return std::fmax(a, b); }

// R2
static inline float kdiv(float x, float y) { return x * (1.0f / y); }

}  // namespace

// Cosine (the adjoint's derivative of the displacement) by Cody-Waite
// reduction with pi/2 = P1 + P2 + P3 (three floats taken from the exact value
// of pi) and Taylor polynomials of degree 9 (sin) and 10 (cos) on
// |r| <= pi/4, all in float with fused multiply-adds.
static const float kTwoOverPi = 0x1.45f306p-1f;
static const float kP1 = 0x1.921fb6p+0f;
static const float kP2 = -0x1.777a5cp-25f;
static const float kP3 = -0x1.ee59dap-50f;

static inline void or_sincos_reduced(float x, float& sr, float& cr, int& q) {
    float k = std::rint(x * kTwoOverPi);
    float r = std::fma(-k, kP1, x);
    r = std::fma(-k, kP2, r);
    r = std::fma(-k, kP3, r);
    float kq = k - 4.0f * std::floor(k * 0.25f);
    q = (int)kq;
    float r2 = r * r;
    float ps = std::fma(r2, 0x1.71de3ap-19f, -0x1.a01a02p-13f);
    ps = std::fma(r2, ps, 0x1.111112p-7f);
    ps = std::fma(r2, ps, -0x1.555556p-3f);
    sr = std::fma(r * r2, ps, r);
    float pc = std::fma(r2, -0x1.27e4fcp-22f, 0x1.a01a02p-16f);
    pc = std::fma(r2, pc, -0x1.6c16c2p-10f);
    pc = std::fma(r2, pc, 0x1.555556p-5f);
    pc = std::fma(r2, pc, -0x1.0p-1f);
    cr = std::fma(r2, pc, 1.0f);
}

// native_sin (R6): reduction by pi = PI1 + PI2 + PI3 (the pi/2 split above
// doubled, exactly) to |r| <= pi/2, the odd Taylor polynomial of degree 13
// in r, and the sign of (-1)^k.  Largest error 1.1e-7 absolute, 1.8 ulp.
static const float kOneOverPi = 0x1.45f306p-2f;
static const float kPi1 = 0x1.921fb6p+1f;
static const float kPi2 = -0x1.777a5cp-24f;
static const float kPi3 = -0x1.ee59dap-49f;

extern "C" float or_sinf(float x) {
    if (!std::isfinite(x)) return x - x;
    const float k = std::rint(x * kOneOverPi);
    float r = std::fma(-k, kPi1, x);
    r = std::fma(-k, kPi2, r);
    r = std::fma(-k, kPi3, r);
    const float r2 = r * r;
    float p = std::fma(r2, 0x1.612462p-33f, -0x1.ae6456p-26f);
    p = std::fma(r2, p, 0x1.71de3ap-19f);
    p = std::fma(r2, p, -0x1.a01a02p-13f);
    p = std::fma(r2, p, 0x1.111112p-7f);
    p = std::fma(r2, p, -0x1.555556p-3f);
    const float sn = std::fma(r * r2, p, r);
    const float odd = k - 2.0f * std::floor(k * 0.5f);
    return odd != 0.0f ? -sn : sn;
}

extern "C" float or_cosf(float x) {
    if (!std::isfinite(x)) return x - x;
    float s, c;
    int q;
    or_sincos_reduced(x, s, c, q);
    switch (q & 3) {
        case 0: return c;
        case 1: return -s;
        case 2: return -c;
        default: return s;
    }
}

namespace {

// kernels/utility.h:121-152 -- p += (v_i * c_j) * P[4i+j], i-major.  Control
// points are float4 (x, y, z, 1) as PatchIndex.cpp:86-89 widens them.
static inline V4 eval_bezier_k(const float* cp, float tx, float ty) {
    float sx = 1 - tx, sy = 1 - ty;
    float vw[4] = {sx * sx * sx, 3 * sx * sx * tx, 3 * sx * tx * tx, tx * tx * tx};
    float cw[4] = {1 * sy * sy * sy, 3 * ty * sy * sy, 3 * ty * ty * sy, 1 * ty * ty * ty};
    V4 p{0, 0, 0, 0};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            float w = vw[i] * cw[j];
            const float* P = cp + 3 * (4 * i + j);
            p.x = std::fma(w, P[0], p.x);
            p.y = std::fma(w, P[1], p.y);
            p.z = std::fma(w, P[2], p.z);
            p.w = std::fma(w, 1.0f, p.w);
        }
    return p;
}

static inline float sel_nan(float x) { return std::isnan(x) ? 0.0f : x; }

// kernels/utility.h:155-206 -- Gregory patch with NaN face blends zeroed.
static inline V4 eval_gregory_k(const float* cp, float tx, float ty) {
    float sx = 1 - tx, sy = 1 - ty;
    float u = tx, v = ty;
    auto P = [&](int k) { return V4{cp[3 * k], cp[3 * k + 1], cp[3 * k + 2], 1.0f}; };
    auto blend = [&](float a, V4 A, float b, V4 B, float den) {
        // (a*A + b*B) / den with R1: fma(b, B, a*A)
        V4 r;
        r.x = sel_nan(kdiv(std::fma(b, B.x, a * A.x), den));
        r.y = sel_nan(kdiv(std::fma(b, B.y, a * A.y), den));
        r.z = sel_nan(kdiv(std::fma(b, B.z, a * A.z), den));
        r.w = sel_nan(kdiv(std::fma(b, B.w, a * A.w), den));
        return r;
    };
    V4 F0 = blend(u, P(12), v, P(16), u + v);
    V4 F1 = blend(1 - u, P(17), v, P(13), 1 - u + v);
    V4 F2 = blend(1 - u, P(14), 1 - v, P(18), 2 - u - v);
    V4 F3 = blend(u, P(19), 1 - v, P(15), 1 + u - v);
    V4 pts[16] = {P(0), P(4), P(9), P(1), P(8), F0, F1, P(5),
                  P(7), F3, F2, P(10), P(3), P(11), P(6), P(2)};
    float vw[4] = {sx * sx * sx, 3 * sx * sx * tx, 3 * sx * tx * tx, tx * tx * tx};
    float cw[4] = {1 * sy * sy * sy, 3 * ty * sy * sy, 3 * ty * ty * sy, 1 * ty * ty * ty};
    V4 p{0, 0, 0, 0};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            float w = vw[i] * cw[j];
            const V4& Q = pts[4 * i + j];
            p.x = std::fma(w, Q.x, p.x);
            p.y = std::fma(w, Q.y, p.y);
            p.z = std::fma(w, Q.z, p.z);
            p.w = std::fma(w, Q.w, p.w);
        }
    return p;
}

// dot() (R1: x*x' + y*y' is fma(x, x', y*y'), then one fused multiply-add
// per further term)
static inline float dot4(const float* a, const V4& b) {
    return std::fma(a[3], b.w, std::fma(a[2], b.z, std::fma(a[0], b.x, a[1] * b.y)));
}
static inline float dot3(const V3& a, const V3& b) {
    return std::fma(a.z, b.z, std::fma(a.x, b.x, a.y * b.y));
}

// kernels/utility.h:174-180 -- row r of a column-major float16 is (m[r], m[4+r], m[8+r], m[12+r]).
static inline V4 mul_m44v4(const float* m, const V4& v) {
    float r0[4] = {m[0], m[4], m[8], m[12]};
    float r1[4] = {m[1], m[5], m[9], m[13]};
    float r2[4] = {m[2], m[6], m[10], m[14]};
    float r3[4] = {m[3], m[7], m[11], m[15]};
    return V4{dot4(r0, v), dot4(r1, v), dot4(r2, v), dot4(r3, v)};
}

static inline V3 cross3(const V3& a, const V3& b) {
    return V3{std::fma(-a.z, b.y, a.y * b.z), std::fma(-a.x, b.z, a.z * b.x),
              std::fma(-a.y, b.x, a.x * b.y)};
}

static inline V3 normalize3(const V3& v) {
    float l = std::sqrt(dot3(v, v));
    return V3{kdiv(v.x, l), kdiv(v.y, l), kdiv(v.z, l)};
}

// glm::perspective<float>(fovy, aspect, near, far), right-handed, depth -1..1.
static void perspective(float fovy_rad, float aspect, float zn, float zf, float* m) {
    float th = std::tan(fovy_rad / 2.0f);
    std::memset(m, 0, 16 * sizeof(float));
    m[0] = 1.0f / (aspect * th);
    m[5] = 1.0f / th;
    m[10] = -(zf + zn) / (zf - zn);
    m[11] = -1.0f;
    m[14] = -(2.0f * zf * zn) / (zf - zn);
}

// kernels/bound_n_split.h:8-100 -- the reference's GPU bound criterion for
// one range, in the kernel arithmetic (R1-R6): 3x3 samples at
// mix(rmin, rmax, (u, v) / 2) through the kernel patch evaluation and the
// modelview, an eye-space bbox with fmin/fmax, screen positions
// screen_matrix * (p.xy / p.w) with screen_matrix = diag(W/2, H/2)
// (Projection.cpp:42-45), outside_frustum with far = 1000
// (Projection.h:49), the eye-plane split rule, then <= on the larger of the
// summed screen distances along u (h) and v (v).
static int bound_gpu(const or_params* P, const or_draw* d, const PatchRange& r) {
    if (r.depth >= (int64_t)P->max_split_depth - 1) return kGpuCull;
    const int W = P->width, H = P->height;
    const float aspect = float(W) / H;
    float proj[16];
    perspective((float)(P->fovy_deg * M_PI / 180), aspect, P->near_plane, 10000.0f, proj);
    Projection pr;
    pr.init(P->fovy_deg, P->near_plane, W, H, P->cull_ribbon);
    const float inf = std::numeric_limits<float>::infinity();
    V3 mn{inf, inf, inf}, mx{-inf, -inf, -inf};
    V2 pp[3][3];
    const int ncp = d->type == 0 ? 16 : 20;
    const float* cp = d->cp + (int64_t)r.patch_id * 3 * ncp;
    for (int u = 0; u < 3; ++u)
        for (int v = 0; v < 3; ++v) {
            float tx = std::fma(r.maxx - r.minx, (float)u * 0.5f, r.minx);
            float ty = std::fma(r.maxy - r.miny, (float)v * 0.5f, r.miny);
            V4 o = d->type == 0 ? eval_bezier_k(cp, tx, ty) : eval_gregory_k(cp, tx, ty);
            V4 p = mul_m44v4(d->mv, o);
            mn = V3{std::fmin(mn.x, p.x), std::fmin(mn.y, p.y), std::fmin(mn.z, p.z)};
            mx = V3{std::fmax(mx.x, p.x), std::fmax(mx.y, p.y), std::fmax(mx.z, p.z)};
            V4 q = mul_m44v4(proj, p);
            float rw = 1.0f / q.w;
            float x = q.x * rw, y = q.y * rw;
            pp[v][u] = V2{std::fma(0.0f, y, pr.vpx * x), std::fma(pr.vpy, y, 0.0f * x)};
        }
    // outside_frustum
    float n = -mx.z, f = -mn.z;
    if (f < P->near_plane || n > 1000.0f) return kGpuCull;
    n = std::fmax(P->near_plane, n);
    // x / n * f.x + screen_size.x * 0.5 with a double literal: the float
    // product is rounded, then W/2 is added exactly in double and the sum
    // rounded to float -- the same as one float addition.
    float sminx = (float)((double)(kdiv(mn.x, mn.x < 0 ? n : f) * pr.fx) + P->width * 0.5);
    float sminy = (float)((double)(kdiv(mn.y, mn.y < 0 ? n : f) * pr.fy) + P->height * 0.5);
    float smaxx = (float)((double)(kdiv(mx.x, mx.x > 0 ? n : f) * pr.fx) + P->width * 0.5);
    float smaxy = (float)((double)(kdiv(mx.y, mx.y > 0 ? n : f) * pr.fy) + P->height * 0.5);
    if (sminx > (float)(W - 1) + P->cull_ribbon || smaxx < -P->cull_ribbon ||
        sminy > (float)(H - 1) + P->cull_ribbon || smaxy < -P->cull_ribbon)
        return kGpuCull;
    // eps = P->near * 0.1 with a double literal
    const float eps = (float)((double)P->near_plane * 0.1);
    if (mn.z < eps && mx.z > P->near_plane) return (r.maxx - r.minx) < (r.maxy - r.miny) ? kGpuVSplit : kGpuHSplit;
    float hlen = 0, vlen = 0;
    for (int i = 0; i < 3; ++i) {
        float h = 0, v = 0;
        for (int j = 0; j < 2; ++j) {
            float hx = pp[i][j].x - pp[i][j + 1].x, hy = pp[i][j].y - pp[i][j + 1].y;
            float vx = pp[j][i].x - pp[j + 1][i].x, vy = pp[j][i].y - pp[j + 1][i].y;
            h += std::sqrt(std::fma(hx, hx, hy * hy));
            v += std::sqrt(std::fma(vx, vx, vy * vy));
        }
        hlen = std::fmax(h, hlen);
        vlen = std::fmax(v, vlen);
    }
    if (hlen <= P->bound_n_split_limit && vlen <= P->bound_n_split_limit) return kGpuDraw;
    return hlen > vlen ? kGpuVSplit : kGpuHSplit;
}

struct Frame {
    const or_params* P;
    int W, H, PS, shift;
    int gx, gy;              // framebuffer tile grid (8-pixel tiles)
    float proj[16];
    float fdisp[3];
    V4 clear;
    float* color;
    int32_t* depth;
    int64_t* win;
    int64_t n_frag = 0;

    void init(const or_params* p, float* c, int32_t* d, int64_t* w) {
        P = p;
        W = p->width;
        H = p->height;
        PS = p->reyes_patch_size;
        shift = p->subpixel_bits;
        gx = (W + 7) / 8;
        gy = (H + 7) / 8;
        // src/base/Projection.cpp:37-40: perspective(fovy*pi/180, aspect, near, 10000)
        float aspect = float(W) / H;
        perspective((float)(p->fovy_deg * M_PI / 180), aspect, p->near_plane, 10000.0f, proj);
        fdisp[0] = 0.04f * p->displacement_amplitude;
        fdisp[1] = 0.02f * p->displacement_amplitude;
        fdisp[2] = 0.01f * p->displacement_amplitude;
        // src/Reyes/Framebuffer.cpp:63-72 -- clear colour ^2.2, alpha 1000
        clear = V4{powf(p->clear_color[0], 2.2f), powf(p->clear_color[1], 2.2f),
                   powf(p->clear_color[2], 2.2f), 1000.0f};
        color = c;
        depth = d;
        win = w;
        // kernels/framebuffer.cl:20-24 and src/Reyes/RendererCL.cpp:123-126
        for (int64_t i = 0; i < (int64_t)gx * gy * 64; ++i) {
            color[4 * i + 0] = clear.x;
            color[4 * i + 1] = clear.y;
            color[4 * i + 2] = clear.z;
            color[4 * i + 3] = clear.w;
            depth[i] = 0x7fffffff;
            if (win) win[i] = -1;
        }
    }

    // kernels/reyes.cl:37-45
    int64_t fb_pos(int x, int y) const {
        int tx = x / 8, ty = y / 8;
        return ((int64_t)(tx + gx * ty)) * 64 + (x - tx * 8) + 8 * (y - ty * 8);
    }

    // kernels/dice.cl:37-80 for one vertex
    void dice_vertex(const or_draw* d, int32_t pid, const float* range, int nu, int nv,
                     V4& pos, int32_t& px, int32_t& py, float& dep) const {
        float tx = std::fma(range[2] - range[0], nu / (float)PS, range[0]);
        float ty = std::fma(range[3] - range[1], nv / (float)PS, range[1]);
        V4 op = (d->type == 0) ? eval_bezier_k(d->cp + (int64_t)pid * 48, tx, ty)
                               : eval_gregory_k(d->cp + (int64_t)pid * 60, tx, ty);
        pos = mul_m44v4(d->mv, op);
        if (P->displacement) {
            const float k[3] = {5, 7, 11};
            for (int i = 0; i < 3; ++i) {
                float f = fdisp[i];
                pos.x = std::fma(or_sinf(pos.y * k[i] * 2), f, pos.x);
                pos.y = std::fma(or_sinf(pos.x * k[i] * 2), f, pos.y);
                pos.z = std::fma(or_sinf(pos.y * k[i] * 2) * or_sinf(pos.x * 3 * 2), f, pos.z);
            }
        }
        V4 p = mul_m44v4(proj, pos);
        int32_t vsx = W << shift, vsy = H << shift;
        float ex = (kdiv(p.x, p.w) * (float)vsx) / 2 + (float)(vsx / 2);
        float ey = (kdiv(p.y, p.w) * (float)vsy) / 2 + (float)(vsy / 2);
        px = f2i_rz_sat(ex);
        py = f2i_rz_sat(ey);
        dep = kdiv(p.z, p.w);
    }

    // kernels/reyes.cl:172-191 -- flat colour of a quad from its 4 eye positions
    V4 shade(const V4* pos, const float* dc) const {
        V3 du{(((pos[1].x - pos[0].x) + pos[3].x) - pos[2].x) * 0.5f,
              (((pos[1].y - pos[0].y) + pos[3].y) - pos[2].y) * 0.5f,
              (((pos[1].z - pos[0].z) + pos[3].z) - pos[2].z) * 0.5f};
        V3 dv{(((pos[2].x - pos[0].x) + pos[3].x) - pos[1].x) * 0.5f,
              (((pos[2].y - pos[0].y) + pos[3].y) - pos[1].y) * 0.5f,
              (((pos[2].z - pos[0].z) + pos[3].z) - pos[1].z) * 0.5f};
        V3 n = normalize3(cross3(dv, du));
        V3 l = normalize3(V3{4, 3, 8});
        float m = fmaxnan(dot3(n, l), 0.0f);
        const float ac[4] = {0.015f, 0.015f, 0.015f, 1.0f};
        // ac*dc + max(dot(n,l),0)*dc + pow(max(dot(n,h),0),60)*sc with sc = 0:
        // the last term is +0 for every finite base, which R3 guarantees.
        return V4{std::fma(m, dc[0], ac[0] * dc[0]) + 0.0f, std::fma(m, dc[1], ac[1] * dc[1]) + 0.0f,
                  std::fma(m, dc[2], ac[2] * dc[2]) + 0.0f, std::fma(m, dc[3], ac[3] * dc[3]) + 0.0f};
    }

    // kernels/reyes.cl:240-265 (wrapping int32, R5)
    static int inside_triangle(const int32_t* Px, const int32_t* Py, int32_t tx, int32_t ty,
                               const float* dv, float* depth) {
        int32_t Dx[3], Dy[3], O[3], C[3], V[3], Dn[3];
        for (int e = 0; e < 3; ++e) {
            int en = (e + 1) % 3;
            Dx[e] = wsub(Py[en], Py[e]);
            Dy[e] = wsub(Px[e], Px[en]);
        }
        for (int e = 0; e < 3; ++e) {
            O[e] = wadd(wmul(Dx[e], Px[e]), wmul(Dy[e], Py[e]));
            C[e] = (Dx[e] > 0 || (Dx[e] == 0 && Dy[e] > 0)) ? -1 : 0;
            V[e] = wsub(wadd(wmul(Dx[e], tx), wmul(Dy[e], ty)), O[e]);
        }
        int success = (V[0] > C[0]) && (V[1] > C[1]) && (V[2] > C[2]);
        // weights = V.yzx / (idot3(Dx.yzx, Dy.yzx, Px, Py) - O.yzx)
        float w[3];
        for (int e = 0; e < 3; ++e) {
            int en = (e + 1) % 3;
            Dn[e] = wsub(wadd(wmul(Dx[en], Px[e]), wmul(Dy[en], Py[e])), O[en]);
            w[e] = kdiv((float)V[en], (float)Dn[e]);
        }
        float d = std::fma(dv[2], w[2], std::fma(dv[1], w[1], dv[0] * w[0]));
        *depth = (success && d < *depth) ? d : *depth;
        return success;
    }

    // kernels/dice.cl + kernels/reyes.cl (shade, sample) for one sub-patch.
    // Quads are visited in (nv, nu) order; a fragment replaces the stored one
    // only when strictly nearer, so ties keep the first writer.
    void draw_subpatch(const or_draw* d, int32_t pid, const float* range, int64_t mp_base) {
        const int G = PS + 1;
        std::vector<V4> pos((size_t)G * G);
        std::vector<int32_t> pxl((size_t)G * G * 2);
        std::vector<float> dep((size_t)G * G);
        for (int nv = 0; nv < G; ++nv)
            for (int nu = 0; nu < G; ++nu) {
                int i = nu + nv * G;
                dice_vertex(d, pid, range, nu, nv, pos[i], pxl[2 * i], pxl[2 * i + 1], dep[i]);
            }
        const int32_t VMAXx = (W << shift) - 1, VMAXy = (H << shift) - 1;
        const int32_t MAXL = (8 << shift) - 1;
        const int BPL = PS / 8;
        for (int bv = 0; bv < BPL; ++bv)
            for (int bu = 0; bu < BPL; ++bu) {
                // shade: block bound over front-facing quads, allnormal flag
                int32_t xmin = VMAXx, ymin = VMAXy, xmax = 0, ymax = 0;
                bool allnormal = true;
                for (int ly = 0; ly < 8; ++ly)
                    for (int lx = 0; lx < 8; ++lx) {
                        int nu = bu * 8 + lx, nv = bv * 8 + ly;
                        int32_t qx[4], qy[4];
                        int32_t pminx = VMAXx, pminy = VMAXy, pmaxx = 0, pmaxy = 0;
                        for (int k = 0; k < 4; ++k) {
                            int gi = (nu + (k & 1)) + (nv + (k >> 1)) * G;
                            if (pos[gi].z == 0) allnormal = false;
                            qx[k] = pxl[2 * gi];
                            qy[k] = pxl[2 * gi + 1];
                            pminx = std::min(pminx, qx[k]);
                            pminy = std::min(pminy, qy[k]);
                            pmaxx = std::max(pmaxx, qx[k]);
                            pmaxy = std::max(pmaxy, qy[k]);
                        }
                        bool ff = true;
                        if (P->backface_culling) {
                            int32_t d1x = wsub(qx[1], qx[0]), d1y = wsub(qy[1], qy[0]);
                            int32_t d2x = wsub(qx[2], qx[0]), d2y = wsub(qy[2], qy[0]);
                            int32_t d3x = wsub(qx[3], qx[0]), d3y = wsub(qy[3], qy[0]);
                            ff = wsub(wmul(d1x, d3y), wmul(d3x, d1y)) < 0 ||
                                 wsub(wmul(d3x, d2y), wmul(d2x, d3y)) < 0;
                        }
                        if (ff) {
                            xmin = std::min(xmin, pminx);
                            ymin = std::min(ymin, pminy);
                            xmax = std::max(xmax, pmaxx);
                            ymax = std::max(ymax, pmaxy);
                        }
                    }
                xmin = std::max(0, xmin);
                ymin = std::max(0, ymin);
                xmax = std::min(VMAXx, xmax);
                ymax = std::min(VMAXy, ymax);
                if (!allnormal) { xmin = 1; ymin = 1; xmax = -1; ymax = -1; }
                // sample (kernels/reyes.cl:270-398), including the
                // is_empty(block_bound.xy, block_bound.zx) test of :287
                if (xmin >= xmax && ymin >= xmin) continue;
                int32_t mintx = xmin >> (shift + 3), minty = ymin >> (shift + 3);
                int32_t maxtx = xmax >> (shift + 3), maxty = ymax >> (shift + 3);
                for (int ly = 0; ly < 8; ++ly)
                    for (int lx = 0; lx < 8; ++lx) {
                        int nu = bu * 8 + lx, nv = bv * 8 + ly;
                        int32_t Px[4], Py[4];
                        float dv4[4];
                        V4 qpos[4];
                        int32_t mingx = VMAXx + 1, mingy = VMAXy + 1, maxgx = -1, maxgy = -1;
                        for (int k = 0; k < 4; ++k) {
                            int gi = (nu + (k & 1)) + (nv + (k >> 1)) * G;
                            Px[k] = pxl[2 * gi];
                            Py[k] = pxl[2 * gi + 1];
                            dv4[k] = dep[gi];
                            qpos[k] = pos[gi];
                            mingx = std::min(mingx, Px[k]);
                            mingy = std::min(mingy, Py[k]);
                            maxgx = std::max(maxgx, Px[k]);
                            maxgy = std::max(maxgy, Py[k]);
                        }
                        V4 c = shade(qpos, d->color);
                        int64_t mp_id = mp_base + nu + (int64_t)nv * PS;
                        const int32_t t1x[3] = {Px[0], Px[1], Px[3]}, t1y[3] = {Py[0], Py[1], Py[3]};
                        const int32_t t2x[3] = {Px[0], Px[3], Px[2]}, t2y[3] = {Py[0], Py[3], Py[2]};
                        const float d1[3] = {dv4[0], dv4[1], dv4[3]};
                        const float d2[3] = {dv4[0], dv4[3], dv4[2]};
                        for (int ty = minty; ty <= maxty; ++ty)
                            for (int tx = mintx; tx <= maxtx; ++tx) {
                                int32_t osx = (tx * 8) << shift, osy = (ty * 8) << shift;
                                int32_t mnx = std::min(std::max(wsub(mingx, osx), 0), MAXL) >> shift;
                                int32_t mny = std::min(std::max(wsub(mingy, osy), 0), MAXL) >> shift;
                                int32_t mxx = std::min(std::max(wsub(maxgx, osx), 0), MAXL) >> shift;
                                int32_t mxy = std::min(std::max(wsub(maxgy, osy), 0), MAXL) >> shift;
                                for (int y = mny; y <= mxy; ++y)
                                    for (int x = mnx; x <= mxx; ++x) {
                                        int32_t tpx = wadd(x << shift, osx), tpy = wadd(y << shift, osy);
                                        float depth = 1;
                                        int in1 = inside_triangle(t1x, t1y, tpx, tpy, d1, &depth);
                                        int in2 = inside_triangle(t2x, t2y, tpx, tpy, d2, &depth);
                                        if (!(in1 || in2)) continue;
                                        ++n_frag;
                                        float cl = std::min(std::max(kdiv(depth, 200.0f), 0.0f), 1.0f);
                                        int32_t idepth = f2i_rz_sat(cl * (float)0x7fffffff);
                                        int64_t fb = fb_pos(tx * 8 + x, ty * 8 + y);
                                        if (idepth < this->depth[fb]) {
                                            this->depth[fb] = idepth;
                                            color[4 * fb + 0] = c.x;
                                            color[4 * fb + 1] = c.y;
                                            color[4 * fb + 2] = c.z;
                                            color[4 * fb + 3] = c.w;
                                            if (win) win[fb] = mp_id;
                                        }
                                    }
                            }
                    }
            }
    }
};

// ---------------------------------------------------------------------------
// FP64 dicer and gradient

struct D3 { double x, y, z; };

static inline double bern(int i, double t) {
    double s = 1 - t;
    switch (i) {
        case 0: return s * s * s;
        case 1: return 3 * s * s * t;
        case 2: return 3 * s * t * t;
        default: return t * t * t;
    }
}

// Weight of every control point of one patch at (tx, ty): 16 for Bezier,
// 20 for Gregory (face blends expanded; NaN blends are zero).
static int cp_weights(int type, double tx, double ty, double* w) {
    if (type == 0) {
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) w[4 * i + j] = bern(i, tx) * bern(j, ty);
        return 16;
    }
    for (int k = 0; k < 20; ++k) w[k] = 0;
    double u = tx, v = ty;
    // slot -> (control point, blend weight) pairs, mirroring eval_gregory_k
    struct Blend { int a; double wa; int b; double wb; };
    auto mk = [](int a, double na, int b, double nb, double den) {
        Blend r{a, na / den, b, nb / den};
        if (!std::isfinite(r.wa) || !std::isfinite(r.wb)) { r.wa = 0; r.wb = 0; }
        return r;
    };
    Blend F0 = mk(12, u, 16, v, u + v);
    Blend F1 = mk(17, 1 - u, 13, v, 1 - u + v);
    Blend F2 = mk(14, 1 - u, 18, 1 - v, 2 - u - v);
    Blend F3 = mk(19, u, 15, 1 - v, 1 + u - v);
    const int slot_cp[16] = {0, 4, 9, 1, 8, -1, -2, 5, 7, -4, -3, 10, 3, 11, 6, 2};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            double b = bern(i, tx) * bern(j, ty);
            int s = slot_cp[4 * i + j];
            if (s >= 0) { w[s] += b; continue; }
            const Blend& F = (s == -1) ? F0 : (s == -2) ? F1 : (s == -3) ? F2 : F3;
            w[F.a] += b * F.wa;
            w[F.b] += b * F.wb;
        }
    return 20;
}

struct DispTrace { double x[4], y[4], z[4]; };

// eye-space position of one dice vertex in FP64 (with displacement).
static D3 vertex_fp64(const or_params* P, const or_draw* d, const double* cp, int32_t pid,
                      const float* range, int nu, int nv, double amp, double* w, int& nw,
                      DispTrace* tr) {
    int PS = P->reyes_patch_size;
    double tx = (double)range[0] + ((double)range[2] - range[0]) * nu / PS;
    double ty = (double)range[1] + ((double)range[3] - range[1]) * nv / PS;
    nw = cp_weights(d->type, tx, ty, w);
    const double* base = cp + (int64_t)pid * nw * 3;
    D3 o{0, 0, 0};
    double wsum = 0;
    for (int k = 0; k < nw; ++k) {
        o.x += w[k] * base[3 * k];
        o.y += w[k] * base[3 * k + 1];
        o.z += w[k] * base[3 * k + 2];
        wsum += w[k];
    }
    const float* m = d->mv;
    D3 e{m[0] * o.x + m[4] * o.y + m[8] * o.z + m[12] * wsum,
         m[1] * o.x + m[5] * o.y + m[9] * o.z + m[13] * wsum,
         m[2] * o.x + m[6] * o.y + m[10] * o.z + m[14] * wsum};
    if (tr) { tr->x[0] = e.x; tr->y[0] = e.y; tr->z[0] = e.z; }
    if (P->displacement) {
        const double K[3] = {10, 14, 22};
        const double F[3] = {0.04 * amp, 0.02 * amp, 0.01 * amp};
        for (int i = 0; i < 3; ++i) {
            e.x += std::sin(K[i] * e.y) * F[i];
            e.y += std::sin(K[i] * e.x) * F[i];
            e.z += std::sin(K[i] * e.y) * std::sin(6 * e.x) * F[i];
            if (tr) { tr->x[i + 1] = e.x; tr->y[i + 1] = e.y; tr->z[i + 1] = e.z; }
        }
    }
    return e;
}

}  // namespace

// ---------------------------------------------------------------------------
// C API

extern "C" int64_t or_bound_n_split(const or_params* p, const or_draw* d, int32_t* pid,
                                    float* range, int64_t cap, int64_t* n_bounds) {
    int64_t n = 0;
    int64_t b = bound_n_split(p, d, [&](const PatchRange& r) {
        if (n < cap) {
            pid[n] = (int32_t)r.patch_id;
            range[4 * n + 0] = r.minx;
            range[4 * n + 1] = r.miny;
            range[4 * n + 2] = r.maxx;
            range[4 * n + 3] = r.maxy;
        }
        ++n;
    });
    if (n_bounds) *n_bounds = b;
    return n;
}

extern "C" int or_render_subpatches(const or_params* p, const or_draw* draws, int32_t n_draws,
                                    int64_t n_sub, const int32_t* sub_draw, const int32_t* sub_pid,
                                    const float* sub_range, float* color, int32_t* depth,
                                    int64_t* win, int64_t* stats) {
    return or_render_subpatches_at(p, draws, n_draws, n_sub, 0, sub_draw, sub_pid, sub_range, color, depth, win,
                                   stats);
}

extern "C" int or_render_subpatches_at(const or_params* p, const or_draw* draws, int32_t n_draws, int64_t n_sub,
                                       int64_t first_index, const int32_t* sub_draw, const int32_t* sub_pid,
                                       const float* sub_range, float* color, int32_t* depth, int64_t* win,
                                       int64_t* stats) {
    if (p->width % 8 || p->height % 8 || (p->reyes_patch_size % 8)) return 1;
    Frame f;
    f.init(p, color, depth, win);
    int64_t PS2 = (int64_t)p->reyes_patch_size * p->reyes_patch_size;
    for (int64_t s = 0; s < n_sub; ++s) {
        int dr = sub_draw ? sub_draw[s] : 0;
        if (dr < 0 || dr >= n_draws) return 2;
        f.draw_subpatch(&draws[dr], sub_pid[s], sub_range + 4 * s, (first_index + s) * PS2);
    }
    if (stats) {
        stats[0] = n_sub;
        stats[1] = n_sub * PS2;
        stats[2] = f.n_frag;
        stats[3] = 0;
    }
    return 0;
}

// One emitted sub-patch of a frame with its canonical sort key.
struct CanonicalSub {
    uint64_t key;     // root << 32 | split path, root = draw's first root + patch id
    int32_t draw;
    int32_t pid;
    float range[4];
};

// Every draw's sub-patches in the canonical order (ascending root, then
// split path: each patch's split tree depth first, low half first), the
// order in which the micropolygons of a frame are numbered.  Its first
// argument the reference does not have: it emits in its stack's order
// (src/Reyes/BoundNSplitCLCPU.cpp:75-159), which this sort puts in a form
// that does not depend on how the work is scheduled.
static std::vector<CanonicalSub> canonical_subpatches(const or_params* p, const or_draw* draws, int32_t n_draws,
                                                      int64_t* n_bounds) {
    std::vector<CanonicalSub> out;
    uint64_t first_root = 0;
    int64_t nb = 0;
    for (int dr = 0; dr < n_draws; ++dr) {
        nb += bound_n_split(p, &draws[dr], [&](const PatchRange& r) {
            const uint64_t root = first_root + (uint64_t)r.patch_id;
            out.push_back(CanonicalSub{(root << 32) | r.path, dr, (int32_t)r.patch_id, {r.minx, r.miny, r.maxx, r.maxy}});
        });
        first_root += (uint64_t)draws[dr].n_patches;
    }
    std::stable_sort(out.begin(), out.end(),
                     [](const CanonicalSub& a, const CanonicalSub& b) { return a.key < b.key; });
    if (n_bounds) *n_bounds = nb;
    return out;
}

extern "C" int64_t or_canonical_subpatches(const or_params* p, const or_draw* draws, int32_t n_draws,
                                           int32_t* draw, int32_t* pid, float* range, uint64_t* key, int64_t cap) {
    const std::vector<CanonicalSub> subs = canonical_subpatches(p, draws, n_draws, nullptr);
    for (int64_t i = 0; i < (int64_t)subs.size() && i < cap; ++i) {
        if (draw) draw[i] = subs[(size_t)i].draw;
        if (pid) pid[i] = subs[(size_t)i].pid;
        if (range) std::memcpy(range + 4 * i, subs[(size_t)i].range, 4 * sizeof(float));
        if (key) key[i] = subs[(size_t)i].key;
    }
    return (int64_t)subs.size();
}

extern "C" int or_render(const or_params* p, const or_draw* draws, int32_t n_draws, float* color,
                         int32_t* depth, int64_t* stats) {
    return or_render_win(p, draws, n_draws, color, depth, nullptr, stats);
}

// The frame with its micropolygons numbered in the canonical order:
// sub-patch s of canonical_subpatches() owns ids s * PS^2 + nu + nv * PS and,
// drawn in that order with the first writer kept at equal depth, the
// smallest id wins a tie.  win (may be NULL) receives the winning id of
// every tiled pixel, or -1.
extern "C" int or_render_win(const or_params* p, const or_draw* draws, int32_t n_draws, float* color,
                             int32_t* depth, int64_t* win, int64_t* stats) {
    if (p->width % 8 || p->height % 8 || (p->reyes_patch_size % 8)) return 1;
    Frame f;
    f.init(p, color, depth, win);
    int64_t PS2 = (int64_t)p->reyes_patch_size * p->reyes_patch_size;
    int64_t n_bounds = 0;
    const std::vector<CanonicalSub> subs = canonical_subpatches(p, draws, n_draws, &n_bounds);
    const int64_t n_sub = (int64_t)subs.size();
    for (int64_t s = 0; s < n_sub; ++s) {
        const CanonicalSub& c = subs[(size_t)s];
        f.draw_subpatch(&draws[c.draw], c.pid, c.range, s * PS2);
    }
    if (stats) {
        stats[0] = n_sub;
        stats[1] = n_sub * PS2;
        stats[2] = f.n_frag;
        stats[3] = n_bounds;
    }
    return 0;
}

extern "C" void or_dice(const or_params* p, const or_draw* d, int32_t pid, const float range[4],
                        float* pos, int32_t* pxl, float* depth) {
    Frame f;
    f.P = p;
    f.W = p->width;
    f.H = p->height;
    f.PS = p->reyes_patch_size;
    f.shift = p->subpixel_bits;
    perspective((float)(p->fovy_deg * M_PI / 180), float(f.W) / f.H, p->near_plane, 10000.0f, f.proj);
    f.fdisp[0] = 0.04f * p->displacement_amplitude;
    f.fdisp[1] = 0.02f * p->displacement_amplitude;
    f.fdisp[2] = 0.01f * p->displacement_amplitude;
    int G = f.PS + 1;
    for (int nv = 0; nv < G; ++nv)
        for (int nu = 0; nu < G; ++nu) {
            int i = nu + nv * G;
            V4 ps;
            f.dice_vertex(d, pid, range, nu, nv, ps, pxl[2 * i], pxl[2 * i + 1], depth[i]);
            pos[4 * i + 0] = ps.x;
            pos[4 * i + 1] = ps.y;
            pos[4 * i + 2] = ps.z;
            pos[4 * i + 3] = ps.w;
        }
}

// kernels/reyes.cl:172-191 for every quad of one sub-patch: colour q =
// nu + nv * PS (the colour grid of calc_color_grid_pos), whether or not its
// 8x8 block is empty.
extern "C" void or_shade_quads(const or_params* p, const or_draw* d, int32_t pid, const float range[4],
                               float* color) {
    const int PS = p->reyes_patch_size, G = PS + 1;
    std::vector<float> pos((size_t)G * G * 4), dep((size_t)G * G);
    std::vector<int32_t> pxl((size_t)G * G * 2);
    or_dice(p, d, pid, range, pos.data(), pxl.data(), dep.data());
    Frame f;
    f.P = p;
    for (int nv = 0; nv < PS; ++nv)
        for (int nu = 0; nu < PS; ++nu) {
            V4 q[4];
            for (int k = 0; k < 4; ++k) {
                const int gi = (nu + (k & 1)) + (nv + (k >> 1)) * G;
                q[k] = V4{pos[4 * gi], pos[4 * gi + 1], pos[4 * gi + 2], pos[4 * gi + 3]};
            }
            const V4 c = f.shade(q, d->color);
            float* o = color + 4 * (nu + nv * PS);
            o[0] = c.x; o[1] = c.y; o[2] = c.z; o[3] = c.w;
        }
}

extern "C" void or_dice_fp64(const or_params* p, const or_draw* d, int32_t pid,
                             const float range[4], double* pos3) {
    int nw = d->type == 0 ? 16 : 20;
    std::vector<double> cp((size_t)(pid + 1) * nw * 3);
    for (size_t i = (size_t)pid * nw * 3; i < cp.size(); ++i) cp[i] = d->cp[i];
    int G = p->reyes_patch_size + 1;
    double w[20];
    for (int nv = 0; nv < G; ++nv)
        for (int nu = 0; nu < G; ++nu) {
            D3 e = vertex_fp64(p, d, cp.data(), pid, range, nu, nv, p->displacement_amplitude, w, nw,
                               nullptr);
            int i = nu + nv * G;
            pos3[3 * i + 0] = e.x;
            pos3[3 * i + 1] = e.y;
            pos3[3 * i + 2] = e.z;
        }
}

// Gradient of L = sum_px sum_ch (c - t)^2 with fixed visibility, by reverse
// accumulation through shade (reyes.cl:172-191), the displacement
// (dice.cl:51-67), the modelview and the Bernstein weights.
extern "C" double or_loss_fp64(const or_params* p, const or_draw* d, int64_t n_sub,
                               const int32_t* sub_pid, const float* sub_range, const int64_t* win,
                               const float* target, const double* cp, double amp,
                               double* grad_cp, double* grad_amp) {
    const int W = p->width, H = p->height, PS = p->reyes_patch_size;
    const int64_t PS2 = (int64_t)PS * PS;
    const int gx = W / 8;
    const double clr[4] = {powf(p->clear_color[0], 2.2f), powf(p->clear_color[1], 2.2f),
                           powf(p->clear_color[2], 2.2f), 1000.0};
    const double ln = std::sqrt(16.0 + 9.0 + 64.0);
    const D3 L{4 / ln, 3 / ln, 8 / ln};
    const double ac[4] = {0.015, 0.015, 0.015, 1.0};
    const double* dc = nullptr;
    double dcv[4] = {d->color[0], d->color[1], d->color[2], d->color[3]};
    dc = dcv;
    int nwp = d->type == 0 ? 16 : 20;
    double loss = 0, gamp = 0;
    if (grad_cp) std::memset(grad_cp, 0, sizeof(double) * (size_t)d->n_patches * nwp * 3);
    double w[4][20];
    DispTrace tr[4];
    for (int64_t i = 0; i < (int64_t)gx * (H / 8) * 64; ++i) {
        const float* t = target + 4 * i;
        int64_t id = win[i];
        if (id < 0 || id >= n_sub * PS2) {
            for (int ch = 0; ch < 4; ++ch) loss += (clr[ch] - t[ch]) * (clr[ch] - t[ch]);
            continue;
        }
        int64_t s = id / PS2;
        int q = (int)(id % PS2);
        int nu = q % PS, nv = q / PS;
        int32_t pid = sub_pid[s];
        const float* rg = sub_range + 4 * s;
        D3 e[4];
        int nw = 0;
        for (int k = 0; k < 4; ++k)
            e[k] = vertex_fp64(p, d, cp, pid, rg, nu + (k & 1), nv + (k >> 1), amp, w[k], nw, &tr[k]);
        D3 du{((e[1].x - e[0].x) + e[3].x - e[2].x) * 0.5, ((e[1].y - e[0].y) + e[3].y - e[2].y) * 0.5,
              ((e[1].z - e[0].z) + e[3].z - e[2].z) * 0.5};
        D3 dv{((e[2].x - e[0].x) + e[3].x - e[1].x) * 0.5, ((e[2].y - e[0].y) + e[3].y - e[1].y) * 0.5,
              ((e[2].z - e[0].z) + e[3].z - e[1].z) * 0.5};
        D3 cr{dv.y * du.z - dv.z * du.y, dv.z * du.x - dv.x * du.z, dv.x * du.y - dv.y * du.x};
        double len = std::sqrt(cr.x * cr.x + cr.y * cr.y + cr.z * cr.z);
        D3 n{cr.x / len, cr.y / len, cr.z / len};
        double nl = n.x * L.x + n.y * L.y + n.z * L.z;
        double m = (nl > 0) ? nl : 0;  // NaN -> 0 as fmax
        double gm = 0;
        for (int ch = 0; ch < 4; ++ch) {
            double c = ac[ch] * dc[ch] + m * dc[ch];
            double r = c - t[ch];
            loss += r * r;
            gm += 2 * r * dc[ch];
        }
        if (!(nl > 0) || !(len > 0) || (!grad_cp && !grad_amp)) continue;
        // m = n.L, n = cr/|cr|: dm/dcr = (L - n (n.L)) / |cr|
        D3 gcr{gm * (L.x - n.x * nl) / len, gm * (L.y - n.y * nl) / len, gm * (L.z - n.z * nl) / len};
        // cr = dv x du: d/d(dv) = du x g, d/d(du) = g x dv
        D3 gdv{du.y * gcr.z - du.z * gcr.y, du.z * gcr.x - du.x * gcr.z, du.x * gcr.y - du.y * gcr.x};
        D3 gdu{gcr.y * dv.z - gcr.z * dv.y, gcr.z * dv.x - gcr.x * dv.z, gcr.x * dv.y - gcr.y * dv.x};
        D3 ge[4];
        const double sdu[4] = {-0.5, 0.5, -0.5, 0.5}, sdv[4] = {-0.5, -0.5, 0.5, 0.5};
        for (int k = 0; k < 4; ++k)
            ge[k] = D3{sdu[k] * gdu.x + sdv[k] * gdv.x, sdu[k] * gdu.y + sdv[k] * gdv.y,
                       sdu[k] * gdu.z + sdv[k] * gdv.z};
        for (int k = 0; k < 4; ++k) {
            double gx_ = ge[k].x, gy_ = ge[k].y, gz_ = ge[k].z;
            if (p->displacement) {
                const double K[3] = {10, 14, 22};
                const double B[3] = {0.04, 0.02, 0.01};
                for (int i = 2; i >= 0; --i) {
                    double F = B[i] * amp;
                    double x0 = tr[k].x[i], y0 = tr[k].y[i];
                    double x1 = tr[k].x[i + 1], y1 = tr[k].y[i + 1];
                    // z1 = z0 + sin(K y1) sin(6 x1) F
                    double sy1 = std::sin(K[i] * y1), s6 = std::sin(6 * x1);
                    gamp += gz_ * sy1 * s6 * B[i];
                    gy_ += gz_ * F * K[i] * std::cos(K[i] * y1) * s6;
                    gx_ += gz_ * F * sy1 * 6 * std::cos(6 * x1);
                    // y1 = y0 + sin(K x1) F
                    gamp += gy_ * std::sin(K[i] * x1) * B[i];
                    gx_ += gy_ * F * K[i] * std::cos(K[i] * x1);
                    // x1 = x0 + sin(K y0) F
                    gamp += gx_ * std::sin(K[i] * y0) * B[i];
                    gy_ += gx_ * F * K[i] * std::cos(K[i] * y0);
                    (void)x0;
                }
            }
            if (!grad_cp) continue;
            const float* mm = d->mv;
            double go[3] = {mm[0] * gx_ + mm[1] * gy_ + mm[2] * gz_,
                            mm[4] * gx_ + mm[5] * gy_ + mm[6] * gz_,
                            mm[8] * gx_ + mm[9] * gy_ + mm[10] * gz_};
            double* gbase = grad_cp + (int64_t)pid * nw * 3;
            for (int j = 0; j < nw; ++j)
                for (int c = 0; c < 3; ++c) gbase[3 * j + c] += w[k][j] * go[c];
        }
    }
    if (grad_amp) *grad_amp = gamp;
    return loss;
}

extern "C" void or_inclusive_scan(const int32_t* in, int32_t* out, int64_t n) {
    int64_t acc = 0;
    for (int64_t i = 0; i < n; ++i) {
        acc += in[i];
        out[i] = (int32_t)acc;
    }
}
