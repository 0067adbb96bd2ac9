// Adjoint of the image with respect to control points and the displacement
// amplitude, with visibility held fixed (the winning micropolygon of every
// pixel comes from the forward pass's depth|id buffer).
//
// One thread per pixel.  The winning quad's four dice vertices are
// recomputed (Bernstein weights, modelview, displacement of
// kernels/dice.cl:51-67) instead of being stored, the flat colour of
// kernels/reyes.cl:172-191 is differentiated back to the four eye
// positions, through the displacement steps in reverse, through the
// modelview, and onto the 16 (Bezier) or 20 (Gregory) control points with
// their Bernstein / face-blend weights.  Lanes of a warp that share one patch
// add their 48 (or 60) partial gradients with warp shuffles before a single
// set of atomics.
#include "mp_internal.h"

namespace mp {

namespace {

__device__ __forceinline__ float bern(int i, float t) {
    float s = 1.0f - t;
    return i == 0 ? s * s * s : i == 1 ? 3.0f * s * s * t : i == 2 ? 3.0f * s * t * t : t * t * t;
}

// Effective weight of every control point at (tx, ty) (the dice evaluators).
__device__ __forceinline__ int cp_weights(int type, float tx, float ty, float* w) {
    if (type == 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) w[4 * i + j] = bern(i, tx) * bern(j, ty);
        return 16;
    }
#pragma unroll
    for (int k = 0; k < 20; ++k) w[k] = 0.0f;
    float u = tx, v = ty;
    auto bl = [](float a, float b, float den, float& wa, float& wb) {
        wa = a / den;
        wb = b / den;
        if (!isfinite(wa) || !isfinite(wb)) { wa = 0.0f; wb = 0.0f; }
    };
    float a0, b0, a1, b1, a2, b2, a3, b3;
    bl(u, v, u + v, a0, b0);                       // F0 = (u P12 + v P16) / (u + v)
    bl(1.0f - u, v, 1.0f - u + v, a1, b1);         // F1 = ((1-u) P17 + v P13) / (1 - u + v)
    bl(1.0f - u, 1.0f - v, 2.0f - u - v, a2, b2);  // F2 = ((1-u) P14 + (1-v) P18) / (2 - u - v)
    bl(u, 1.0f - v, 1.0f + u - v, a3, b3);         // F3 = (u P19 + (1-v) P15) / (1 + u - v)
    const int slot[16] = {0, 4, 9, 1, 8, -1, -2, 5, 7, -4, -3, 10, 3, 11, 6, 2};
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            float b = bern(i, tx) * bern(j, ty);
            int sl = slot[4 * i + j];
            if (sl >= 0) w[sl] += b;
            else if (sl == -1) { w[12] += b * a0; w[16] += b * b0; }
            else if (sl == -2) { w[17] += b * a1; w[13] += b * b1; }
            else if (sl == -3) { w[14] += b * a2; w[18] += b * b2; }
            else { w[19] += b * a3; w[15] += b * b3; }
        }
    return 20;
}

struct VertexTrace {
    float x[4], y[4], z[4];   // eye position before each displacement step and after the last
};

__device__ __forceinline__ void vertex_forward(const DrawDev& d, const FrameDev& fr, const float4* P, float4 r,
                                               int nu, int nv, float4& pos, VertexTrace& tr) {
    float tx = ffma(fsub(r.z, r.x), fdiv((float)nu, (float)fr.PS), r.x);
    float ty = ffma(fsub(r.w, r.y), fdiv((float)nv, (float)fr.PS), r.y);
    float4 o = (d.type == 0) ? eval_bezier_dice(P, tx, ty) : eval_gregory_dice(P, tx, ty);
    pos = mul_m44v4(d.mv, o);
    tr.x[0] = pos.x; tr.y[0] = pos.y; tr.z[0] = pos.z;
    if (fr.displacement) {
        const float k[3] = {5.0f, 7.0f, 11.0f};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            pos.x = ffma(mp_sinf(fmul(fmul(pos.y, k[i]), 2.0f)), fr.fdisp[i], pos.x);
            pos.y = ffma(mp_sinf(fmul(fmul(pos.x, k[i]), 2.0f)), fr.fdisp[i], pos.y);
            pos.z = ffma(fmul(mp_sinf(fmul(fmul(pos.y, k[i]), 2.0f)), mp_sinf(fmul(fmul(pos.x, 3.0f), 2.0f))),
                         fr.fdisp[i], pos.z);
            tr.x[i + 1] = pos.x; tr.y[i + 1] = pos.y; tr.z[i + 1] = pos.z;
        }
    }
}

// 128-thread blocks, three per SM within the register file (about 160
// registers a thread): 12 warps per SM where 256-thread blocks fit only one
// block (8 warps).
constexpr int kAdjBlock = 128;

__global__ void __launch_bounds__(kAdjBlock, 3) adjoint_kernel(const DrawDev* __restrict__ draws, FrameDev frp,
                                                            SubPatches sub, Framebuffer fb,
                                                            const float4* __restrict__ grad_color, float* grad_amp,
                                                            int view) {
    FrameDev fr = frp;
    load_amplitude(fr);
    const int PS = fr.PS;
    const int lane = threadIdx.x & 31;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool active = false;
    int pid = -1, draw = -1, ncp = 16;
    float go_acc[4][3];
    float tx4[4], ty4[4];
    float gamp = 0.0f;
    const DrawDev* dp = nullptr;
    if (i < fb.pixels) {
        int px, py;
        fb_pixel(fr, i, px, py);
        unsigned long long key = fb.keys[(long long)view * fb.key_pixels + key_index(fr, px, py)];
        if (key != kClearKey) {
            unsigned id = (unsigned)(key & 0xffffffffu);
            unsigned s = id / (unsigned)(PS * PS), q = id % (unsigned)(PS * PS);
            int nu = (int)(q % PS), nv = (int)(q / PS);
            float4 r = sub.range[s];
            int2 m = sub.meta[s];
            dp = &draws[m.y];
            const DrawDev& d = *dp;
            if (d.grad_cp) {
                active = true;
                pid = m.x;
                draw = m.y;
                ncp = d.type == 0 ? 16 : 20;
                const float4* P = d.cp + (size_t)pid * ncp;
                float4 pos[4];
                VertexTrace tr[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    vertex_forward(d, fr, P, r, nu + (k & 1), nv + (k >> 1), pos[k], tr[k]);
                    tx4[k] = ffma(fsub(r.z, r.x), fdiv((float)(nu + (k & 1)), (float)PS), r.x);
                    ty4[k] = ffma(fsub(r.w, r.y), fdiv((float)(nv + (k >> 1)), (float)PS), r.y);
                }
                // shade forward
                V3 du{0.5f * (((pos[1].x - pos[0].x) + pos[3].x) - pos[2].x),
                      0.5f * (((pos[1].y - pos[0].y) + pos[3].y) - pos[2].y),
                      0.5f * (((pos[1].z - pos[0].z) + pos[3].z) - pos[2].z)};
                V3 dv{0.5f * (((pos[2].x - pos[0].x) + pos[3].x) - pos[1].x),
                      0.5f * (((pos[2].y - pos[0].y) + pos[3].y) - pos[1].y),
                      0.5f * (((pos[2].z - pos[0].z) + pos[3].z) - pos[1].z)};
                V3 cr{dv.y * du.z - dv.z * du.y, dv.z * du.x - dv.x * du.z, dv.x * du.y - dv.y * du.x};
                float len = sqrtf(cr.x * cr.x + cr.y * cr.y + cr.z * cr.z);
                V3 n{cr.x / len, cr.y / len, cr.z / len};
                float ln = sqrtf(89.0f);
                V3 L{4.0f / ln, 3.0f / ln, 8.0f / ln};
                float nl = n.x * L.x + n.y * L.y + n.z * L.z;
                float4 gc = grad_color[(long long)view * fb.pixels + i];
                float gm = gc.x * d.color[0] + gc.y * d.color[1] + gc.z * d.color[2] + gc.w * d.color[3];
#pragma unroll
                for (int k = 0; k < 4; ++k) go_acc[k][0] = go_acc[k][1] = go_acc[k][2] = 0.0f;
                if (nl > 0.0f && len > 0.0f && isfinite(len)) {
                    V3 gcr{gm * (L.x - n.x * nl) / len, gm * (L.y - n.y * nl) / len, gm * (L.z - n.z * nl) / len};
                    V3 gdv{du.y * gcr.z - du.z * gcr.y, du.z * gcr.x - du.x * gcr.z, du.x * gcr.y - du.y * gcr.x};
                    V3 gdu{gcr.y * dv.z - gcr.z * dv.y, gcr.z * dv.x - gcr.x * dv.z, gcr.x * dv.y - gcr.y * dv.x};
                    const float sdu[4] = {-0.5f, 0.5f, -0.5f, 0.5f}, sdv[4] = {-0.5f, -0.5f, 0.5f, 0.5f};
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        float gx = sdu[k] * gdu.x + sdv[k] * gdv.x;
                        float gy = sdu[k] * gdu.y + sdv[k] * gdv.y;
                        float gz = sdu[k] * gdu.z + sdv[k] * gdv.z;
                        if (fr.displacement) {
                            const float K[3] = {10.0f, 14.0f, 22.0f};
                            const float B[3] = {0.04f, 0.02f, 0.01f};
#pragma unroll
                            for (int st = 2; st >= 0; --st) {
                                float F = fr.fdisp[st];
                                float y0 = tr[k].y[st];
                                float x1 = tr[k].x[st + 1], y1 = tr[k].y[st + 1];
                                float sy1 = mp_sinf(K[st] * y1), s6 = mp_sinf(6.0f * x1);
                                gamp += gz * sy1 * s6 * B[st];
                                gy += gz * F * K[st] * mp_cosf(K[st] * y1) * s6;
                                gx += gz * F * sy1 * 6.0f * mp_cosf(6.0f * x1);
                                gamp += gy * mp_sinf(K[st] * x1) * B[st];
                                gx += gy * F * K[st] * mp_cosf(K[st] * x1);
                                gamp += gx * mp_sinf(K[st] * y0) * B[st];
                                gy += gx * F * K[st] * mp_cosf(K[st] * y0);
                            }
                        }
                        const float* mm = d.mv;
                        go_acc[k][0] = mm[0] * gx + mm[1] * gy + mm[2] * gz;
                        go_acc[k][1] = mm[4] * gx + mm[5] * gy + mm[6] * gz;
                        go_acc[k][2] = mm[8] * gx + mm[9] * gy + mm[10] * gz;
                    }
                }
            }
        }
    }
    // amplitude gradient: one atomic per warp
    float ga = __shfl_xor_sync(0xffffffffu, gamp, 16) + gamp;
    ga += __shfl_xor_sync(0xffffffffu, ga, 8);
    ga += __shfl_xor_sync(0xffffffffu, ga, 4);
    ga += __shfl_xor_sync(0xffffffffu, ga, 2);
    ga += __shfl_xor_sync(0xffffffffu, ga, 1);
    if (lane == 0 && grad_amp && ga != 0.0f) atomicAdd(grad_amp, ga);

    // control-point gradients: sum_k w_j(vertex k) * go(vertex k)
    long long key = active ? ((long long)draw << 32) | (unsigned)pid : -1;
    unsigned peers = __match_any_sync(0xffffffffu, key);
    bool uniform = __all_sync(0xffffffffu, peers == 0xffffffffu) && key != -1;
    float wv[4][20];
    int nw = ncp;
    if (active) {
#pragma unroll
        for (int k = 0; k < 4; ++k) nw = cp_weights(dp->type, tx4[k], ty4[k], wv[k]);
    }
    if (uniform) {
        // every lane holds the same patch: reduce each coordinate across the warp
        float* g = dp->grad_cp + (size_t)pid * nw * 3;
        for (int j = 0; j < nw; ++j)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float v = wv[0][j] * go_acc[0][c] + wv[1][j] * go_acc[1][c] + wv[2][j] * go_acc[2][c] +
                          wv[3][j] * go_acc[3][c];
                v += __shfl_xor_sync(0xffffffffu, v, 16);
                v += __shfl_xor_sync(0xffffffffu, v, 8);
                v += __shfl_xor_sync(0xffffffffu, v, 4);
                v += __shfl_xor_sync(0xffffffffu, v, 2);
                v += __shfl_xor_sync(0xffffffffu, v, 1);
                if (lane == 0 && v != 0.0f) atomicAdd(g + 3 * j + c, v);
            }
    } else if (active) {
        float* g = dp->grad_cp + (size_t)pid * nw * 3;
        for (int j = 0; j < nw; ++j)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float v = wv[0][j] * go_acc[0][c] + wv[1][j] * go_acc[1][c] + wv[2][j] * go_acc[2][c] +
                          wv[3][j] * go_acc[3][c];
                if (v != 0.0f) atomicAdd(g + 3 * j + c, v);
            }
    }
}

}  // namespace

void launch_adjoint(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, const Framebuffer& fb,
                    const float4* grad_color, float* grad_amp, int view, cudaStream_t s) {
    long long n = fb.pixels;
    adjoint_kernel<<<(unsigned)((n + kAdjBlock - 1) / kAdjBlock), kAdjBlock, 0, s>>>(draws, fr, sub, fb, grad_color,
                                                                                    grad_amp, view);
}

}  // namespace mp
