// Dice, shade and rasterize kernels.
//
// Batched path: raster_fused dices each sub-patch into shared memory (one
// warp per sub-patch, control points staged once per warp), applies the
// reference's per-8x8-block rules (a block with a vertex at eye z == 0 is
// dropped, kernels/reyes.cl:130-162; the block bound over front-facing quads
// and its is_empty test of kernels/reyes.cl:287) and rasterizes every quad
// with the integer edge functions of kernels/reyes.cl:240-265.  Visibility is
// one 64-bit atomicMin of (idepth << 32 | micropolygon id) per covered
// pixel, so the nearest fragment wins exactly and ties go to the smaller id.
// No grid is stored: resolve recomputes the winning quad's colour from its id.
//
// Quads whose pixel bbox is small (<= 1024 fixed-point units) and whose
// coordinates are within +-2^19 are rasterized over their own bbox: there the
// wrapped int32 edge functions equal the exact ones, so no pixel outside the
// bbox can pass and the bbox holds every pixel the reference's tile loop
// would accept.  Any other quad goes to raster_big, which replays the
// reference's per-tile candidate loop (kernels/reyes.cl:333-381) exactly.
//
// Plain path: dice_grid / shade_grid / sample_grid keep the reference's
// per-pass structure (kernels/dice.cl, kernels/reyes.cl shade and sample)
// with position, pixel, depth and colour grids in HBM; pass_resolve takes a
// winning fragment's colour from this pass's colour grid.
#include "mp_internal.h"

namespace mp {

namespace {

__device__ __forceinline__ unsigned long long* cw(unsigned long long* ctrl, int w) { return ctrl + w * kCtrlStride; }

constexpr int kFastCoord = 1 << 19;
constexpr int kFastExtent = 1024;

// Block bound of kernels/reyes.cl:97-166 for one quad: pmin/pmax start at
// the viewport max/min, is_front_facing on the wrapped integer coordinates.
struct QuadBound {
    int pminx, pminy, pmaxx, pmaxy;
    bool ff;
};
__device__ __forceinline__ QuadBound quad_block_bound(const FrameDev& fr, const int* qx, const int* qy) {
    const int vmaxx = (fr.W << fr.shift) - 1, vmaxy = (fr.H << fr.shift) - 1;
    QuadBound b{vmaxx, vmaxy, 0, 0, true};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        b.pminx = min(b.pminx, qx[k]);
        b.pminy = min(b.pminy, qy[k]);
        b.pmaxx = max(b.pmaxx, qx[k]);
        b.pmaxy = max(b.pmaxy, qy[k]);
    }
    if (fr.backface) {
        int d1x = wsub(qx[1], qx[0]), d1y = wsub(qy[1], qy[0]);
        int d2x = wsub(qx[2], qx[0]), d2y = wsub(qy[2], qy[0]);
        int d3x = wsub(qx[3], qx[0]), d3y = wsub(qy[3], qy[0]);
        b.ff = wsub(wmul(d1x, d3y), wmul(d3x, d1y)) < 0 || wsub(wmul(d3x, d2y), wmul(d2x, d3y)) < 0;
    }
    return b;
}

// Final block bound (clamp, allnormal) -> tile range; returns false when the
// block is skipped by the is_empty(block_bound.xy, block_bound.zx) test.
__device__ __forceinline__ bool block_tiles(const FrameDev& fr, int xmin, int ymin, int xmax, int ymax,
                                            bool allnormal, int* tiles) {
    const int vmaxx = (fr.W << fr.shift) - 1, vmaxy = (fr.H << fr.shift) - 1;
    xmin = max(0, xmin);
    ymin = max(0, ymin);
    xmax = min(vmaxx, xmax);
    ymax = min(vmaxy, ymax);
    if (!allnormal) { xmin = 1; ymin = 1; xmax = -1; ymax = -1; }
    if (xmin >= xmax && ymin >= xmin) return false;
    tiles[0] = xmin >> (fr.shift + 3);
    tiles[1] = ymin >> (fr.shift + 3);
    tiles[2] = xmax >> (fr.shift + 3);
    tiles[3] = ymax >> (fr.shift + 3);
    return true;
}

__device__ __forceinline__ bool quad_is_fast(const int* qx, const int* qy, int& minx, int& miny, int& maxx,
                                             int& maxy) {
    minx = min(min(qx[0], qx[1]), min(qx[2], qx[3]));
    maxx = max(max(qx[0], qx[1]), max(qx[2], qx[3]));
    miny = min(min(qy[0], qy[1]), min(qy[2], qy[3]));
    maxy = max(max(qy[0], qy[1]), max(qy[2], qy[3]));
    if (minx < -kFastCoord || maxx > kFastCoord || miny < -kFastCoord || maxy > kFastCoord) return false;
    return (maxx - minx) <= kFastExtent && (maxy - miny) <= kFastExtent;
}

// Fast path: rasterize one quad over its own pixel bbox (see file header).
__device__ __forceinline__ int raster_quad_fast(const FrameDev& fr, unsigned long long* keys, const int* qx,
                                                const int* qy, const float* qd, int minx, int miny, int maxx,
                                                int maxy, unsigned mp_id) {
    // a quad whose two triangles both have the rejected winding covers nothing
    int d1x = qx[1] - qx[0], d1y = qy[1] - qy[0];
    int d2x = qx[2] - qx[0], d2y = qy[2] - qy[0];
    int d3x = qx[3] - qx[0], d3y = qy[3] - qy[0];
    if (!(d1x * d3y - d3x * d1y < 0 || d3x * d2y - d2x * d3y < 0)) return 0;
    const int one = (1 << fr.shift) - 1;
    int x0 = max((minx + one) >> fr.shift, 0), x1 = min(maxx >> fr.shift, fr.W - 1);
    int y0 = max((miny + one) >> fr.shift, 0), y1 = min(maxy >> fr.shift, fr.H - 1);
    if (x0 > x1 || y0 > y1) return 0;
    Tri t1, t2;
    tri_setup(t1, qx[0], qy[0], qd[0], qx[1], qy[1], qd[1], qx[3], qy[3], qd[3]);
    tri_setup(t2, qx[0], qy[0], qd[0], qx[3], qy[3], qd[3], qx[2], qy[2], qd[2]);
    int frags = 0;
    for (int y = y0; y <= y1; ++y)
        for (int x = x0; x <= x1; ++x) {
            int tx = x << fr.shift, ty = y << fr.shift;
            float depth = 1.0f;
            bool in1 = tri_test(t1, tx, ty, depth);
            bool in2 = tri_test(t2, tx, ty, depth);
            if (in1 || in2) {
                unsigned long long key = ((unsigned long long)idepth_of(depth) << 32) | mp_id;
                atomicMin(keys + fb_index(fr, x, y), key);
                ++frags;
            }
        }
    return frags;
}

__device__ __forceinline__ void push_big(BigQuad* big, long long big_cap, unsigned long long* ctrl, const int* qx,
                                         const int* qy, const float* qd, unsigned mp_id, int view,
                                         const int* tiles) {
    unsigned long long i = atomicAdd(cw(ctrl, kBigCount), 1ull);
    if ((long long)i >= big_cap) {
        atomicAdd(cw(ctrl, kBigOverflow), 1ull);
        atomicCAS(cw(ctrl, kStatus), 0ull, (unsigned long long)kErrOverflow);
        return;
    }
    BigQuad b;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        b.px[k] = qx[k];
        b.py[k] = qy[k];
        b.depth[k] = qd[k];
        b.tile[k] = tiles[k];
    }
    b.mp_id = mp_id;
    b.view = view;
    big[i] = b;
}

constexpr int kRasterWarps = 8;

template <int PS>
struct RasterSmem {
    float4 cp[kRasterWarps][20];
    int2 pxl[kRasterWarps][(PS + 1) * (PS + 1)];
    float dep[kRasterWarps][(PS + 1) * (PS + 1)];
};

template <int PS>
__global__ void __launch_bounds__(kRasterWarps * 32) raster_fused_kernel(const DrawDev* __restrict__ draws,
                                                                        FrameDev fr, SubPatches sub,
                                                                        Framebuffer fb, BigQuad* big,
                                                                        long long big_cap,
                                                                        unsigned long long* ctrl) {
    constexpr int G = PS + 1, NV = G * G, NQ = PS * PS, BPL = PS / 8, NB = BPL * BPL;
    __shared__ RasterSmem<PS> sm;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long S = (long long)*(volatile unsigned long long*)cw(ctrl, kOutCount);
    if (S > sub.capacity) S = sub.capacity;
    long long frags = 0;
    const long long nwarps = (long long)gridDim.x * kRasterWarps;
    for (long long s = (long long)blockIdx.x * kRasterWarps + warp; s < S; s += nwarps) {
        const float4 r = sub.range[s];
        const int2 m = sub.meta[s];
        const DrawDev& d = draws[m.y];
        const int ncp = d.type == 0 ? 16 : 20;
        if (lane < ncp) sm.cp[warp][lane] = __ldg(d.cp + (size_t)m.x * ncp + lane);
        __syncwarp();
        unsigned zblocks = 0;
        for (int v = lane; v < NV; v += 32) {
            int nu = v % G, nv = v / G;
            float4 pos = dice_eye(d, fr, sm.cp[warp], r, nu, nv);
            int px, py;
            float dep;
            project_vertex(d, fr, pos, px, py, dep);
            sm.pxl[warp][v] = make_int2(px, py);
            sm.dep[warp][v] = dep;
            if (pos.z == 0.0f) {
                // the vertex belongs to the quads (nu-1..nu, nv-1..nv)
                for (int bv = max(nv - 1, 0) / 8; bv <= min(nv, PS - 1) / 8; ++bv)
                    for (int bu = max(nu - 1, 0) / 8; bu <= min(nu, PS - 1) / 8; ++bu) zblocks |= 1u << (bu + bv * BPL);
            }
        }
        zblocks = __reduce_or_sync(0xffffffffu, zblocks);
        __syncwarp();
        // block bounds over front-facing quads (kernels/reyes.cl:120-166)
        int bxmin[NB], bymin[NB], bxmax[NB], bymax[NB];
        const int vmaxx = (fr.W << fr.shift) - 1, vmaxy = (fr.H << fr.shift) - 1;
#pragma unroll
        for (int b = 0; b < NB; ++b) { bxmin[b] = vmaxx; bymin[b] = vmaxy; bxmax[b] = 0; bymax[b] = 0; }
        for (int q = lane; q < NQ; q += 32) {
            int nu = q % PS, nv = q / PS, i0 = nu + nv * G;
            int qx[4], qy[4];
            int2 a = sm.pxl[warp][i0], b1 = sm.pxl[warp][i0 + 1], c = sm.pxl[warp][i0 + G], e = sm.pxl[warp][i0 + G + 1];
            qx[0] = a.x; qy[0] = a.y; qx[1] = b1.x; qy[1] = b1.y; qx[2] = c.x; qy[2] = c.y; qx[3] = e.x; qy[3] = e.y;
            QuadBound qb = quad_block_bound(fr, qx, qy);
            if (qb.ff) {
                int blk = (nu >> 3) + (nv >> 3) * BPL;
#pragma unroll
                for (int b = 0; b < NB; ++b)
                    if (b == blk) {
                        bxmin[b] = min(bxmin[b], qb.pminx);
                        bymin[b] = min(bymin[b], qb.pminy);
                        bxmax[b] = max(bxmax[b], qb.pmaxx);
                        bymax[b] = max(bymax[b], qb.pmaxy);
                    }
            }
        }
        int tiles[NB][4];
        unsigned live = 0;
#pragma unroll
        for (int b = 0; b < NB; ++b) {
            int x0 = __reduce_min_sync(0xffffffffu, bxmin[b]);
            int y0 = __reduce_min_sync(0xffffffffu, bymin[b]);
            int x1 = __reduce_max_sync(0xffffffffu, bxmax[b]);
            int y1 = __reduce_max_sync(0xffffffffu, bymax[b]);
            if (block_tiles(fr, x0, y0, x1, y1, !((zblocks >> b) & 1), tiles[b])) live |= 1u << b;
        }
        if (live) {
            unsigned long long* keys = fb.keys + (long long)d.view * fb.pixels;
            for (int q = lane; q < NQ; q += 32) {
                int nu = q % PS, nv = q / PS, blk = (nu >> 3) + (nv >> 3) * BPL;
                if (!((live >> blk) & 1)) continue;
                int i0 = nu + nv * G;
                const int idx[4] = {i0, i0 + 1, i0 + G, i0 + G + 1};
                int qx[4], qy[4];
                float qd[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    int2 p = sm.pxl[warp][idx[k]];
                    qx[k] = p.x;
                    qy[k] = p.y;
                    qd[k] = sm.dep[warp][idx[k]];
                }
                unsigned mp_id = (unsigned)(s * NQ + nu + nv * PS);
                int minx, miny, maxx, maxy;
                if (quad_is_fast(qx, qy, minx, miny, maxx, maxy)) {
                    frags += raster_quad_fast(fr, keys, qx, qy, qd, minx, miny, maxx, maxy, mp_id);
                } else {
                    int t4[4];
#pragma unroll
                    for (int b = 0; b < NB; ++b)
                        if (b == blk) { t4[0] = tiles[b][0]; t4[1] = tiles[b][1]; t4[2] = tiles[b][2]; t4[3] = tiles[b][3]; }
                    push_big(big, big_cap, ctrl, qx, qy, qd, mp_id, d.view, t4);
                }
            }
        }
        __syncwarp();
    }
    frags = __reduce_add_sync(0xffffffffu, (unsigned)frags);
    if (lane == 0 && frags) atomicAdd(cw(ctrl, kFragments), (unsigned long long)frags);
}

// Exact replay of the reference's per-tile candidate loop for one quad
// (kernels/reyes.cl:333-381): the candidate set is the product of the x and y
// candidates of every tile in the block's tile range, each clamped to
// [0, 8 << shift) after subtracting the tile origin.
constexpr int kBigThreads = 256;
constexpr int kBigMaxAxis = 4096;

__global__ void __launch_bounds__(kBigThreads) raster_big_kernel(FrameDev fr, Framebuffer fb,
                                                                 const BigQuad* __restrict__ big,
                                                                 long long big_cap, unsigned long long* ctrl) {
    __shared__ short s_x[kBigMaxAxis], s_y[kBigMaxAxis];
    __shared__ int s_nx, s_ny;
    __shared__ int s_frags;
    long long n = (long long)*(volatile unsigned long long*)cw(ctrl, kBigCount);
    if (n > big_cap) n = big_cap;
    const int maxl = (8 << fr.shift) - 1;
    for (long long bi = blockIdx.x; bi < n; bi += gridDim.x) {
        const BigQuad b = big[bi];
        if (threadIdx.x == 0) {
            const int vmaxx = (fr.W << fr.shift) - 1, vmaxy = (fr.H << fr.shift) - 1;
            int mingx = vmaxx + 1, mingy = vmaxy + 1, maxgx = -1, maxgy = -1;
            for (int k = 0; k < 4; ++k) {
                mingx = min(mingx, b.px[k]);
                mingy = min(mingy, b.py[k]);
                maxgx = max(maxgx, b.px[k]);
                maxgy = max(maxgy, b.py[k]);
            }
            int nx = 0, ny = 0;
            for (int tx = b.tile[0]; tx <= b.tile[2]; ++tx) {
                int os = (tx * 8) << fr.shift;
                int lo = min(max(wsub(mingx, os), 0), maxl) >> fr.shift;
                int hi = min(max(wsub(maxgx, os), 0), maxl) >> fr.shift;
                for (int x = lo; x <= hi && nx < kBigMaxAxis; ++x) s_x[nx++] = (short)(tx * 8 + x);
            }
            for (int ty = b.tile[1]; ty <= b.tile[3]; ++ty) {
                int os = (ty * 8) << fr.shift;
                int lo = min(max(wsub(mingy, os), 0), maxl) >> fr.shift;
                int hi = min(max(wsub(maxgy, os), 0), maxl) >> fr.shift;
                for (int y = lo; y <= hi && ny < kBigMaxAxis; ++y) s_y[ny++] = (short)(ty * 8 + y);
            }
            s_nx = nx;
            s_ny = ny;
            s_frags = 0;
        }
        __syncthreads();
        Tri t1, t2;
        tri_setup(t1, b.px[0], b.py[0], b.depth[0], b.px[1], b.py[1], b.depth[1], b.px[3], b.py[3], b.depth[3]);
        tri_setup(t2, b.px[0], b.py[0], b.depth[0], b.px[3], b.py[3], b.depth[3], b.px[2], b.py[2], b.depth[2]);
        unsigned long long* keys = fb.keys + (long long)b.view * fb.pixels;
        long long total = (long long)s_nx * s_ny;
        int frags = 0;
        for (long long c = threadIdx.x; c < total; c += kBigThreads) {
            int x = s_x[c % s_nx], y = s_y[c / s_nx];
            int tx = wadd(x << fr.shift, 0), ty = y << fr.shift;
            float depth = 1.0f;
            bool in1 = tri_test(t1, tx, ty, depth);
            bool in2 = tri_test(t2, tx, ty, depth);
            if (in1 || in2) {
                unsigned long long key = ((unsigned long long)idepth_of(depth) << 32) | b.mp_id;
                atomicMin(keys + fb_index(fr, x, y), key);
                ++frags;
            }
        }
        atomicAdd(&s_frags, frags);
        __syncthreads();
        if (threadIdx.x == 0 && s_frags) atomicAdd(cw(ctrl, kFragments), (unsigned long long)s_frags);
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && n > 0) atomicAdd(cw(ctrl, kBigTotal), (unsigned long long)n);
}

__global__ void clear_kernel(Framebuffer fb, FrameDev fr, int with_color) {
    long long n = fb.pixels * fb.views;
    float4 cc = make_float4(fr.clear[0], fr.clear[1], fr.clear[2], fr.clear[3]);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        fb.keys[i] = kClearKey;
        if (with_color) {
            fb.color[i] = cc;
            fb.depth[i] = 0x7fffffff;
        }
    }
}

// Colour of micropolygon `id` recomputed from its sub-patch record.
template <int PS>
__device__ __forceinline__ float4 mp_color(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub,
                                           unsigned id) {
    const unsigned s = id / (PS * PS), q = id % (PS * PS);
    const int nu = (int)(q % PS), nv = (int)(q / PS);
    const float4 r = sub.range[s];
    const int2 m = sub.meta[s];
    const DrawDev& d = draws[m.y];
    const float4* P = d.cp + (size_t)m.x * (d.type == 0 ? 16 : 20);
    float4 pos[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) pos[k] = dice_eye(d, fr, P, r, nu + (k & 1), nv + (k >> 1));
    return shade_quad(pos, d.color);
}

template <int PS>
__global__ void resolve_kernel(const DrawDev* __restrict__ draws, FrameDev fr, SubPatches sub, Framebuffer fb) {
    long long n = fb.pixels * fb.views;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long key = fb.keys[i];
        if (key == kClearKey) {
            fb.color[i] = make_float4(fr.clear[0], fr.clear[1], fr.clear[2], fr.clear[3]);
            fb.depth[i] = 0x7fffffff;
        } else {
            fb.color[i] = mp_color<PS>(draws, fr, sub, (unsigned)(key & 0xffffffffu));
            fb.depth[i] = (int)(key >> 32);
        }
    }
}

// ---------------------------------------------------------------------------
// Plain per-pass kernels

template <int PS>
__global__ void dice_grid_kernel(const DrawDev* __restrict__ draws, FrameDev fr, SubPatches sub, long long base,
                                 int count, float4* pos_grid, int2* pxl_grid, float* depth_grid) {
    constexpr int G = PS + 1, NV = G * G;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)count * NV) return;
    int s = (int)(i / NV), v = (int)(i % NV);
    int nu = v % G, nv = v / G;
    const float4 r = sub.range[base + s];
    const int2 m = sub.meta[base + s];
    const DrawDev& d = draws[m.y];
    const float4* P = d.cp + (size_t)m.x * (d.type == 0 ? 16 : 20);
    float4 pos = dice_eye(d, fr, P, r, nu, nv);
    int px, py;
    float dep;
    project_vertex(d, fr, pos, px, py, dep);
    // grid index nu + nv*(PS+1) + range*(PS+1)^2 (kernels/dice.cl:21-24)
    pos_grid[i] = pos;
    pxl_grid[i] = make_int2(px, py);
    depth_grid[i] = dep;
}

// One 8x8 thread block per 8x8 quad block (kernels/reyes.cl:84-199).
template <int PS>
__global__ void __launch_bounds__(64) shade_grid_kernel(const DrawDev* __restrict__ draws, FrameDev fr,
                                                        SubPatches sub, long long base, const float4* pos_grid,
                                                        const int2* pxl_grid, int4* block_index,
                                                        float4* color_grid) {
    constexpr int G = PS + 1, BPL = PS / 8, BPP = BPL * BPL;
    __shared__ int s_b[4];
    __shared__ int s_allnormal;
    const int s = blockIdx.x / BPP, blk = blockIdx.x % BPP;
    const int lx = threadIdx.x & 7, ly = threadIdx.x >> 3;
    const int nu = (blk % BPL) * 8 + lx, nv = (blk / BPL) * 8 + ly;
    const int vmaxx = (fr.W << fr.shift) - 1, vmaxy = (fr.H << fr.shift) - 1;
    if (threadIdx.x == 0) {
        s_b[0] = vmaxx; s_b[1] = vmaxy; s_b[2] = 0; s_b[3] = 0;
        s_allnormal = 1;
    }
    __syncthreads();
    float4 pos[4];
    int qx[4], qy[4];
    const long long g0 = (long long)s * G * G;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        long long gi = g0 + (nu + (k & 1)) + (nv + (k >> 1)) * G;
        pos[k] = pos_grid[gi];
        int2 p = pxl_grid[gi];
        qx[k] = p.x;
        qy[k] = p.y;
        if (pos[k].z == 0.0f) s_allnormal = 0;
    }
    QuadBound qb = quad_block_bound(fr, qx, qy);
    if (qb.ff) {
        atomicMin(&s_b[0], qb.pminx);
        atomicMin(&s_b[1], qb.pminy);
        atomicMax(&s_b[2], qb.pmaxx);
        atomicMax(&s_b[3], qb.pmaxy);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int xmin = max(0, s_b[0]), ymin = max(0, s_b[1]), xmax = min(vmaxx, s_b[2]), ymax = min(vmaxy, s_b[3]);
        if (!s_allnormal) { xmin = 1; ymin = 1; xmax = -1; ymax = -1; }
        block_index[(long long)s * BPP + blk] = make_int4(xmin, ymin, xmax, ymax);
    }
    const DrawDev& d = draws[sub.meta[base + s].y];
    color_grid[(long long)s * PS * PS + nu + nv * PS] = shade_quad(pos, d.color);
}

// One thread per quad; the block bound decides the tile range (kernels/reyes.cl:270-398).
template <int PS>
__global__ void sample_grid_kernel(const DrawDev* __restrict__ draws, FrameDev fr, SubPatches sub, long long base,
                                   int count, const int4* block_index, const int2* pxl_grid,
                                   const float* depth_grid, Framebuffer fb, BigQuad* big, long long big_cap,
                                   unsigned long long* ctrl) {
    constexpr int G = PS + 1, BPL = PS / 8, BPP = BPL * BPL;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int frags = 0;
    if (i < (long long)count * PS * PS) {
        int s = (int)(i / (PS * PS)), q = (int)(i % (PS * PS));
        int nu = q % PS, nv = q / PS;
        int blk = (nu >> 3) + (nv >> 3) * BPL;
        int4 bb = block_index[(long long)s * BPP + blk];
        if (!(bb.x >= bb.z && bb.y >= bb.x)) {
            int tiles[4] = {bb.x >> (fr.shift + 3), bb.y >> (fr.shift + 3), bb.z >> (fr.shift + 3),
                            bb.w >> (fr.shift + 3)};
            long long g0 = (long long)s * G * G + nu + nv * G;
            const long long idx[4] = {g0, g0 + 1, g0 + G, g0 + G + 1};
            int qx[4], qy[4];
            float qd[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                int2 p = pxl_grid[idx[k]];
                qx[k] = p.x;
                qy[k] = p.y;
                qd[k] = depth_grid[idx[k]];
            }
            const int view = draws[sub.meta[base + s].y].view;
            unsigned long long* keys = fb.keys + (long long)view * fb.pixels;
            unsigned mp_id = (unsigned)((base + s) * PS * PS + nu + nv * PS);
            int minx, miny, maxx, maxy;
            if (quad_is_fast(qx, qy, minx, miny, maxx, maxy))
                frags = raster_quad_fast(fr, keys, qx, qy, qd, minx, miny, maxx, maxy, mp_id);
            else
                push_big(big, big_cap, ctrl, qx, qy, qd, mp_id, view, tiles);
        }
    }
    frags = __reduce_add_sync(0xffffffffu, (unsigned)frags);
    if ((threadIdx.x & 31) == 0 && frags) atomicAdd(cw(ctrl, kFragments), (unsigned long long)frags);
}

// Pixels won by a micropolygon of this pass take its colour from the colour grid.
__global__ void pass_resolve_kernel(FrameDev fr, Framebuffer fb, unsigned long long id_lo, unsigned long long id_hi,
                                    const float4* color_grid) {
    long long n = fb.pixels * fb.views;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        unsigned long long key = fb.keys[i];
        unsigned long long id = key & 0xffffffffull;
        if (key != kClearKey && id >= id_lo && id < id_hi) {
            fb.color[i] = color_grid[id - id_lo];
            fb.depth[i] = (int)(key >> 32);
        }
    }
}

// 64-bit atomicMin throughput probe: pattern 0 = uniform random slots,
// pattern 1 = each warp updates one 8x8-pixel tile (micropolygon-like locality).
__global__ void atomic_bench_kernel(unsigned long long* buf, long long n_slots, long long n_ops, int pattern) {
    long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    unsigned long long x = 0x9E3779B97F4A7C15ull * (unsigned long long)(tid + 1);
    for (long long i = tid; i < n_ops; i += stride) {
        x ^= x << 13; x ^= x >> 7; x ^= x << 17;
        long long slot;
        if (pattern == 0) {
            slot = (long long)(x % (unsigned long long)n_slots);
        } else {
            long long tile = (long long)((i >> 5) * 2654435761ull % (unsigned long long)(n_slots >> 6));
            slot = (tile << 6) + (long long)((i & 31) + (x & 31)) % 64;
        }
        atomicMin(buf + slot, x >> 1);
    }
}

template <int PS>
int fused_grid_impl() {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, raster_fused_kernel<PS>, kRasterWarps * 32, 0);
    if (per_sm < 1) per_sm = 1;
    return sms * per_sm;
}

int grid_for(long long n, int block) {
    long long g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 1 << 20) g = 1 << 20;
    return (int)g;
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers

void launch_clear(const Framebuffer& fb, const FrameDev& fr, int with_color, cudaStream_t s) {
    clear_kernel<<<grid_for(fb.pixels * fb.views, 256), 256, 0, s>>>(fb, fr, with_color);
}

int raster_fused_grid(int PS) { return PS == 16 ? fused_grid_impl<16>() : fused_grid_impl<8>(); }

void launch_raster_fused(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, const Framebuffer& fb,
                         BigQuad* big, long long big_cap, unsigned long long* ctrl, int grid, cudaStream_t s) {
    if (fr.PS == 16)
        raster_fused_kernel<16><<<grid, kRasterWarps * 32, 0, s>>>(draws, fr, sub, fb, big, big_cap, ctrl);
    else
        raster_fused_kernel<8><<<grid, kRasterWarps * 32, 0, s>>>(draws, fr, sub, fb, big, big_cap, ctrl);
}

void launch_raster_big(const DrawDev*, const FrameDev& fr, const Framebuffer& fb, const BigQuad* big,
                       long long big_cap, unsigned long long* ctrl, cudaStream_t s) {
    raster_big_kernel<<<256, kBigThreads, 0, s>>>(fr, fb, big, big_cap, ctrl);
}

void launch_resolve(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, const Framebuffer& fb,
                    cudaStream_t s) {
    int g = grid_for(fb.pixels * fb.views, 256);
    if (fr.PS == 16)
        resolve_kernel<16><<<g, 256, 0, s>>>(draws, fr, sub, fb);
    else
        resolve_kernel<8><<<g, 256, 0, s>>>(draws, fr, sub, fb);
}

void launch_dice_grid(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, long long base, int count,
                      float4* pos, int2* pxl, float* depth, cudaStream_t s) {
    if (count <= 0) return;
    long long n = (long long)count * (fr.PS + 1) * (fr.PS + 1);
    if (fr.PS == 16)
        dice_grid_kernel<16><<<grid_for(n, 128), 128, 0, s>>>(draws, fr, sub, base, count, pos, pxl, depth);
    else
        dice_grid_kernel<8><<<grid_for(n, 128), 128, 0, s>>>(draws, fr, sub, base, count, pos, pxl, depth);
}

void launch_shade_grid(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, long long base, int count,
                       const float4* pos, const int2* pxl, int4* block_index, float4* color, cudaStream_t s) {
    if (count <= 0) return;
    int bpp = (fr.PS / 8) * (fr.PS / 8);
    if (fr.PS == 16)
        shade_grid_kernel<16><<<count * bpp, 64, 0, s>>>(draws, fr, sub, base, pos, pxl, block_index, color);
    else
        shade_grid_kernel<8><<<count * bpp, 64, 0, s>>>(draws, fr, sub, base, pos, pxl, block_index, color);
}

void launch_sample_grid(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, long long base, int count,
                        const int4* block_index, const int2* pxl, const float* depth, const Framebuffer& fb,
                        BigQuad* big, long long big_cap, unsigned long long* ctrl, cudaStream_t s) {
    if (count <= 0) return;
    long long n = (long long)count * fr.PS * fr.PS;
    if (fr.PS == 16)
        sample_grid_kernel<16><<<grid_for(n, 128), 128, 0, s>>>(draws, fr, sub, base, count, block_index, pxl, depth,
                                                                fb, big, big_cap, ctrl);
    else
        sample_grid_kernel<8><<<grid_for(n, 128), 128, 0, s>>>(draws, fr, sub, base, count, block_index, pxl, depth,
                                                               fb, big, big_cap, ctrl);
}

void launch_pass_resolve(const FrameDev& fr, const Framebuffer& fb, long long base, int count, const float4* color,
                         cudaStream_t s) {
    if (count <= 0) return;
    unsigned long long lo = (unsigned long long)base * fr.PS * fr.PS;
    unsigned long long hi = lo + (unsigned long long)count * fr.PS * fr.PS;
    pass_resolve_kernel<<<grid_for(fb.pixels * fb.views, 256), 256, 0, s>>>(fr, fb, lo, hi, color);
}

void launch_dice_debug(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, int count, float4* pos,
                       int2* pxl, float* depth, cudaStream_t s) {
    launch_dice_grid(draws, fr, sub, 0, count, pos, pxl, depth, s);
}

void launch_atomic_bench(unsigned long long* buf, long long n_slots, long long n_ops, int pattern, cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    atomic_bench_kernel<<<sms * 8, 256, 0, s>>>(buf, n_slots, n_ops, pattern);
}

}  // namespace mp
