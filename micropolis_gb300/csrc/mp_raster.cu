// Dice, shade and rasterize kernels.
//
// Batched path: raster_fused dices groups of sub-patches into shared memory
// (a block per group, the group's control points and matrices staged with
// cp.async while the previous group is processed), applies the
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
#include "mp_bns_loop.cuh"

namespace mp {

namespace {

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

// A small quad whose two triangles both have the rejected winding covers
// nothing (small quads: the products below cannot overflow).
__device__ __forceinline__ bool quad_winding_ok(const int* qx, const int* qy) {
    int d1x = qx[1] - qx[0], d1y = qy[1] - qy[0];
    int d2x = qx[2] - qx[0], d2y = qy[2] - qy[0];
    int d3x = qx[3] - qx[0], d3y = qy[3] - qy[0];
    return d1x * d3y - d3x * d1y < 0 || d3x * d2y - d2x * d3y < 0;
}
// Pixels whose sample point lies in the fixed-point bbox, clipped to the
// frame; false when there are none.
__device__ __forceinline__ bool quad_pixels(const FrameDev& fr, int minx, int miny, int maxx, int maxy, int& x0,
                                            int& y0, int& x1, int& y1) {
    const int one = (1 << fr.shift) - 1;
    x0 = max((minx + one) >> fr.shift, 0);
    x1 = min(maxx >> fr.shift, fr.W - 1);
    y0 = max((miny + one) >> fr.shift, 0);
    y1 = min(maxy >> fr.shift, fr.H - 1);
    return x0 <= x1 && y0 <= y1;
}

// Fast path: rasterize one quad over its own pixel bbox (see file header).
__device__ __forceinline__ int raster_quad_fast(const FrameDev& fr, unsigned long long* keys, const int* qx,
                                                const int* qy, const float* qd, int minx, int miny, int maxx,
                                                int maxy, unsigned mp_id) {
    if (!quad_winding_ok(qx, qy)) return 0;
    int x0, y0, x1, y1;
    if (!quad_pixels(fr, minx, miny, maxx, maxy, x0, y0, x1, y1)) return 0;
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
                // the reference writes only depths below the cleared 0x7fffffff (kernels/reyes.cl:389)
                const unsigned idp = idepth_of(depth);
                if (idp < 0x7fffffffu) atomicMin(keys + key_index(fr, x, y), ((unsigned long long)idp << 32) | mp_id);
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

// The fused kernel works on groups of NS sub-patches per block:
// NS * (PS+1)^2 dice vertices are spread over all threads (22 * 81 = 1782 =
// 7 rounds of 256 at PS = 8), then the block bounds, then one thread per quad
// that can touch a pixel.  The inputs of the next group (sub-patch records,
// control points, matrices) are copied into the other half of a double
// buffer with cp.async while the current group is diced and rasterized.
// Groups of 11 (PS = 8) and 3 (PS = 16) run half-size blocks of 128 threads,
// twice as many per SM, the others 256.
template <int NS>
constexpr int fused_threads() {
    return (NS == 11 || NS == 3) ? 128 : 256;
}

static_assert(offsetof(DrawDev, proj) == offsetof(DrawDev, mv) + 16 * sizeof(float), "mv, proj adjacent");
static_assert(offsetof(DrawDev, mv) % 16 == 0 && sizeof(DrawDev) % 16 == 0, "16-byte copies of mv/proj");

// Inputs of one group.
template <int NS>
struct GroupStage {
    float4 cp[NS][20];
    float mvp[NS][32];        // modelview, then projection
    float4 range[NS];
    int2 meta[NS];            // (patch id, draw)
    int tv[NS][2];            // draw type, view
};

template <int PS, int NS_>
struct FusedSmem {
    static constexpr int NS = NS_, G = PS + 1, NV = G * G, NB = (PS / 8) * (PS / 8);
    GroupStage<NS> st[2];
    // per group state, double-buffered with st: block bounds, blocks with a
    // vertex at eye z == 0, and the number of listed quads
    int bound[2][NS][NB][4];
    unsigned zero[2][NS];
    unsigned n_live[2];
    unsigned short live[NS * PS * PS];   // quads that may touch a pixel, in bound-phase order
    float tx[NS][G], ty[NS][G];
    float4 vw[NS][G], cw[NS][G];
    float4 edep[NS * NV];     // eye position and NDC depth of each dice vertex
    int2 pxy[NS * NV];        // fixed-point pixel coordinates
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    const size_t ga = __cvta_generic_to_global(gmem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(ga) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    const size_t ga = __cvta_generic_to_global(gmem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(ga) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Copies, for the n sub-patches whose records are already in st.meta, their
// control points, matrices, type and view (asynchronous; the caller waits).
template <int NS>
__device__ __forceinline__ void stage_inputs(GroupStage<NS>& st, int n, const DrawDev* __restrict__ draws) {
    for (int i = threadIdx.x; i < n * 32; i += fused_threads<NS>()) {
        const int k = i >> 5, c = i & 31;
        const int2 m = st.meta[k];
        const DrawDev* d = draws + m.y;
        if (c < 20) {
            const int ncp = d->type == 0 ? 16 : 20;
            if (c < ncp) cp_async16(&st.cp[k][c], d->cp + (size_t)m.x * ncp + c);
        } else if (c < 28) {
            cp_async16(&st.mvp[k][4 * (c - 20)], d->mv + 4 * (c - 20));
        } else if (c == 28) {
            cp_async4(&st.tv[k][0], &d->type);
        } else if (c == 29) {
            cp_async4(&st.tv[k][1], &d->view);
        }
    }
    cp_async_commit();
}

// Prepares the state of a group of n sub-patches whose records are in
// sm.st[b]: the dice parameters and Bernstein weights of each row / column of
// vertices, reset block bounds (viewport max, 0), eye-plane flags and listed
// quad count.  This thread takes the items first, first + threads, ...
template <int PS, int NS>
__device__ __forceinline__ void prepare_group(FusedSmem<PS, NS>& sm, int b, int n, const FrameDev& fr, int first) {
    constexpr int G = PS + 1, NB = (PS / 8) * (PS / 8);
    const GroupStage<NS>& st = sm.st[b];
    for (int i = first; i < n * 2 * G; i += fused_threads<NS>()) {
        const int k = i / (2 * G), c = i % (2 * G);
        const float4 rg = st.range[k];
        if (c < G) {
            const float t = dice_param(rg.x, rg.z, c, fr);
            sm.tx[k][c] = t;
            sm.vw[k][c] = row_weights(t);
        } else {
            const float t = dice_param(rg.y, rg.w, c - G, fr);
            sm.ty[k][c - G] = t;
            sm.cw[k][c - G] = col_weights(t);
        }
    }
    const int vmaxx = (fr.W << fr.shift) - 1, vmaxy = (fr.H << fr.shift) - 1;
    for (int i = first; i < n * NB; i += fused_threads<NS>()) {
        int* bb = sm.bound[b][i / NB][i % NB];
        bb[0] = vmaxx; bb[1] = vmaxy; bb[2] = 0; bb[3] = 0;
    }
    if (first < n) sm.zero[b][first] = 0;
    if (first == 0) sm.n_live[b] = 0;
}

// Stages the group [base, base + n) into sm.st[0] from scratch (records,
// then inputs) and prepares it; ends with a barrier.
template <int PS, int NS>
__device__ __forceinline__ void stage_group(FusedSmem<PS, NS>& sm, long long base, int n, const SubPatches& sub,
                                            const DrawDev* __restrict__ draws, const FrameDev& fr) {
    GroupStage<NS>& st = sm.st[0];
    if ((int)threadIdx.x < n) {
        st.range[threadIdx.x] = sub.range[base + threadIdx.x];
        st.meta[threadIdx.x] = sub.meta[base + threadIdx.x];
    }
    __syncthreads();
    stage_inputs(st, n, draws);
    prepare_group(sm, 0, n, fr, threadIdx.x);
    cp_async_wait_all();
    __syncthreads();
}

// Dices, shades and rasterizes the n (<= NS) sub-patches at [base, base+n)
// of the emitted list, whose inputs are staged and prepared in buffer b, with
// the whole block; meanwhile stages and prepares the n_next sub-patches at
// next_base in buffer b ^ 1.  Three phases (dice; block bounds and the list
// of quads that can touch a pixel; raster), each ending with a barrier after
// which both groups' buffers are complete.
template <int PS, int NS>
__device__ __forceinline__ void raster_group(FusedSmem<PS, NS>& sm, int b, long long base, int n,
                                             long long next_base, int n_next, const DrawDev* __restrict__ draws,
                                             const FrameDev& fr, const SubPatches& sub, const Framebuffer& fb,
                                             float* __restrict__ mshade, BigQuad* big, long long big_cap,
                                             unsigned long long* ctrl, const V3& light, long long& frags) {
    using SM = FusedSmem<PS, NS>;
    constexpr int G = SM::G, NV = SM::NV, NQ = PS * PS, BPL = PS / 8, NB = SM::NB, TH = fused_threads<NS>();
    GroupStage<NS>& cur = sm.st[b];
    GroupStage<NS>& nxt = sm.st[b ^ 1];
    const int tid = threadIdx.x, lane = tid & 31;
    const int vmaxx = (fr.W << fr.shift) - 1, vmaxy = (fr.H << fr.shift) - 1;
    // the next group's records travel in registers until this group's
    // vertices are done
    float4 next_range = make_float4(0.f, 0.f, 0.f, 0.f);
    int2 next_meta = make_int2(0, 0);
    if (tid < n_next) {
        next_range = sub.range[next_base + tid];
        next_meta = sub.meta[next_base + tid];
    }
    // dice vertices (kernels/dice.cl:37-80); vertex i is (k, nu, nv) with
    // i = k * NV + nv * G + nu, stepped by TH without divisions
    constexpr int DK = TH / NV, DNV = (TH % NV) / G, DNU = (TH % NV) % G;
    int k = tid / NV, nv = (tid % NV) / G, nu = (tid % NV) % G;
    for (int i = tid; i < n * NV; i += TH) {
        const float* mvp = cur.mvp[k];
        float4 pos = dice_eye_w(cur.tv[k][0], mvp, fr, cur.cp[k], sm.tx[k][nu], sm.ty[k][nv], sm.vw[k][nu],
                                sm.cw[k][nv]);
        int px, py;
        float dep;
        project_vertex_persp(mvp + 16, fr, pos, px, py, dep);
        sm.pxy[i] = make_int2(px, py);
        sm.edep[i] = make_float4(pos.x, pos.y, pos.z, dep);
        if (pos.z == 0.0f) {
            // a vertex at eye z == 0 drops every 8x8 block it belongs to (kernels/reyes.cl:130-162)
            unsigned zb = 0;
            for (int bv = max(nv - 1, 0) / 8; bv <= min(nv, PS - 1) / 8; ++bv)
                for (int bu = max(nu - 1, 0) / 8; bu <= min(nu, PS - 1) / 8; ++bu) zb |= 1u << (bu + bv * BPL);
            atomicOr(&sm.zero[b][k], zb);
        }
        k += DK;
        nv += DNV;
        nu += DNU;
        if (nu >= G) { nu -= G; ++nv; }
        if (nv >= G) { nv -= G; ++k; }
    }
    if (tid < n_next) {
        nxt.range[tid] = next_range;
        nxt.meta[tid] = next_meta;
    }
    __syncthreads();
    if (n_next > 0) stage_inputs(nxt, n_next, draws);
    // Block bounds over front-facing quads (kernels/reyes.cl:120-166), and
    // the list of quads that can touch a pixel: a quad with a large bbox, or
    // a small one with an accepted winding and a pixel centre in its bbox.
    // n * NQ is a multiple of 32, so whole warps run each round; the quads of
    // one warp share a sub-patch, and their 8x8 blocks are fixed by the lane:
    // one block at PS = 8, and at PS = 16 two, lanes with bit 3 clear / set.
    for (int i = tid; i < n * NQ; i += TH) {
        const int k = i / NQ, q = i % NQ;
        const int nu = q % PS, nv = q / PS, i0 = k * NV + nu + nv * G;
        const int2 c0 = sm.pxy[i0], c1 = sm.pxy[i0 + 1], c2 = sm.pxy[i0 + G], c3 = sm.pxy[i0 + G + 1];
        const int qx[4] = {c0.x, c1.x, c2.x, c3.x};
        const int qy[4] = {c0.y, c1.y, c2.y, c3.y};
        const int minx = min(min(qx[0], qx[1]), min(qx[2], qx[3]));
        const int maxx = max(max(qx[0], qx[1]), max(qx[2], qx[3]));
        const int miny = min(min(qy[0], qy[1]), min(qy[2], qy[3]));
        const int maxy = max(max(qy[0], qy[1]), max(qy[2], qy[3]));
        // is_front_facing (kernels/reyes.cl:54-65) on wrapped int32
        const int d1x = wsub(qx[1], qx[0]), d1y = wsub(qy[1], qy[0]);
        const int d2x = wsub(qx[2], qx[0]), d2y = wsub(qy[2], qy[0]);
        const int d3x = wsub(qx[3], qx[0]), d3y = wsub(qy[3], qy[0]);
        const bool wind = wsub(wmul(d1x, d3y), wmul(d3x, d1y)) < 0 || wsub(wmul(d3x, d2y), wmul(d2x, d3y)) < 0;
        const bool fast = minx >= -kFastCoord && maxx <= kFastCoord && miny >= -kFastCoord && maxy <= kFastCoord &&
                          maxx - minx <= kFastExtent && maxy - miny <= kFastExtent;
        // with backface culling, a warp whose quads are all small and face
        // away lists none of them and leaves its block bound as it is (the
        // steps below would add (viewport max, 0)): it skips them (about half
        // the warps of a scene of randomly oriented patches)
        if (fr.backface && __all_sync(0xffffffffu, fast && !wind)) continue;
        int x0, y0, x1, y1;
        const bool live = !fast || (wind && quad_pixels(fr, minx, miny, maxx, maxy, x0, y0, x1, y1));
        const unsigned lm = __ballot_sync(0xffffffffu, live);
        unsigned at = 0;
        if (lane == 0 && lm) at = atomicAdd(&sm.n_live[b], (unsigned)__popc(lm));
        at = __shfl_sync(0xffffffffu, at, 0);
        if (live) sm.live[at + __popc(lm & lanemask_lt())] = (unsigned short)i;
        // the block bound starts at (viewport max, 0) and takes front-facing quads
        const bool ff = !fr.backface || wind;
        const unsigned grp = PS == 8 ? 0xffffffffu : ((lane & 8) ? 0xff00ff00u : 0x00ff00ffu);
        const int bx0 = __reduce_min_sync(grp, ff ? min(vmaxx, minx) : vmaxx);
        const int by0 = __reduce_min_sync(grp, ff ? min(vmaxy, miny) : vmaxy);
        const int bx1 = __reduce_max_sync(grp, ff ? max(0, maxx) : 0);
        const int by1 = __reduce_max_sync(grp, ff ? max(0, maxy) : 0);
        if ((lane & (PS == 8 ? 31 : 23)) == 0) {
            int* bb = sm.bound[b][k][(nu >> 3) + (nv >> 3) * BPL];
            atomicMin(bb + 0, bx0);
            atomicMin(bb + 1, by0);
            atomicMax(bb + 2, bx1);
            atomicMax(bb + 3, by1);
        }
    }
    __syncthreads();
    // the next group's weights and state, from the highest thread down (the
    // raster below occupies the lowest threads)
    prepare_group(sm, b ^ 1, n_next, fr, TH - 1 - tid);
    // rasterize the listed quads of live blocks
    const int n_live = (int)sm.n_live[b];
    for (int j = tid; j < n_live; j += TH) {
        const int i = sm.live[j];
        const int k = i / NQ, q = i % NQ;
        const int nu = q % PS, nv = q / PS, blk = (nu >> 3) + (nv >> 3) * BPL;
        // the block's tile range, or skip it (clamp, eye-plane flag, is_empty)
        const int* bb = sm.bound[b][k][blk];
        int tiles[4];
        if (!block_tiles(fr, bb[0], bb[1], bb[2], bb[3], !((sm.zero[b][k] >> blk) & 1), tiles)) continue;
        const int i0 = k * NV + nu + nv * G;
        const int idx[4] = {i0, i0 + 1, i0 + G, i0 + G + 1};
        int qx[4], qy[4];
        float qd[4];
        float4 e[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int2 q = sm.pxy[idx[c]];
            e[c] = sm.edep[idx[c]];
            qx[c] = q.x;
            qy[c] = q.y;
            qd[c] = e[c].w;
        }
        const long long s = base + k;
        const unsigned mp_id = (unsigned)(s * NQ + nu + nv * PS);
        const int view = cur.tv[k][1];
        unsigned long long* keys = fb.keys + (long long)view * fb.key_pixels;
        int minx, miny, maxx, maxy, f = 0;
        const bool fast = quad_is_fast(qx, qy, minx, miny, maxx, maxy);
        if (fast)
            f = raster_quad_fast(fr, keys, qx, qy, qd, minx, miny, maxx, maxy, mp_id);
        else
            push_big(big, big_cap, ctrl, qx, qy, qd, mp_id, view, tiles);
        if (f > 0 || !fast) {
            // the diffuse factor of a quad that may own pixels; resolve
            // turns it into the colour of kernels/reyes.cl:191
            mshade[mp_id] = shade_m_l(light, e[0].x, e[0].y, e[0].z, e[1].x, e[1].y, e[1].z, e[2].x, e[2].y, e[2].z,
                                      e[3].x, e[3].y, e[3].z);
        }
        frags += f;
    }
    cp_async_wait_all();
    __syncthreads();
}

template <int PS, int NS>
__global__ void __launch_bounds__(fused_threads<NS>(), 768 / fused_threads<NS>())
    raster_fused_kernel(const DrawDev* __restrict__ draws, FrameDev frp, SubPatches sub, Framebuffer fb,
                        float* __restrict__ mshade, BigQuad* big, long long big_cap, unsigned long long* ctrl) {
    using SM = FusedSmem<PS, NS>;
    FrameDev fr = frp;
    load_amplitude(fr);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SM& sm = *reinterpret_cast<SM*>(smem_raw);
    // an earlier stage of the frame failed (the host reports it): the list
    // may be incomplete, so nothing is rasterized
    if (*(volatile unsigned long long*)cw(ctrl, kStatus) != 0) return;
    long long S = (long long)*(volatile unsigned long long*)cw(ctrl, kOutCount);
    if (S > sub.capacity) S = sub.capacity;
    const V3 light = light_dir();
    long long frags = 0;
    const long long stride = (long long)gridDim.x * NS;
    long long base = (long long)blockIdx.x * NS;
    if (base < S) stage_group(sm, base, (int)min((long long)NS, S - base), sub, draws, fr);
    for (int b = 0; base < S; base += stride, b ^= 1) {
        const long long next = base + stride;
        raster_group<PS, NS>(sm, b, base, (int)min((long long)NS, S - base), next,
                             next < S ? (int)min((long long)NS, S - next) : 0, draws, fr, sub, fb, mshade, big,
                             big_cap, ctrl, light, frags);
    }
    frags = __reduce_add_sync(0xffffffffu, (unsigned)frags);
    if ((threadIdx.x & 31) == 0 && frags) atomicAdd(cw(ctrl, kFragments), (unsigned long long)frags);
}

// One launch per frame: blocks [0, n_bns_ctas) first run the bound-and-split
// warp loop (each emitted slot is marked with the frame's epoch); then every
// block claims groups of NS consecutive emitted slots, waits (bounded) until
// they are marked or lie beyond the final count, and rasterizes them.  The
// grid is sized to what is resident at once, and the bound-and-split blocks
// have the lowest indices, so the blocks that wait never wait on a block that
// has not started; a wait that runs out stops consumption and reports
// MP_ERR_TIMEOUT.
// Shared memory of the frame kernel: the raster's, or what its
// bound-and-split blocks stage (draw records, nine samples per thread).
constexpr int kFrameStagedDraws = 64;
constexpr size_t kFramePtsOffset = (kFrameStagedDraws * sizeof(DrawDev) + 15) / 16 * 16;
template <int PS, int NS>
constexpr size_t frame_smem() {
    return sizeof(FusedSmem<PS, NS>) > kFramePtsOffset + 27 * fused_threads<NS>() * sizeof(float)
               ? sizeof(FusedSmem<PS, NS>)
               : kFramePtsOffset + 27 * fused_threads<NS>() * sizeof(float);
}

template <int PS, int NS>
__global__ void __launch_bounds__(fused_threads<NS>(), 768 / fused_threads<NS>())
    frame_kernel(const DrawDev* __restrict__ gdraws, const int* __restrict__ root_prefix, int n_draws, FrameDev frp,
                 Queue q, SubPatches sub, Framebuffer fb, float* __restrict__ mshade, BigQuad* big, long long big_cap,
                 unsigned long long* ctrl, long long spin_limit, int n_bns_ctas) {
    using SM = FusedSmem<PS, NS>;
    FrameDev fr = frp;
    load_amplitude(fr);
    // bound-and-split blocks: draw records, then the bound samples of each thread
    // (frame_smem() sizes the launch for both uses)
    constexpr int kStaged = kFrameStagedDraws;
    constexpr size_t kPtsOffset = kFramePtsOffset;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ long long s_group;
    if ((int)blockIdx.x < n_bns_ctas) {
        // draw constants staged in the (not yet used) raster buffer
        DrawDev* sd = reinterpret_cast<DrawDev*>(smem_raw);
        const bool staged = n_draws <= kStaged;
        if (staged) {
            const int words = n_draws * (int)(sizeof(DrawDev) / 4);
            for (int i = threadIdx.x; i < words; i += blockDim.x)
                reinterpret_cast<int*>(sd)[i] = __ldg(reinterpret_cast<const int*>(gdraws) + i);
            __syncthreads();
        }
        // the CPU criterion only: the host runs the GPU criterion as two launches
        float* pts = reinterpret_cast<float*>(smem_raw + kPtsOffset);
        bns_warp_loop<0, fused_threads<NS>()>(staged ? sd : gdraws, root_prefix, n_draws, fr, q, sub, sub.seq, ctrl,
                                        spin_limit, pts);
        __syncthreads();
    }
    SM& sm = *reinterpret_cast<SM*>(smem_raw);
    const unsigned epoch = (unsigned)*(volatile unsigned long long*)cw(ctrl, kEpoch);
    const V3 light = light_dir();
    long long frags = 0;
    while (true) {
        if (threadIdx.x == 0) s_group = (long long)atomicAdd(cw(ctrl, kGroupTicket), 1ull);
        __syncthreads();
        const long long base = s_group * NS;
        int ready = 0, gave_up = 0;
        if ((int)threadIdx.x < NS) {
            const long long slot = base + threadIdx.x;
            long long idle = 0;
            unsigned ns = 32;
            while (true) {
                if (slot < sub.capacity && ld_acquire_u32(sub.seq + slot) == epoch) {
                    ready = 1;
                    break;
                }
                if (ld_acquire_u64(cw(ctrl, kDone))) {
                    // every emit's count update precedes the done flag
                    const long long fin = (long long)atomicAdd(cw(ctrl, kOutCount), 0ull);
                    if (slot >= fin || slot >= sub.capacity) break;  // beyond the end of the list
                }
                if (++idle > spin_limit) {
                    set_status(ctrl, kErrTimeout);
                    gave_up = 1;
                    break;
                }
                __nanosleep(ns);
                if (ns < 256) ns <<= 1;
            }
        }
        const int n = __syncthreads_count(ready);
        if (n == 0 || __syncthreads_or(gave_up)) break;
        stage_group(sm, base, n, sub, gdraws, fr);
        raster_group<PS, NS>(sm, 0, base, n, 0, 0, gdraws, fr, sub, fb, mshade, big, big_cap, ctrl, light, frags);
    }
    frags = __reduce_add_sync(0xffffffffu, (unsigned)frags);
    if ((threadIdx.x & 31) == 0 && frags) atomicAdd(cw(ctrl, kFragments), (unsigned long long)frags);
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
        unsigned long long* keys = fb.keys + (long long)b.view * fb.key_pixels;
        long long total = (long long)s_nx * s_ny;
        int frags = 0;
        for (long long c = threadIdx.x; c < total; c += kBigThreads) {
            int x = s_x[c % s_nx], y = s_y[c / s_nx];
            int tx = wadd(x << fr.shift, 0), ty = y << fr.shift;
            float depth = 1.0f;
            bool in1 = tri_test(t1, tx, ty, depth);
            bool in2 = tri_test(t2, tx, ty, depth);
            if (in1 || in2) {
                const unsigned idp = idepth_of(depth);
                if (idp < 0x7fffffffu)
                    atomicMin(keys + key_index(fr, x, y), ((unsigned long long)idp << 32) | b.mp_id);
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

__global__ void clear_kernel(Framebuffer fb, FrameDev fr, int with_color, unsigned long long* reset_ctrl,
                             long long roots) {
    // the frame's bound-and-split reset rides along (one thread)
    if (reset_ctrl && blockIdx.x == 0 && threadIdx.x == 0) bns_reset(reset_ctrl, roots);
    const long long nk = fb.key_pixels * fb.views, n = fb.pixels * fb.views;
    const float4 cc = make_float4(fr.clear[0], fr.clear[1], fr.clear[2], fr.clear[3]);
    const long long stride = (long long)gridDim.x * blockDim.x;
    // the key buffer is a whole number of 32x32 tiles per view: two keys per 16-byte store
    ulonglong2* k2 = reinterpret_cast<ulonglong2*>(fb.keys);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nk / 2; i += stride)
        k2[i] = make_ulonglong2(kClearKey, kClearKey);
    if (with_color)
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
            fb.color[i] = cc;
            fb.depth[i] = 0x7fffffff;
        }
}

// Key of output pixel i (all views).
__device__ __forceinline__ unsigned long long key_of(const FrameDev& fr, const Framebuffer& fb, long long i) {
    const long long v = i / fb.pixels;
    int x, y;
    fb_pixel(fr, i - v * fb.pixels, x, y);
    return fb.keys[v * fb.key_pixels + key_index(fr, x, y)];
}

// Colour of each pixel from its winning micropolygon: the diffuse factor the
// fused kernel stored, the draw's colour (kernels/reyes.cl:191), and the
// winning depth (kernels/reyes.cl:389).  Each thread takes kResolvePixels
// pixels a grid apart and issues their key loads, then their gathers, before
// any use, so the dependent loads of several pixels are in flight at once.
constexpr int kResolvePixels = 4;
template <int PS>
__global__ void resolve_kernel(const DrawDev* __restrict__ draws, FrameDev fr, SubPatches sub, Framebuffer fb,
                               const float* __restrict__ mshade) {
    const long long n = fb.pixels * fb.views;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; i0 < n; i0 += kResolvePixels * stride) {
        unsigned long long key[kResolvePixels];
#pragma unroll
        for (int u = 0; u < kResolvePixels; ++u) {
            const long long i = i0 + u * stride;
            key[u] = i < n ? key_of(fr, fb, i) : kClearKey;
        }
        int draw[kResolvePixels];
        float m[kResolvePixels];
#pragma unroll
        for (int u = 0; u < kResolvePixels; ++u) {
            draw[u] = 0;
            m[u] = 0.0f;
            if (key[u] != kClearKey) {
                const unsigned id = (unsigned)(key[u] & 0xffffffffu);
                draw[u] = sub.meta[id / (PS * PS)].y;
                m[u] = mshade[id];
            }
        }
#pragma unroll
        for (int u = 0; u < kResolvePixels; ++u) {
            const long long i = i0 + u * stride;
            if (i >= n) break;
            if (key[u] == kClearKey) {
                fb.color[i] = make_float4(fr.clear[0], fr.clear[1], fr.clear[2], fr.clear[3]);
                fb.depth[i] = 0x7fffffff;
            } else {
                fb.color[i] = shade_color(m[u], draws[draw[u]].color);
                fb.depth[i] = (int)(key[u] >> 32);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Plain per-pass kernels

template <int PS>
__global__ void dice_grid_kernel(const DrawDev* __restrict__ draws, FrameDev frp, SubPatches sub, long long base,
                                 int count, float4* pos_grid, int2* pxl_grid, float* depth_grid) {
    FrameDev fr = frp;
    load_amplitude(fr);
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
            unsigned long long* keys = fb.keys + (long long)view * fb.key_pixels;
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
        const unsigned long long key = key_of(fr, fb, i);
        const unsigned long long id = key & 0xffffffffull;
        if (key != kClearKey && id >= id_lo && id < id_hi) {
            fb.color[i] = color_grid[id - id_lo];
            fb.depth[i] = (int)(key >> 32);
        }
    }
}

// Display image of one framebuffer layer, as the reference's tex_draw shader
// shows it (shaders/tex_draw.frag): untile, gamma pow(c, 0.454545) on RGB,
// then the unorm8 conversion of an 8-bit window (round(clamp(c, 0, 1) * 255)).
// Rows are written top first; the shader's gl_FragCoord.y counts from the
// bottom, so output row r is framebuffer row H - 1 - r.
__global__ void image_kernel(const float4* __restrict__ color, FrameDev fr, unsigned char* __restrict__ rgb) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long long)fr.W * fr.H) return;
    const int x = (int)(i % fr.W), r = (int)(i / fr.W);
    const float4 c = color[fb_index(fr, x, fr.H - 1 - r)];
    const float v[3] = {c.x, c.y, c.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float g = fminf(fmaxf(powf(v[k], 0.454545f), 0.0f), 1.0f);
        rgb[3 * i + k] = (unsigned char)__float2int_rn(fmul(g, 255.0f));
    }
}

// 64-bit atomicMin throughput probe: pattern 0 = uniform random slots,
// pattern 1 = each warp updates one 8x8-pixel tile (micropolygon-like locality).
__global__ void widen_points_kernel(const float* __restrict__ xyz, float4* __restrict__ out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 1.0f);
}

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

template <typename K>
int resident_grid(K kernel, size_t smem, int threads) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    if (per_sm < 1) per_sm = 1;
    return sms * per_sm;
}

// Calls f(kernel instantiation tag) for the (PS, dice_group) pair.
template <int PS, int NS>
struct Tag {
    static constexpr int ps = PS, ns = NS;
};
template <typename F>
void dispatch_group(int PS, int group, F&& f) {
    if (PS == 16) {
        if (group == 2) f(Tag<16, 2>{});
        else if (group == 3) f(Tag<16, 3>{});
        else if (group == 4) f(Tag<16, 4>{});
        else f(Tag<16, 6>{});
    } else {
        if (group == 8) f(Tag<8, 8>{});
        else if (group == 11) f(Tag<8, 11>{});
        else if (group == 16) f(Tag<8, 16>{});
        else f(Tag<8, 22>{});
    }
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

void launch_clear(const Framebuffer& fb, const FrameDev& fr, int with_color, cudaStream_t s,
                  unsigned long long* reset_ctrl, long long roots) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = with_color ? fb.pixels * fb.views : fb.key_pixels * fb.views / 2;
    clear_kernel<<<(int)std::min<long long>(grid_for(want, 256), (long long)sms * 8), 256, 0, s>>>(fb, fr, with_color,
                                                                                             reset_ctrl, roots);
}

int raster_fused_grid(int PS, int group) {
    int g = 0;
    dispatch_group(PS, group, [&](auto t) {
        using T = decltype(t);
        g = resident_grid(raster_fused_kernel<T::ps, T::ns>, sizeof(FusedSmem<T::ps, T::ns>),
                          fused_threads<T::ns>());
    });
    return g;
}

void launch_raster_fused(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, const Framebuffer& fb,
                         float* mshade, BigQuad* big, long long big_cap, unsigned long long* ctrl, int grid, int group,
                         cudaStream_t s) {
    dispatch_group(fr.PS, group, [&](auto t) {
        using T = decltype(t);
        raster_fused_kernel<T::ps, T::ns><<<grid, fused_threads<T::ns>(), sizeof(FusedSmem<T::ps, T::ns>), s>>>(
            draws, fr, sub, fb, mshade, big, big_cap, ctrl);
    });
}

int frame_kernel_grid(int PS, int group) {
    int g = 0;
    dispatch_group(PS, group, [&](auto t) {
        using T = decltype(t);
        g = resident_grid(frame_kernel<T::ps, T::ns>, frame_smem<T::ps, T::ns>(), fused_threads<T::ns>());
    });
    return g;
}

void launch_frame_kernel(const DrawDev* draws, const int* root_prefix, int n_draws, const FrameDev& fr, const Queue& q,
                         const SubPatches& sub, const Framebuffer& fb, float* mshade, BigQuad* big, long long big_cap,
                         unsigned long long* ctrl, long long spin_limit, int grid, int n_bns_ctas, int group,
                         cudaStream_t s) {
    dispatch_group(fr.PS, group, [&](auto t) {
        using T = decltype(t);
        frame_kernel<T::ps, T::ns><<<grid, fused_threads<T::ns>(), frame_smem<T::ps, T::ns>(), s>>>(
            draws, root_prefix, n_draws, fr, q, sub, fb, mshade, big, big_cap, ctrl, spin_limit, n_bns_ctas);
    });
}

void launch_raster_big(const DrawDev*, const FrameDev& fr, const Framebuffer& fb, const BigQuad* big,
                       long long big_cap, unsigned long long* ctrl, cudaStream_t s) {
    raster_big_kernel<<<256, kBigThreads, 0, s>>>(fr, fb, big, big_cap, ctrl);
}

void launch_resolve(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, const Framebuffer& fb,
                    const float* mshade, cudaStream_t s) {
    int g = grid_for((fb.pixels * fb.views + kResolvePixels - 1) / kResolvePixels, 256);
    if (fr.PS == 16)
        resolve_kernel<16><<<g, 256, 0, s>>>(draws, fr, sub, fb, mshade);
    else
        resolve_kernel<8><<<g, 256, 0, s>>>(draws, fr, sub, fb, mshade);
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

void launch_widen_points(const float* xyz, float4* out, long long n, cudaStream_t s) {
    if (n > 0) widen_points_kernel<<<grid_for(n, 256), 256, 0, s>>>(xyz, out, n);
}

void launch_image(const float4* color, const FrameDev& fr, unsigned char* rgb, cudaStream_t s) {
    const long long n = (long long)fr.W * fr.H;
    image_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(color, fr, rgb);
}

void launch_atomic_bench(unsigned long long* buf, long long n_slots, long long n_ops, int pattern, cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    atomic_bench_kernel<<<sms * 8, 256, 0, s>>>(buf, n_slots, n_ops, pattern);
}

}  // namespace mp
