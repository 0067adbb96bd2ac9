// The bound-and-split warp loop, shared by the standalone persistent kernel
// (mp_bns.cu) and the frame kernel that overlaps it with rasterization
// (mp_raster.cu).  See mp_bns.cu for the queue protocol.
#pragma once
#include "mp_internal.h"

namespace mp {

__device__ __forceinline__ unsigned long long* cw(unsigned long long* ctrl, int w) { return ctrl + w * kCtrlStride; }

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// A release fence followed by relaxed stores: each store publishes every
// write this thread made before the fence (the PTX release pattern), so two
// flags need one fence.
__device__ __forceinline__ void fence_acq_rel_gpu() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
__device__ __forceinline__ void st_relaxed_u32(unsigned* p, unsigned v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// The per-frame reset of the bound-and-split control words: roots tickets
// filled and outstanding, counters cleared, the frame epoch advanced.
__device__ __forceinline__ void bns_reset(unsigned long long* ctrl, long long roots) {
    *cw(ctrl, kQTail) = ((unsigned long long)roots << 32) | (unsigned long long)roots;
    *cw(ctrl, kQHead) = 0;
    *cw(ctrl, kOutstanding) = 0;
    *cw(ctrl, kOutCount) = 0;
    *cw(ctrl, kDone) = roots == 0 ? 1 : 0;
    *cw(ctrl, kStatus) = 0;
    *cw(ctrl, kEpoch) = *cw(ctrl, kEpoch) + 1;
    *cw(ctrl, kRoots) = (unsigned long long)roots;
    *cw(ctrl, kBigCount) = 0;
    *cw(ctrl, kFragments) = 0;
    *cw(ctrl, kBigOverflow) = 0;
    *cw(ctrl, kGroupTicket) = 0;
    *cw(ctrl, kMaxDepth) = 0;
    *cw(ctrl, kSortDone) = 0;
}

__device__ __forceinline__ void set_status(unsigned long long* ctrl, int code) {
    atomicCAS(cw(ctrl, kStatus), 0ull, (unsigned long long)code);
}

// kQTail packs two counters updated by one atomic: the high 32 bits count
// queue tickets ever filled (roots included), the low 32 bits the items pushed
// but not yet finished.  A warp step adds (2*splits << 32) + (2*splits -
// processed); the borrow of a negative low part is cancelled by the carry.
constexpr unsigned long long kLow32 = 0xffffffffull;

constexpr unsigned long long kNoTicket = ~0ull;

// Runs one warp's share of a frame's bound-and-split until the done flag is
// raised.  Emitted sub-patches go to `out`; when out_seq is given, each
// emitted slot is also marked with the frame's epoch (release) for consumers
// that run concurrently.  CRIT selects the bound criterion (bns_decide).
// With the CPU criterion and ST > 0 (the block's thread count), children take
// six of their nine bound samples from the parent through the queue's pts
// records (which must exist); `pts` is shared memory of 27 floats per thread
// (point layout of spi()).
template <int CRIT, int ST>
__device__ __forceinline__ void bns_warp_loop(const DrawDev* draws, const int* __restrict__ root_prefix, int n_draws,
                                              const FrameDev& fr, const Queue& q, const SubPatches& out,
                                              unsigned* out_seq, unsigned long long* ctrl, long long spin_limit,
                                              float* pts) {
    constexpr bool inherit = CRIT == 0 && ST > 0;
    constexpr int st = ST;
    float* sp = inherit ? pts + threadIdx.x : nullptr;
    const int lane = threadIdx.x & 31;
    const unsigned epoch = (unsigned)*(volatile unsigned long long*)cw(ctrl, kEpoch);
    const unsigned long long R = *(volatile unsigned long long*)cw(ctrl, kRoots);
    unsigned long long ticket = kNoTicket;
    long long idle = 0;
    unsigned sleep_ns = 32;
    unsigned max_depth = 0;   // deepest emitted sub-patch of this warp so far (lane 0)
    while (true) {
        // hand new tickets to the lanes that have none
        unsigned need = __ballot_sync(0xffffffffu, ticket == kNoTicket);
        if (need) {
            int leader = __ffs(need) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(cw(ctrl, kQHead), (unsigned long long)__popc(need));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (ticket == kNoTicket) ticket = base + __popc(need & lanemask_lt());
        }
        bool ready = false;
        if (ticket < R) {
            ready = true;
        } else {
            unsigned long long slot = ticket - R;
            if ((long long)slot < q.capacity) ready = ld_acquire_u32(q.seq + slot) == epoch;
        }
        unsigned rmask = __ballot_sync(0xffffffffu, ready);
        if (rmask == 0) {
            unsigned long long done = 0;
            if (lane == 0) done = *(volatile unsigned long long*)cw(ctrl, kDone);
            done = __shfl_sync(0xffffffffu, done, 0);
            if (done) break;
            if (++idle > spin_limit) {
                if (lane == 0) {
                    set_status(ctrl, kErrTimeout);
                    st_release_u64(cw(ctrl, kDone), 1ull);
                }
                break;
            }
            __nanosleep(sleep_ns);
            if (sleep_ns < 512) sleep_ns <<= 1;
            continue;
        }
        idle = 0;
        sleep_ns = 32;
        float4 r = make_float4(0.f, 0.f, 1.f, 1.f);
        int pid = 0, draw = 0, depth = 0;
        unsigned path = 0;
        int dec = -1;
        if (ready) {
            int flag = kInheritNone;
            if (ticket < R) {
                // root: find the draw whose patch range holds this ticket
                int lo = 0, hi = n_draws - 1;
                while (lo < hi) {
                    int mid = (lo + hi + 1) >> 1;
                    if ((unsigned long long)__ldg(root_prefix + mid) <= ticket) lo = mid; else hi = mid - 1;
                }
                draw = lo;
                pid = (int)(ticket - (unsigned long long)__ldg(root_prefix + lo));
            } else {
                unsigned long long slot = ticket - R;
                r = __ldcg(q.range + slot);
                uint2 m = __ldcg(q.meta + slot);
                pid = (int)m.x;
                draw = (int)(m.y & 0xffffffu);
                depth = (int)(m.y >> 24);
                if (q.path) path = __ldcg(q.path + slot);
                if (inherit) flag = load_inherited(q.pts + slot * kPtsPerSlot, sp, st);
            }
            if (inherit)
                dec = bns_decide_inherit(draws[draw], fr, pid, r, depth, flag, sp, st);
            else
                dec = bns_decide<CRIT>(draws[draw], fr, pid, r, depth);
        }
        // One lane issues the step's three independent atomics back to back,
        // so their round trips overlap: output slots for emitted sub-patches,
        // the packed ticket / outstanding-work update for split children (see
        // kQTail above), and the next tickets of the lanes finished here.
        const unsigned emask = __ballot_sync(0xffffffffu, dec == kDraw);
        const bool split = dec == kSplitX || dec == kSplitY;
        const unsigned smask = __ballot_sync(0xffffffffu, split);
        const long long n_child = 2ll * __popc(smask);
        const long long net = n_child - (long long)__popc(rmask);
        const unsigned emit_depth = __reduce_max_sync(0xffffffffu, dec == kDraw ? (unsigned)depth : 0u);
        unsigned long long obase = 0, old = 0, tbase = 0;
        if (lane == 0) {
            if (emask) obase = atomicAdd(cw(ctrl, kOutCount), (unsigned long long)__popc(emask));
            if (emit_depth > max_depth) {
                // the sort packs the frame's keys into root bits above this many path bits
                max_depth = emit_depth;
                atomicMax(cw(ctrl, kMaxDepth), (unsigned long long)emit_depth);
            }
            old = atomicAdd(cw(ctrl, kQTail), ((unsigned long long)n_child << 32) + (unsigned long long)net);
            tbase = atomicAdd(cw(ctrl, kQHead), (unsigned long long)__popc(rmask));
        }
        obase = __shfl_sync(0xffffffffu, obase, 0);
        old = __shfl_sync(0xffffffffu, old, 0);
        tbase = __shfl_sync(0xffffffffu, tbase, 0);
        // emitted sub-patches
        if (dec == kDraw) {
            unsigned long long o = obase + __popc(emask & lanemask_lt());
            if ((long long)o < out.capacity) {
                out.range[o] = r;
                out.meta[o] = make_int2(pid, draw);
                if (out.path) out.path[o] = path;
                // consumers running in the same launch wait for this flag
                if (out_seq) st_release_u32(out_seq + o, epoch);
            } else {
                set_status(ctrl, kErrOverflow);
            }
        }
        bool fits = true;
        if (split) {
            const unsigned long long t0 = (old >> 32) + 2ull * __popc(smask & lanemask_lt());
            const unsigned long long s0 = t0 - R;
            fits = (long long)(s0 + 1) < q.capacity;
            if (fits) {
                float4 c0, c1;
                split_children(r, dec, c0, c1);
                const unsigned meta_y = (unsigned)draw | ((unsigned)(depth + 1) << 24);
                q.range[s0] = c0;
                q.range[s0 + 1] = c1;
                q.meta[s0] = make_uint2((unsigned)pid, meta_y);
                q.meta[s0 + 1] = make_uint2((unsigned)pid, meta_y);
                if (q.path) {
                    // the high half sets bit 31 - depth (paths deeper than 32 keep their first 32 bits)
                    q.path[s0] = path;
                    q.path[s0 + 1] = depth < 32 ? path | (0x80000000u >> depth) : path;
                }
                if (inherit) {
                    store_inherited(q.pts + s0 * kPtsPerSlot, dec, 0, depth + 1, sp, st);
                    store_inherited(q.pts + (s0 + 1) * kPtsPerSlot, dec, 1, depth + 1, sp, st);
                }
                // release: the item stores above are visible before the slots' epochs
                fence_acq_rel_gpu();
                st_relaxed_u32(q.seq + s0, epoch);
                st_relaxed_u32(q.seq + s0 + 1, epoch);
            } else {
                set_status(ctrl, kErrOverflow);
            }
        }
        const unsigned lost = __ballot_sync(0xffffffffu, !fits);
        if (lane == 0) {
            long long remaining = (long long)(old & kLow32) + net;
            if (lost) {
                // children that found no slot are never processed: take them back
                const long long back = -2ll * __popc(lost);
                unsigned long long o2 = atomicAdd(cw(ctrl, kQTail), (unsigned long long)back);
                remaining = (long long)(o2 & kLow32) + back;
            }
            if (remaining == 0) st_release_u64(cw(ctrl, kDone), 1ull);
        }
        if (ready) ticket = tbase + __popc(rmask & lanemask_lt());
    }
}

}  // namespace mp
