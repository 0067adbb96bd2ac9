// Bound-and-split kernels.
//
// Batched path: one persistent launch per frame over every draw's patches.
// Warps hold queue tickets; a ticket below the root count is a root range
// (0,0)-(1,1) of one patch, any other ticket is a slot that another warp
// fills with a split child.  Emitted sub-patches and children are compacted
// with warp ballots (one atomic per warp and role).  Termination: an
// outstanding-work counter updated with one net atomic per warp step; the warp
// that brings it to zero raises the done flag.  Every wait is bounded and
// reports kErrTimeout instead of hanging.
//
// Plain path: the reference's BOUNDED structure
// (src/Reyes/BoundNSplitCLBounded.cpp:170-214, kernels/bound_n_split_multipass.cl):
// pop up to reyes_patches_per_pass ranges from a stack, bound them, compact
// draws and splits with a single-pass decoupled look-back prefix sum (the
// role of kernels/prefix_sum.cl and src/CL/PrefixSum.cpp), move draws to the
// output and children back onto the stack; the host reads the counts.
//
// The bound criterion of both paths is the reference's CPU one
// (src/Reyes/BoundNSplitCLCPU.cpp:117-148), evaluated by mp::bns_decide.
#include "mp_bns_loop.cuh"

namespace mp {

namespace {


constexpr int kBnsBlock = 128;
constexpr int kBnsSmemDraws = 64;

template <int CRIT>
__global__ void __launch_bounds__(kBnsBlock) bns_persistent_kernel(const DrawDev* __restrict__ gdraws,
                                                                   const int* __restrict__ root_prefix,
                                                                   int n_draws, FrameDev fr, Queue q,
                                                                   SubPatches out, unsigned long long* ctrl,
                                                                   long long spin_limit) {
    // draw constants staged in shared memory when they fit
    __shared__ DrawDev s_draws[kBnsSmemDraws];
    __shared__ float s_pts[27 * kBnsBlock];   // nine bound samples per thread
    const bool staged = n_draws <= kBnsSmemDraws;
    if (staged) {
        const int words = n_draws * (int)(sizeof(DrawDev) / 4);
        for (int i = threadIdx.x; i < words; i += blockDim.x)
            reinterpret_cast<int*>(s_draws)[i] = __ldg(reinterpret_cast<const int*>(gdraws) + i);
        __syncthreads();
    }
    bns_warp_loop<CRIT, CRIT == 0 ? kBnsBlock : 0>(staged ? s_draws : gdraws, root_prefix, n_draws, fr, q, out, nullptr,
                                                   ctrl, spin_limit, s_pts);
}

// ---------------------------------------------------------------------------
// Plain path

__global__ void bns_init_stack_kernel(Queue stack, int draw, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // src/Reyes/BoundNSplitCLCPU.cpp:41-44: one root range per patch
    stack.range[i] = make_float4(0.f, 0.f, 1.f, 1.f);
    stack.meta[i] = make_uint2((unsigned)i, (unsigned)draw);
}

constexpr int kScanBlock = 256;
constexpr int kScanItems = 4;
constexpr int kScanTileItems = kScanBlock * kScanItems;
constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagPrefix = 2ull << 62;
constexpr unsigned long long kValMask = (1ull << 62) - 1;

// bound kernel of one pass: decision, copy of the range to the pads, packed
// scan key (draw + split << 31); also clears the scan state of this pass.
template <int CRIT>
__global__ void bns_pass_bound_kernel(const DrawDev* __restrict__ draws, FrameDev fr, Queue stack,
                                      long long offset, int batch, float4* pad_range, uint2* pad_meta,
                                      unsigned char* dec_out, unsigned long long* keys,
                                      unsigned long long* scan_state, long long n_tiles,
                                      unsigned long long* ctrl) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long t = i; t < n_tiles; t += (long long)gridDim.x * blockDim.x) scan_state[t] = 0;
    if (i == 0) *cw(ctrl, kScanTile) = 0;
    if (i >= batch) return;
    float4 r = stack.range[offset + i];
    uint2 m = stack.meta[offset + i];
    int draw = (int)(m.y & 0xffffffu), depth = (int)(m.y >> 24);
    int dec = bns_decide<CRIT>(draws[draw], fr, (int)m.x, r, depth);
    pad_range[i] = r;
    pad_meta[i] = m;
    dec_out[i] = (unsigned char)dec;
    keys[i] = (dec == kDraw ? 1ull : 0ull) | ((dec == kSplitX || dec == kSplitY) ? (1ull << 31) : 0ull);
}

// Single-pass exclusive prefix sum over 62-bit values with decoupled
// look-back (Merrill & Garland).  Tiles take their index from a ticket
// counter, so a tile only ever waits for tiles that are already running.
__global__ void __launch_bounds__(kScanBlock) scan_kernel(const unsigned long long* __restrict__ in,
                                                          unsigned long long* out, long long n,
                                                          unsigned long long* state, unsigned long long* ctrl,
                                                          long long spin_limit, int inclusive) {
    __shared__ unsigned long long s_items[kScanTileItems];
    __shared__ unsigned long long s_warp[kScanBlock / 32];
    __shared__ unsigned long long s_prefix;
    __shared__ long long s_tile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = (long long)atomicAdd(cw(ctrl, kScanTile), 1ull);
    __syncthreads();
    const long long tile = s_tile;
    const long long base = tile * kScanTileItems;
    for (int k = 0; k < kScanItems; ++k) {
        long long idx = base + k * kScanBlock + tid;
        s_items[k * kScanBlock + tid] = idx < n ? in[idx] : 0ull;
    }
    __syncthreads();
    unsigned long long v[kScanItems];
    unsigned long long tsum = 0;
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = s_items[tid * kScanItems + k];
        tsum += v[k];
    }
    // exclusive scan of thread sums across the block
    unsigned long long x = tsum;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < kScanBlock / 32 ? s_warp[lane] : 0ull;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kScanBlock / 32) s_warp[lane] = w;
    }
    __syncthreads();
    unsigned long long warp_excl = warp == 0 ? 0ull : s_warp[warp - 1];
    unsigned long long thread_excl = warp_excl + x - tsum;
    const unsigned long long agg = s_warp[kScanBlock / 32 - 1];
    if (tid == 0) {
        unsigned long long prefix = 0;
        if (tile == 0) {
            st_release_u64(state + 0, kFlagPrefix | (agg & kValMask));
        } else {
            st_release_u64(state + tile, kFlagAgg | (agg & kValMask));
            long long pred = tile - 1;
            long long spins = 0;
            while (pred >= 0) {
                unsigned long long s = ld_acquire_u64(state + pred);
                unsigned long long flag = s & ~kValMask;
                if (flag == 0) {
                    if (++spins > spin_limit) {
                        set_status(ctrl, kErrTimeout);
                        break;
                    }
                    __nanosleep(64);
                    continue;
                }
                prefix += s & kValMask;
                if (flag == kFlagPrefix) break;
                --pred;
            }
            st_release_u64(state + tile, kFlagPrefix | ((prefix + agg) & kValMask));
        }
        s_prefix = prefix;
        long long n_tiles = (n + kScanTileItems - 1) / kScanTileItems;
        if (tile == n_tiles - 1) *cw(ctrl, kScanTotal) = (prefix + agg) & kValMask;
    }
    __syncthreads();
    unsigned long long run = s_prefix + thread_excl;
    for (int k = 0; k < kScanItems; ++k) {
        unsigned long long e = run;
        run += v[k];
        s_items[tid * kScanItems + k] = inclusive ? run : e;
    }
    __syncthreads();
    for (int k = 0; k < kScanItems; ++k) {
        long long idx = base + k * kScanBlock + tid;
        if (idx < n) out[idx] = s_items[k * kScanBlock + tid];
    }
}

// move kernel of one pass (kernels/bound_n_split_multipass.cl:55-127): draws
// to the output list, the two halves of each split back onto the stack.
__global__ void bns_pass_move_kernel(const float4* __restrict__ pad_range, const uint2* __restrict__ pad_meta,
                                     const unsigned char* __restrict__ dec_in,
                                     const unsigned long long* __restrict__ prefix, int batch, Queue stack,
                                     long long offset, SubPatches out, long long out_base,
                                     unsigned long long* ctrl) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= batch) return;
    int dec = dec_in[i];
    unsigned long long p = prefix[i];
    float4 r = pad_range[i];
    uint2 m = pad_meta[i];
    if (dec == kDraw) {
        long long o = out_base + (long long)(p & 0x7fffffffull);
        if (o < out.capacity) {
            out.range[o] = r;
            out.meta[o] = make_int2((int)m.x, (int)(m.y & 0xffffffu));
        } else {
            set_status(ctrl, kErrOverflow);
        }
    } else if (dec == kSplitX || dec == kSplitY) {
        long long o = offset + 2 * (long long)(p >> 31);
        if (o + 1 < stack.capacity) {
            float4 c0, c1;
            split_children(r, dec, c0, c1);
            uint2 cm = make_uint2(m.x, (m.y & 0xffffffu) | ((((m.y >> 24) + 1) & 0xffu) << 24));
            stack.range[o] = c0;
            stack.range[o + 1] = c1;
            stack.meta[o] = cm;
            stack.meta[o + 1] = cm;
        } else {
            set_status(ctrl, kErrOverflow);
        }
    }
}

__global__ void i32_to_u64_kernel(const int* in, unsigned long long* out, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (unsigned long long)(long long)in[i] & kValMask;
}
__global__ void u64_to_i32_kernel(const unsigned long long* in, int* out, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (int)(long long)in[i];
}
__global__ void reset_scan_kernel(unsigned long long* state, long long n_tiles, unsigned long long* ctrl) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (long long t = i; t < n_tiles; t += (long long)gridDim.x * blockDim.x) state[t] = 0;
    if (i == 0) {
        *cw(ctrl, kScanTile) = 0;
        *cw(ctrl, kStatus) = 0;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers


int bns_persistent_grid(int criterion) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (criterion == 1)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bns_persistent_kernel<1>, kBnsBlock, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bns_persistent_kernel<0>, kBnsBlock, 0);
    if (per_sm < 1) per_sm = 1;
    return sms * per_sm;
}

void launch_bns_persistent(const DrawDev* draws, const int* root_prefix, int n_draws, const FrameDev& fr,
                           const Queue& q, const SubPatches& out, unsigned long long* ctrl, int grid,
                           long long spin_limit, cudaStream_t s) {
    if (fr.criterion == 1)
        bns_persistent_kernel<1><<<grid, kBnsBlock, 0, s>>>(draws, root_prefix, n_draws, fr, q, out, ctrl, spin_limit);
    else
        bns_persistent_kernel<0><<<grid, kBnsBlock, 0, s>>>(draws, root_prefix, n_draws, fr, q, out, ctrl, spin_limit);
}

void launch_bns_init_stack(const Queue& stack, int draw, int n_patches, cudaStream_t s) {
    if (n_patches <= 0) return;
    bns_init_stack_kernel<<<(n_patches + 255) / 256, 256, 0, s>>>(stack, draw, n_patches);
}

long long scan_state_words(long long n) { return (n + kScanTileItems - 1) / kScanTileItems + 1; }

void launch_bns_pass(const DrawDev* draws, const FrameDev& fr, const Queue& stack, long long offset, int batch,
                     float4* pad_range, uint2* pad_meta, unsigned char* dec, unsigned long long* keys,
                     unsigned long long* scan_state, const SubPatches& out, long long out_base,
                     unsigned long long* ctrl, long long spin_limit, cudaStream_t s) {
    if (batch <= 0) return;
    long long n_tiles = scan_state_words(batch);
    int blocks = (batch + 127) / 128;
    if (fr.criterion == 1)
        bns_pass_bound_kernel<1><<<blocks, 128, 0, s>>>(draws, fr, stack, offset, batch, pad_range, pad_meta, dec, keys,
                                                        scan_state, n_tiles, ctrl);
    else
        bns_pass_bound_kernel<0><<<blocks, 128, 0, s>>>(draws, fr, stack, offset, batch, pad_range, pad_meta, dec, keys,
                                                        scan_state, n_tiles, ctrl);
    int tiles = (int)((batch + kScanTileItems - 1) / kScanTileItems);
    scan_kernel<<<tiles, kScanBlock, 0, s>>>(keys, keys, batch, scan_state, ctrl, spin_limit, 0);
    bns_pass_move_kernel<<<(batch + 255) / 256, 256, 0, s>>>(pad_range, pad_meta, dec, keys, batch, stack, offset,
                                                             out, out_base, ctrl);
}

void launch_inclusive_scan_i32(const int* in, int* out, long long n, unsigned long long* scan_state,
                               unsigned long long* ctrl, long long spin_limit, cudaStream_t s) {
    if (n <= 0) return;
    // scan_state holds scan_state_words(n) words, followed by 2n words of scratch
    long long n_tiles = scan_state_words(n);
    unsigned long long* tmp = scan_state + n_tiles;
    reset_scan_kernel<<<1, 256, 0, s>>>(scan_state, n_tiles, ctrl);
    i32_to_u64_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(in, tmp, n);
    int tiles = (int)((n + kScanTileItems - 1) / kScanTileItems);
    scan_kernel<<<tiles, kScanBlock, 0, s>>>(tmp, tmp + n, n, scan_state, ctrl, spin_limit, 1);
    u64_to_i32_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(tmp + n, out, n);
}

}  // namespace mp
