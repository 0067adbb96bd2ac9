// Canonical order of a frame's emitted sub-patches.
//
// Bound-and-split emits sub-patches in whatever order its warps finish
// them, and the rasterizer numbers micropolygons by their sub-patch's list
// position (ties in depth go to the smaller number).  So that a frame's
// numbering, its winners at depth ties and everything read back from it are
// the same on every run, the list is put into one canonical order before
// rasterization: ascending (root, split path), where root = the draw's first
// root + patch id (draws in call order, as the reference's Scene::draw
// issues them, src/micropolis/Scene.cpp:179-197) and the split path holds,
// from the root down, 1 for each split whose high half the sub-patch lies in
// (bit 31 - d for the split at depth d).  Within one patch that is the
// depth-first order of its split tree, low half first.  The oracle numbers
// its sub-patches in the same order, so the two break ties identically.
//
// The sort is a least-significant-digit radix sort over 8-bit digits of a
// key that packs the root above the frame's D path bits (D = the deepest
// emitted sub-patch, which bound-and-split records; below bit 32 - D every
// path is zero, so the order is that of (root << 32 | path)).  Keys are 32
// bits wide when the frame's root and path bits fit, else 64.  It is one
// launch of a resident grid, in phases separated by grid barriers (bounded
// waits on a counter of the frame's control words):
//   counts -- the digit counts of every pass at once (Adinets & Merrill's
//             one-sweep radix sort; warp matches aggregate a warp's equal
//             digits into one shared add), added to the frame's table;
//   plan   -- every block reads the table: a pass whose digit is the same
//             for every key moves nothing and is skipped;
//   passes -- each moving pass splits the keys into tiles of kSortTile, one
//             per block at a time (rounds of nblk tiles): each tile
//             ranks its digits stably (per-warp counters, warp matches),
//             publishes its digit counts, reorders itself by digit in shared
//             memory while it waits until every tile of its round and the
//             earlier ones has published, adds up the counts of the tiles
//             before it (independent loads, no chain of waits), and writes
//             each digit's run of the tile to consecutive addresses.  The
//             first moving pass forms the keys from the records; the last
//             writes the sub-patch records themselves in canonical order.
// Every wait is bounded (MP_ERR_TIMEOUT, no write after it).
#include "mp_bns_loop.cuh"

namespace mp {

namespace {

constexpr int kKeysBlock = 1024;
constexpr int kSortBlock = 512;
constexpr int kSortWarps = kSortBlock / 32;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortBlock * kSortItems;   // keys per tile
constexpr int kDigits = 256;

__device__ __forceinline__ long long sort_count(const unsigned long long* ctrl, const SubPatches& in,
                                                const SortBuffers& sb) {
    long long n = (long long)*(volatile const unsigned long long*)(ctrl + kOutCount * kCtrlStride);
    if (n > in.capacity) n = in.capacity;
    if (n > sb.capacity) n = sb.capacity;
    return n;
}

__device__ __forceinline__ unsigned frame_epoch(const unsigned long long* ctrl) {
    return (unsigned)*(volatile const unsigned long long*)(ctrl + kEpoch * kCtrlStride);
}

// Counts of the frame's passes: one table per frame parity, so that a
// frame clears the next frame's table while its own is read.
__device__ __forceinline__ unsigned* hist_of(const SortBuffers& sb, unsigned epoch) {
    return sb.hist + (epoch & 1u) * kSortPasses * kDigits;
}

template <typename K>
__device__ __forceinline__ unsigned digit_of(K key, int pass) {
    return (unsigned)(key >> (8 * pass)) & 0xffu;
}

// The root above D path bits (the path's bits below 32 - D are zero).
__device__ __forceinline__ unsigned long long pack_key(unsigned root, unsigned path, unsigned D) {
    return D == 0 ? (unsigned long long)root : ((unsigned long long)root << D) | (path >> (32u - D));
}

// Lanes of the warp whose 8-bit digit equals this lane's (valid = false
// lanes form a group of their own).
__device__ __forceinline__ unsigned match_digit(unsigned d, bool valid) {
    return __match_any_sync(0xffffffffu, valid ? d : 0x100u);
}

// Bits of the frame's keys: the root bits of its root count above D path bits.
__device__ __forceinline__ int key_bits(const unsigned long long* ctrl, unsigned* D_out) {
    const unsigned long long R = *(volatile const unsigned long long*)(ctrl + kRoots * kCtrlStride);
    unsigned D = (unsigned)*(volatile const unsigned long long*)(ctrl + kMaxDepth * kCtrlStride);
    if (D > 32) D = 32;
    if (D_out) *D_out = D;
    const int root_bits = R > 1 ? 64 - __clzll((long long)(R - 1)) : 0;
    return root_bits + (int)D;
}

// Waits (bounded) until all nblk working blocks have arrived at barrier
// number `k` of the frame (the counter ctrl kSortDone is zeroed by the
// frame's reset); false when the wait ran out (the status is then set).
__device__ __forceinline__ bool grid_barrier(unsigned long long* ctrl, unsigned long long k, int nblk,
                                             long long spin_limit, int* s_flag) {
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long* ctr = ctrl + kSortDone * kCtrlStride;
        __threadfence();
        atomicAdd(ctr, 1ull);
        const unsigned long long need = k * (unsigned long long)nblk;
        long long spins = 0;
        int ok = 1;
        while (ld_acquire_u64(ctr) < need) {
            if (++spins > spin_limit) {
                ok = 0;
                set_status(ctrl, kErrTimeout);
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
        *s_flag = ok;
    }
    __syncthreads();
    return *s_flag != 0;
}

// Shared memory of one pass block (the 64-bit layout; 32-bit keys use the
// front half of `keys`).
struct PassSmem {
    unsigned long long keys[kSortTile];           // the tile in digit order
    unsigned vals[kSortTile];
    unsigned short wcount[kSortWarps][kDigits];   // per warp digit counts, then offsets in the tile's digit run
    unsigned tstart[kDigits];                     // exclusive digit starts within the tile
    unsigned start[kDigits];                      // exclusive digit starts of the pass
    unsigned base[kDigits];                       // global position of the tile's first key of each digit
    unsigned part[kDigits];                       // the earlier tiles of the tile's own group, per digit
    unsigned warp_sum[kSortWarps];
    int fail;
};

// Exclusive prefix over the 256 values that threads 0-255 hold (every
// thread of the block calls it; ends with a barrier).
__device__ __forceinline__ unsigned scan_digits(unsigned v, unsigned* warp_sum) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    unsigned x = v;
    if (tid < kDigits) {
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sum[warp] = x;
    }
    __syncthreads();
    unsigned before = 0;
    if (tid < kDigits)
        for (int w = 0; w < warp; ++w) before += warp_sum[w];
    __syncthreads();
    return before + x - v;
}

// One moving pass over keys of type K (see sort_kernel).
//   from_records -- the first moving pass: keys formed from the records
//   last         -- the last moving pass: records written in key order
template <typename K>
__device__ __forceinline__ bool pass_body(PassSmem& sm, const int* __restrict__ root_prefix, const SubPatches& in,
                                          const SubPatches& out, const SortBuffers& sb, unsigned long long* ctrl,
                                          int pass, long long n, unsigned D, int moves_before, bool last,
                                          unsigned h_pass, long long spin_limit, int nblk) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool from_records = moves_before == 0;
    // (selects, not an indexed load: the parameter arrays stay in registers)
    const int src = (moves_before - 1) & 1, dst_buf = moves_before & 1;
    const K* __restrict__ kin = reinterpret_cast<const K*>(src ? sb.keys[1] : sb.keys[0]);
    const unsigned* __restrict__ vin = src ? sb.vals[1] : sb.vals[0];
    K* kout = reinterpret_cast<K*>(dst_buf ? sb.keys[1] : sb.keys[0]);
    unsigned* vout = dst_buf ? sb.vals[1] : sb.vals[0];
    K* skeys = reinterpret_cast<K*>(sm.keys);
    unsigned* groups = sb.group_counts + (long long)pass * sb.groups * kDigits;
    unsigned long long* published = ctrl + (kSortTicket + pass) * kCtrlStride;
    {
        const unsigned st = scan_digits(tid < kDigits ? h_pass : 0u, sm.warp_sum);
        if (tid < kDigits) sm.start[tid] = st;
        if (tid == 0) sm.fail = 0;
    }
    const long long n_tiles = (n + kSortTile - 1) / kSortTile;
    const unsigned lt = (1u << lane) - 1u;
    for (long long tile = blockIdx.x; tile < n_tiles; tile += nblk) {
        const long long t0 = tile * kSortTile;
        const int tn = (int)(n - t0 < kSortTile ? n - t0 : kSortTile);
        for (int i = tid; i < kSortWarps * kDigits; i += kSortBlock) (&sm.wcount[0][0])[i] = 0;
        __syncthreads();
        // warp w ranks the keys [t0 + w * 32 * kSortItems, + 32 * kSortItems):
        // item i of lane l is key i * 32 + l of that run, so the ranks follow key order
        const long long run = t0 + (long long)warp * 32 * kSortItems;
        K k[kSortItems];
        unsigned v[kSortItems];
#pragma unroll
        for (int i = 0; i < kSortItems; ++i) {
            const long long idx = run + i * 32 + lane;
            k[i] = 0;
            v[i] = 0;
            if (idx < n) {
                if (from_records) {
                    const int2 m = __ldcg(in.meta + idx);
                    k[i] = (K)pack_key((unsigned)(__ldg(root_prefix + m.y) + m.x), __ldcg(in.path + idx), D);
                    v[i] = (unsigned)idx;
                } else {
                    k[i] = __ldcg(kin + idx);
                    v[i] = __ldcg(vin + idx);
                }
            }
        }
        unsigned short* wc = sm.wcount[warp];
        unsigned rank[kSortItems];
#pragma unroll
        for (int i = 0; i < kSortItems; ++i) {
            const bool valid = run + i * 32 + lane < n;
            const unsigned d = digit_of(k[i], pass);
            const unsigned peers = match_digit(d, valid);
            const unsigned before = valid ? wc[d] : 0u;
            rank[i] = before + (unsigned)__popc(peers & lt);
            __syncwarp();
            if (valid && (peers & lt) == 0) wc[d] = (unsigned short)(before + (unsigned)__popc(peers));
            __syncwarp();
        }
        __syncthreads();
        // thread d: the warps' offsets within digit d's run of the tile, the
        // tile's count of d (published), and the tile's digit starts
        unsigned tot = 0;
        if (tid < kDigits) {
#pragma unroll
            for (int w = 0; w < kSortWarps; ++w) {
                const unsigned c = sm.wcount[w][tid];
                sm.wcount[w][tid] = (unsigned short)tot;
                tot += c;
            }
            sb.counts[tile * kDigits + tid] = tot;
            if (tot) atomicAdd(groups + (tile / kSortGroup) * kDigits + tid, tot);
            __threadfence();
        }
        const unsigned ts = scan_digits(tot, sm.warp_sum);
        if (tid == 0) {
            // publish (every count above is fenced before the barrier in scan_digits)
            __threadfence();
            atomicAdd(published, 1ull);
        }
        if (tid < kDigits) sm.tstart[tid] = ts;
        __syncthreads();
        // the tile in digit order, in shared memory
#pragma unroll
        for (int i = 0; i < kSortItems; ++i) {
            if (run + i * 32 + lane < n) {
                const unsigned d = digit_of(k[i], pass);
                const unsigned local = sm.tstart[d] + sm.wcount[warp][d] + rank[i];
                skeys[local] = k[i];
                sm.vals[local] = v[i];
            }
        }
        if (tid == 0) {
            // wait until every tile up to the end of this round has published
            const long long round_end = (tile / nblk + 1) * nblk;
            const unsigned long long need = (unsigned long long)(round_end < n_tiles ? round_end : n_tiles);
            long long spins = 0;
            while (ld_acquire_u64(published) < need) {
                if (++spins > spin_limit) {
                    sm.fail = 1;
                    break;
                }
                __nanosleep(64);
            }
            __threadfence();
        }
        __syncthreads();
        if (sm.fail) {
            // a wait ran out: report it and write nothing with a wrong base
            if (tid == 0) set_status(ctrl, kErrTimeout);
            return false;
        }
        {
            // counts of the earlier tiles, digit d: thread d adds the whole
            // groups before this tile's group, thread d + 256 the earlier
            // tiles of its own group
            const int d = tid & (kDigits - 1);
            const long long g = tile / kSortGroup;
            unsigned sum = 0;
            if (tid < kDigits) {
                for (long long j = 0; j < g; j += 16) {
                    unsigned x[16];
#pragma unroll
                    for (int u = 0; u < 16; ++u) x[u] = j + u < g ? __ldcg(groups + (j + u) * kDigits + d) : 0u;
#pragma unroll
                    for (int u = 0; u < 16; ++u) sum += x[u];
                }
            } else {
                for (long long j = g * kSortGroup; j < tile; j += 16) {
                    unsigned x[16];
#pragma unroll
                    for (int u = 0; u < 16; ++u) x[u] = j + u < tile ? __ldcg(sb.counts + (j + u) * kDigits + d) : 0u;
#pragma unroll
                    for (int u = 0; u < 16; ++u) sum += x[u];
                }
                sm.part[d] = sum;
            }
            __syncthreads();
            if (tid < kDigits) sm.base[d] = sm.start[d] + sum + sm.part[d];
            __syncthreads();
        }
        // each digit's run of the tile to consecutive addresses
        if (last) {
            // the records, gathered two at a time with their loads issued together
            constexpr int kBatch = 2;
            for (int j0 = tid; j0 < tn; j0 += kBatch * kSortBlock) {
                float4 rg[kBatch];
                int2 mt[kBatch];
                long long dst[kBatch];
#pragma unroll
                for (int u = 0; u < kBatch; ++u) {
                    const int j = j0 + u * kSortBlock;
                    dst[u] = -1;
                    if (j < tn) {
                        const unsigned d = digit_of(skeys[j], pass);
                        const long long o = (long long)sm.base[d] + (j - (int)sm.tstart[d]);
                        const unsigned sv = sm.vals[j];
                        if (o < n && o < out.capacity && sv < (unsigned)n) {
                            dst[u] = o;
                            rg[u] = __ldcg(in.range + sv);
                            mt[u] = __ldcg(in.meta + sv);
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < kBatch; ++u)
                    if (dst[u] >= 0) {
                        out.range[dst[u]] = rg[u];
                        out.meta[dst[u]] = mt[u];
                    }
            }
        } else {
            for (int j = tid; j < tn; j += kSortBlock) {
                const K key = skeys[j];
                const unsigned d = digit_of(key, pass);
                const long long dst = (long long)sm.base[d] + (j - (int)sm.tstart[d]);
                if (dst < n) {
                    kout[dst] = key;
                    vout[dst] = sm.vals[j];
                }
            }
        }
        __syncthreads();
    }
    return true;
}

// The whole sort in one launch of a resident grid (see the file header).
// A tile's start in digit bin d is the bin's start plus the counts of the
// earlier tiles, read as the sums of whole groups of kSortGroup tiles
// (accumulated as tiles publish) and the single counts of its own group's
// earlier tiles.
__global__ void __launch_bounds__(kSortBlock, 2) sort_kernel(const int* __restrict__ root_prefix, SubPatches in,
                                                             SubPatches out, SortBuffers sb, unsigned long long* ctrl,
                                                             int n_passes, long long spin_limit) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PassSmem& sm = *reinterpret_cast<PassSmem*>(smem_raw);
    __shared__ int s_flag;
    const int tid = threadIdx.x, lane = tid & 31;
    const long long n = sort_count(ctrl, in, sb);
    const unsigned epoch = frame_epoch(ctrl);
    unsigned D = 0;
    const int bits = key_bits(ctrl, &D);
    const int active = (bits + 7) / 8 < n_passes ? (bits + 7) / 8 : n_passes;
    unsigned* hist = hist_of(sb, epoch);
    // the working blocks: one per tile of this frame's keys, at most the
    // grid (a small frame leaves most of the resident grid idle); the others
    // return at once and every barrier counts the working blocks only
    const long long tiles = (n + kSortTile - 1) / kSortTile;
    const int nblk = (int)(tiles < 1 ? 1 : tiles < gridDim.x ? tiles : gridDim.x);
    if ((int)blockIdx.x >= nblk) return;
    {
        // counts: of this block's stripe of keys into shared memory (the
        // front of the pass buffers), then into the frame's table; the next
        // frame's table, the group counts and the passes' published-tile
        // counters are cleared for later
        unsigned* s_hist = reinterpret_cast<unsigned*>(smem_raw);
        for (int i = tid; i < kSortPasses * kDigits; i += kSortBlock) s_hist[i] = 0;
        unsigned* next = hist_of(sb, epoch + 1);
        const long long gt = (long long)blockIdx.x * kSortBlock + tid, gstride = (long long)nblk * kSortBlock;
        for (long long i = gt; i < kSortPasses * kDigits; i += gstride) next[i] = 0;
        for (long long i = gt; i < kSortPasses * sb.groups * kDigits; i += gstride) sb.group_counts[i] = 0;
        if (blockIdx.x == 0 && tid < kSortPasses) ctrl[(kSortTicket + tid) * kCtrlStride] = 0;
        __syncthreads();
        const unsigned lt = (1u << lane) - 1u;
        // whole warps step together so that the warp matches below see every lane
        for (long long base = (long long)blockIdx.x * kSortBlock + (tid & ~31); base < n; base += gstride) {
            const long long i = base + lane;
            const bool valid = i < n;
            unsigned long long key = 0;
            if (valid) {
                const int2 m = __ldcg(in.meta + i);
                key = pack_key((unsigned)(__ldg(root_prefix + m.y) + m.x), __ldcg(in.path + i), D);
            }
            for (int p = 0; p < active; ++p) {
                const unsigned d = digit_of(key, p);
                const unsigned peers = match_digit(d, valid);
                if (valid && (peers & lt) == 0) atomicAdd(&s_hist[p * kDigits + d], (unsigned)__popc(peers));
            }
        }
        __syncthreads();
        for (int i = tid; i < active * kDigits; i += kSortBlock) {
            const unsigned v = s_hist[i];
            if (v) atomicAdd(hist + i, v);
        }
    }
    unsigned long long barrier = 0;
    if (!grid_barrier(ctrl, ++barrier, nblk, spin_limit, &s_flag)) return;
    // plan: a pass moves keys unless one digit holds them all
    int moving = 0;
    unsigned moves_mask = 0;
#pragma unroll 1
    for (int q = 0; q < active; ++q) {
        const unsigned hq = tid < kDigits ? __ldcg(hist + q * kDigits + tid) : 0u;
        if (!__syncthreads_or(tid < kDigits && (long long)hq == n)) {
            moves_mask |= 1u << q;
            ++moving;
        }
    }
    if (moving == 0) {
        // no pass moves anything (n <= 1): the records are already in order
        const long long stride = (long long)nblk * kSortBlock;
        for (long long j = (long long)blockIdx.x * kSortBlock + tid; j < n && j < out.capacity; j += stride) {
            out.range[j] = in.range[j];
            out.meta[j] = in.meta[j];
        }
        return;
    }
    int before = 0;
#pragma unroll 1
    for (int q = 0; q < active; ++q) {
        if (!((moves_mask >> q) & 1u)) continue;
        const unsigned hq = tid < kDigits ? __ldcg(hist + q * kDigits + tid) : 0u;   // thread d: count of digit d
        const bool last = before == moving - 1;
        bool ok;
        if (bits <= 32)
            ok = pass_body<unsigned>(sm, root_prefix, in, out, sb, ctrl, q, n, D, before, last, hq, spin_limit, nblk);
        else
            ok = pass_body<unsigned long long>(sm, root_prefix, in, out, sb, ctrl, q, n, D, before, last, hq,
                                               spin_limit, nblk);
        if (!ok) return;
        // the next pass reads what every block of this one wrote
        if (!last && !grid_barrier(ctrl, ++barrier, nblk, spin_limit, &s_flag)) return;
        ++before;
    }
}

int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

}  // namespace

long long sort_tiles(long long n) { return (n + kSortTile - 1) / kSortTile; }

int canonical_sort_passes(int max_split_depth, long long roots) {
    // leaves lie at depth <= max_split_depth + 1; a path keeps 32 bits
    const int path_bits = max_split_depth + 1 < 32 ? max_split_depth + 1 : 32;
    int root_bits = 0;
    while (root_bits < 32 && ((roots - 1) >> root_bits) > 0) ++root_bits;
    const int bits = path_bits + root_bits;
    return bits <= 8 ? 1 : (bits + 7) / 8;
}

int canonical_sort_grid() {
    // blocks resident at once (the grid barriers and round waits rely on it)
    cudaFuncSetAttribute(sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(PassSmem));
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sort_kernel, kSortBlock, sizeof(PassSmem));
    return sm_count() * (per_sm < 1 ? 1 : per_sm);
}

void launch_canonical_sort(const int* root_prefix, const SubPatches& in, const SubPatches& out, const SortBuffers& sb,
                           unsigned long long* ctrl, long long spin_limit, int n_passes, int resident_grid,
                           cudaStream_t s) {
    const long long tiles = sb.tiles < 1 ? 1 : sb.tiles;
    const int grid = (int)(tiles < resident_grid ? tiles : resident_grid);
    sort_kernel<<<grid, kSortBlock, sizeof(PassSmem), s>>>(root_prefix, in, out, sb, ctrl, n_passes, spin_limit);
}

}  // namespace mp
