// mp_inclusive_scan_noalloc: the decoupled look-back prefix sum for callers
// that may not allocate device memory.
//
// Some callers cannot call cudaMalloc or cudaFree at the moment they need a
// prefix sum: a real-time render loop with a fixed device-memory budget, where
// cudaFree would synchronize the whole device in the middle of a frame, or a
// host that owns every device allocation through its own allocator.  This
// entry point takes device input and output buffers from the caller and keeps
// its only scratch -- the per-tile look-back states, the tile ticket and a
// status word -- in a file-scope __device__ array of fixed size, so it
// allocates nothing.
//
// Limits and sharing: at most kNoAllocMaxElements elements per call.  The
// array exists once per device that loads the library and lives until the
// process exits.  Every call on a device uses the same array and leaves its
// contents behind, so the states the scan relies on are cleared at the start
// of each call, and calls whose work overlaps on the GPU (two streams, or two
// host threads) race on the array and must be serialized by the caller.
//
// Device address: in host code the array's name is only a host-side handle,
// so its device address is looked up with cudaGetSymbolAddress once per
// device, with that device current, by the first call made on that device.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/mp_core.h"

namespace {

constexpr int kNoAllocBlock = 256;
constexpr int kNoAllocItems = 4;
constexpr int kNoAllocTileItems = kNoAllocBlock * kNoAllocItems;
constexpr long long kNoAllocMaxElements = 1ll << 22;  // 4,194,304 int32 values
constexpr int kNoAllocMaxTiles = (int)(kNoAllocMaxElements / kNoAllocTileItems);
constexpr int kWordTicket = kNoAllocMaxTiles;       // tile ticket counter
constexpr int kWordStatus = kNoAllocMaxTiles + 1;   // 0 ok, else mp_status
constexpr int kScratchWords = kNoAllocMaxTiles + 32;
constexpr long long kNoAllocSpinLimit = 1ll << 20;  // bounded look-back wait

constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagPrefix = 2ull << 62;
constexpr unsigned long long kValMask = (1ull << 62) - 1;

// 4,128 words = 33 KB per device.
static __device__ __align__(256) unsigned long long g_noalloc_scan_scratch[kScratchWords];

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Clears the states of the tiles this call uses, the ticket and the status.
__global__ void noalloc_reset_kernel(unsigned long long* scratch, int n_tiles) {
    for (int i = threadIdx.x; i < n_tiles; i += blockDim.x) scratch[i] = 0;
    if (threadIdx.x == 0) {
        scratch[kWordTicket] = 0;
        scratch[kWordStatus] = 0;
    }
}

// Inclusive prefix sum of int32 values (sums wrap modulo 2^32 like int32
// arithmetic), single pass with decoupled look-back over 1,024-element tiles.
__global__ void __launch_bounds__(kNoAllocBlock) noalloc_scan_kernel(const int* __restrict__ in, int* out,
                                                                     long long n, unsigned long long* scratch) {
    __shared__ unsigned long long s_items[kNoAllocTileItems];
    __shared__ unsigned long long s_warp[kNoAllocBlock / 32];
    __shared__ unsigned long long s_prefix;
    __shared__ int s_tile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_tile = (int)atomicAdd(scratch + kWordTicket, 1ull);
    __syncthreads();
    const int tile = s_tile;
    const long long base = (long long)tile * kNoAllocTileItems;
    for (int k = 0; k < kNoAllocItems; ++k) {
        const long long idx = base + k * kNoAllocBlock + tid;
        s_items[k * kNoAllocBlock + tid] = idx < n ? (unsigned long long)(unsigned)in[idx] : 0ull;
    }
    __syncthreads();
    unsigned long long v[kNoAllocItems];
    unsigned long long tsum = 0;
    for (int k = 0; k < kNoAllocItems; ++k) {
        v[k] = s_items[tid * kNoAllocItems + k];
        tsum += v[k];
    }
    unsigned long long x = tsum;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < kNoAllocBlock / 32 ? s_warp[lane] : 0ull;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kNoAllocBlock / 32) s_warp[lane] = w;
    }
    __syncthreads();
    const unsigned long long thread_excl = (warp == 0 ? 0ull : s_warp[warp - 1]) + x - tsum;
    const unsigned long long agg = s_warp[kNoAllocBlock / 32 - 1] & kValMask;
    if (tid == 0) {
        unsigned long long prefix = 0;
        if (tile == 0) {
            st_release(scratch + 0, kFlagPrefix | agg);
        } else {
            st_release(scratch + tile, kFlagAgg | agg);
            long long spins = 0;
            for (int pred = tile - 1; pred >= 0;) {
                const unsigned long long s = ld_acquire(scratch + pred);
                const unsigned long long flag = s & ~kValMask;
                if (flag == 0) {
                    if (++spins > kNoAllocSpinLimit) {
                        atomicCAS(scratch + kWordStatus, 0ull, (unsigned long long)MP_ERR_TIMEOUT);
                        break;
                    }
                    __nanosleep(64);
                    continue;
                }
                prefix += s & kValMask;
                if (flag == kFlagPrefix) break;
                --pred;
            }
            st_release(scratch + tile, kFlagPrefix | ((prefix + agg) & kValMask));
        }
        s_prefix = prefix;
    }
    __syncthreads();
    unsigned long long run = s_prefix + thread_excl;
    for (int k = 0; k < kNoAllocItems; ++k) {
        run += v[k];
        s_items[tid * kNoAllocItems + k] = run;
    }
    __syncthreads();
    for (int k = 0; k < kNoAllocItems; ++k) {
        const long long idx = base + k * kNoAllocBlock + tid;
        if (idx < n) out[idx] = (int)(unsigned)s_items[k * kNoAllocBlock + tid];
    }
}

// Device address of the scratch array, looked up once per device.
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned long long* g_scratch_dev[kMaxDevices] = {};

cudaError_t scratch_address(int device, unsigned long long** out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_dev[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scan_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_dev[device] = static_cast<unsigned long long*>(p);
    }
    *out = g_scratch_dev[device];
    return cudaSuccess;
}

}  // namespace

extern "C" mp_status mp_inclusive_scan_noalloc(const int32_t* in_dev, int32_t* out_dev, int64_t n, void* stream) {
    if (n < 0 || n > kNoAllocMaxElements) return MP_ERR_INVALID_ARG;
    if (n == 0) return MP_OK;
    if (!in_dev || !out_dev) return MP_ERR_INVALID_ARG;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) return MP_ERR_CUDA;
    unsigned long long* scratch = nullptr;
    if (scratch_address(device, &scratch) != cudaSuccess) {
        cudaGetLastError();
        return MP_ERR_CUDA;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int tiles = (int)((n + kNoAllocTileItems - 1) / kNoAllocTileItems);
    // an error left by the caller's earlier work stays the caller's: only a
    // launch error of this call (which replaces it) is reported, and cleared
    const cudaError_t before = cudaPeekAtLastError();
    noalloc_reset_kernel<<<1, 256, 0, s>>>(scratch, tiles);
    noalloc_scan_kernel<<<tiles, kNoAllocBlock, 0, s>>>(in_dev, out_dev, n, scratch);
    const cudaError_t after = cudaPeekAtLastError();
    if (after != cudaSuccess && after != before) {
        cudaGetLastError();
        return MP_ERR_CUDA;
    }
    unsigned long long status = 0;
    if (cudaMemcpyAsync(&status, scratch + kWordStatus, sizeof(status), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        return MP_ERR_CUDA;
    }
    return status == 0 ? MP_OK : (mp_status)status;
}
