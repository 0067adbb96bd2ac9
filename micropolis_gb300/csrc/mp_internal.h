// Internal interface between the C-ABI host layer (mp_host.cu) and the
// kernel translation units.  Not part of the public ABI.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "mp_device.cuh"

namespace mp {

// Control words of one frame, each on its own 128-byte line so that the hot
// atomics of different roles land in different L2 slices.
enum CtrlWord {
    kQTail = 0,        // queue tickets ever filled (virtual roots included)
    kQHead,            // queue tickets handed out
    kOutstanding,      // items pushed but not finished
    kOutCount,         // sub-patches emitted
    kDone,             // bound-and-split finished
    kStatus,           // first error code (mp_status values)
    kEpoch,            // frame number, marks queue slots written this frame
    kRoots,            // number of root items (all draws' patches)
    kBigCount,         // quads routed to the exact slow raster path
    kFragments,        // covered (micropolygon, pixel) pairs
    kScanTile,         // tile ticket of the decoupled look-back scan
    kScanTotal,        // packed totals of the last scan (draws | splits << 32)
    kBigOverflow,      // big quads that did not fit
    kBigTotal,         // big quads rasterized over the frame
    kGroupTicket,      // sub-patch groups claimed by the frame kernel's rasterizers
    kMaxDepth,         // deepest split path of an emitted sub-patch (canonical sort keys)
    kSortTicket,       // tile tickets of the canonical sort, one word per radix pass (kSortPasses)
    kSortDone = kSortTicket + 8,   // grid-barrier arrivals of the sort kernel this frame
    kNumCtrl
};
constexpr int kCtrlStride = 16;  // unsigned long long words per line

struct Queue {              // bound-and-split work queue (structure of arrays)
    float4* range;          // (min.x, min.y, max.x, max.y)
    uint2* meta;            // (patch id, draw | depth << 24)
    unsigned* seq;          // epoch of the frame that wrote the slot
    // kPtsPerSlot float4 per slot: six of the item's nine bound samples, taken
    // from its parent, and which three are missing (or nullptr: none kept)
    float4* pts;
    // split path of each range: bit 31 - d is 1 when the range is the high
    // half of its depth-d ancestor's split (nullptr: not kept)
    unsigned* path;
    long long capacity;
};

struct SubPatches {         // emitted sub-patch list
    float4* range;
    int2* meta;             // (patch id, draw)
    long long capacity;
    unsigned* seq;          // epoch of the frame that emitted the slot (frame kernel only)
    unsigned* path;         // split path (Queue::path) of each sub-patch (nullptr: not kept)
};

// Canonical order of a frame's sub-patches: ascending (root, split path),
// root = the draw's first root + patch id.  Scratch of the radix sort that
// establishes it (mp_sort.cu).
constexpr int kSortPasses = 8;          // 8-bit digits of the 64-bit key
struct SortBuffers {
    unsigned long long* keys[2];        // ping-pong keys
    unsigned* vals[2];                  // ping-pong source slots
    unsigned* hist;                     // 2 (frame parity) x kSortPasses x 256 digit counts
    unsigned* counts;                   // per pass: digit counts of each tile, tiles x 256
    unsigned* group_counts;             // kSortPasses x groups x 256: counts of groups of kSortGroup tiles
    long long capacity;                 // keys per buffer
    long long tiles;                    // tiles at capacity
    long long groups;                   // tile groups at capacity
};
constexpr int kSortGroup = 32;          // tiles per group of the pass's prefix

struct BigQuad {            // a quad rasterized by the exact tile emulation
    int px[4], py[4];
    float depth[4];
    unsigned mp_id;
    int view;
    int tile[4];            // block tile range (min x, min y, max x, max y)
};

struct Framebuffer {
    unsigned long long* keys;   // (idepth << 32 | mp_id) per pixel, tiled, per view
    float4* color;              // tiled colour, per view
    int* depth;                 // tiled int depth, per view
    long long pixels;           // W * H (colour / depth per view)
    long long key_pixels;       // key buffer per view (whole key tiles)
    int views;
};

// status codes shared with the public header
enum { kOk = 0, kErrInvalidArg = 1, kErrOutOfMemory = 2, kErrOverflow = 3, kErrTimeout = 4, kErrCuda = 5 };

// ---- bound-and-split (mp_bns.cu)
void launch_bns_persistent(const DrawDev* draws, const int* root_prefix, int n_draws, const FrameDev& fr,
                           const Queue& q, const SubPatches& out, unsigned long long* ctrl, int grid,
                           long long spin_limit, cudaStream_t s);
int bns_persistent_grid(int criterion);
// plain per-pass bound-and-split (the reference's BOUNDED structure)
void launch_bns_init_stack(const Queue& stack, int draw, int n_patches, cudaStream_t s);
void launch_bns_pass(const DrawDev* draws, const FrameDev& fr, const Queue& stack, long long offset, int batch,
                     float4* pad_range, uint2* pad_meta, unsigned char* dec, unsigned long long* keys,
                     unsigned long long* scan_state, const SubPatches& out, long long out_base,
                     unsigned long long* ctrl, long long spin_limit, cudaStream_t s);
void launch_inclusive_scan_i32(const int* in, int* out, long long n, unsigned long long* scan_state,
                               unsigned long long* ctrl, long long spin_limit, cudaStream_t s);
long long scan_state_words(long long n);

// ---- canonical sub-patch order (mp_sort.cu)
long long sort_tiles(long long n);
// Sorts the n_out (device count kOutCount) sub-patches of `in` by (root,
// path) and gathers them into `out`; root_prefix as for bound-and-split.
// One launch; the keys have at most n_passes 8-bit digits (a pass whose digit
// is the same for every key of the frame is skipped).
void launch_canonical_sort(const int* root_prefix, const SubPatches& in, const SubPatches& out, const SortBuffers& sb,
                           unsigned long long* ctrl, long long spin_limit, int n_passes, int resident_grid,
                           cudaStream_t s);
// Blocks of the sort kernel resident at once (also sets its shared memory
// size; call outside stream capture).
int canonical_sort_grid();
// The radix passes the keys of a frame can need: root bits up to `roots`
// above at most min(32, max_split_depth + 1) path bits.
int canonical_sort_passes(int max_split_depth, long long roots);

// ---- dice / shade / raster / resolve (mp_raster.cu)
// clears the key buffer (and with_color: colour and depth); with reset_ctrl,
// also resets the frame's bound-and-split control words for `roots` roots
void launch_clear(const Framebuffer& fb, const FrameDev& fr, int with_color, cudaStream_t s,
                  unsigned long long* reset_ctrl = nullptr, long long roots = 0);
void launch_raster_fused(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, const Framebuffer& fb,
                         float* mshade, BigQuad* big, long long big_cap, unsigned long long* ctrl, int grid, int group,
                         cudaStream_t s);
int raster_fused_grid(int PS, int group);
// bound-and-split and rasterization overlapped in one launch: the first
// n_bns_ctas blocks run bound-and-split, then every block consumes emitted
// sub-patches as they become ready
void launch_frame_kernel(const DrawDev* draws, const int* root_prefix, int n_draws, const FrameDev& fr, const Queue& q,
                         const SubPatches& sub, const Framebuffer& fb, float* mshade, BigQuad* big, long long big_cap,
                         unsigned long long* ctrl, long long spin_limit, int grid, int n_bns_ctas, int group,
                         cudaStream_t s);
int frame_kernel_grid(int PS, int group);
void launch_raster_big(const DrawDev* draws, const FrameDev& fr, const Framebuffer& fb, const BigQuad* big,
                       long long big_cap, unsigned long long* ctrl, cudaStream_t s);
void launch_resolve(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, const Framebuffer& fb,
                    const float* mshade, cudaStream_t s);
// plain per-pass path
void launch_dice_grid(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, long long base, int count,
                      float4* pos, int2* pxl, float* depth, cudaStream_t s);
void launch_shade_grid(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, long long base, int count,
                       const float4* pos, const int2* pxl, int4* block_index, float4* color, cudaStream_t s);
void launch_sample_grid(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, long long base, int count,
                        const int4* block_index, const int2* pxl, const float* depth, const Framebuffer& fb,
                        BigQuad* big, long long big_cap, unsigned long long* ctrl, cudaStream_t s);
void launch_pass_resolve(const FrameDev& fr, const Framebuffer& fb, long long base, int count, const float4* color,
                         cudaStream_t s);
// dice positions of given sub-patches (parity checks)
void launch_dice_debug(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, int count, float4* pos,
                       int2* pxl, float* depth, cudaStream_t s);

// ---- adjoint (mp_adjoint.cu)
void launch_adjoint(const DrawDev* draws, const FrameDev& fr, const SubPatches& sub, const Framebuffer& fb,
                    const float4* grad_color, float* grad_amp, int view, cudaStream_t s);

// ---- microbenchmark (mp_raster.cu)
void launch_image(const float4* color, const FrameDev& fr, unsigned char* rgb, cudaStream_t s);
// (x, y, z) -> (x, y, z, 1) for n points (src/Reyes/PatchIndex.cpp:83-98)
void launch_widen_points(const float* xyz, float4* out, long long n, cudaStream_t s);
void launch_atomic_bench(unsigned long long* buf, long long n_slots, long long n_ops, int pattern, cudaStream_t s);

}  // namespace mp
