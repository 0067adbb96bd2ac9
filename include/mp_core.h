/*
 * mp_core.h -- C ABI of the GB300 REYES core (libmpcore.so).
 *
 * Drop-in for the reference's renderer boundary, the abstract Reyes::Renderer
 * (src/Reyes/Renderer.h:29-45) and its OpenCL implementation RendererCL
 * (src/Reyes/RendererCL.cpp:115-260).  Plain pointers and sizes only; every
 * call returns an mp_status and never throws.  One context per host thread;
 * all device work of a context runs on its CUDA stream.
 */
#ifndef MP_CORE_H
#define MP_CORE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes.  The reference signals errors with C++ exceptions
 * (CL::Exception via OPENCL_ASSERT, src/CL/Exception.h) and assert(); here
 * every entry point returns one of these and mp_last_error() gives the text. */
typedef enum {
    MP_OK = 0,
    MP_ERR_INVALID_ARG = 1,  /* bad option, handle, size or pointer */
    MP_ERR_OUT_OF_MEMORY = 2,
    MP_ERR_OVERFLOW = 3,     /* a queue or output capacity was exceeded and could not grow */
    MP_ERR_TIMEOUT = 4,      /* a bounded device wait gave up (no GPU hang) */
    MP_ERR_CUDA = 5,         /* a CUDA runtime call failed */
    MP_ERR_NOT_LOADED = 6,   /* draw of a handle with no loaded patches */
    MP_ERR_STATE = 7         /* call out of order (e.g. draw before prepare) */
} mp_status;

/* src/Reyes/PatchType.h:6-9 */
typedef enum { MP_BEZIER = 0, MP_GREGORY = 1 } mp_patch_type;

/* Execution path of a frame. */
typedef enum {
    MP_PATH_PLAIN = 0,   /* per-pass: bound&split up to reyes_patches_per_pass, then dice,
                            shade, sample with grids in device memory, host sync per pass */
    MP_PATH_BATCHED = 1  /* one persistent launch per stage over all draws of the frame,
                            replayed as a CUDA graph; no grids stored */
} mp_path;

/* Options, named as in the reference's reyes.options (values there are the
 * defaults filled by mp_options_default). */
/* Which bound criterion bound-and-split applies. */
typedef enum {
    /* the reference's CPU bound-and-split (src/Reyes/BoundNSplitCLCPU.cpp:117-148):
     * eye-space 3x3 bbox projected by Projection::bound, strict < limit, split
     * the direction with the longer eye-space arc length; the default, and the
     * one the sub-patch set is bit-exact to */
    MP_BOUND_CPU = 0,
    /* the reference's GPU criterion (kernels/bound_n_split.h:43-100, used by
     * its BOUNDED / LOCAL / BREADTH methods): screen-projected sample arc
     * lengths with <=, the eye-plane split rule, far cull at 1000, cull at
     * depth >= max_split_depth - 1; kernel arithmetic (R1-R6) */
    MP_BOUND_GPU = 1
} mp_bound_criterion;

typedef struct {
    int32_t window_size[2];         /* framebuffer size; multiples of 8, at most 4096 */
    int32_t reyes_patch_size;       /* dice grid: 8 or 16 quads per side */
    float bound_n_split_limit;      /* pixels */
    int32_t reyes_patches_per_pass; /* plain path pass size */
    float cull_ribbon;              /* pixels */
    int32_t max_split_depth;        /* at most 254 */
    int32_t bound_sample_rate;      /* must be 3 (the CPU criterion samples 3x3) */
    int32_t subpixel_bits;          /* fixed-point bits of pixel coordinates (1..8) */
    int32_t framebuffer_tile_size;  /* must be 8 (the sample kernel's tile) */
    int32_t backface_culling;
    int32_t displacement;
    float displacement_amplitude;   /* multiplies the hard-coded 0.04/0.02/0.01 */
    float clear_color[4];
    int32_t batch_views;            /* framebuffer layers (independent views) */
    int32_t path;                   /* mp_path */
    /* capacities (elements); 0 = automatic.  They grow on overflow. */
    int64_t queue_capacity;         /* bound&split work items */
    int64_t subpatch_capacity;      /* emitted sub-patches per frame */
    int64_t spin_limit;             /* bounded-wait iterations before MP_ERR_TIMEOUT */
    /* batched path: run bound&split and rasterization in one launch that
     * rasterizes sub-patches while they are being emitted (1) or as separate
     * launches (0, the default).  With 1 the sub-patches keep the order in
     * which they were emitted, which depends on scheduling, so the winner
     * between two equally deep micropolygons can differ between runs; with 0
     * they are put in the canonical order first (see mp_subpatches).
     * bns_blocks = blocks that start with bound&split (0 = auto) */
    int32_t overlap;
    int32_t bns_blocks;
    /* tuning knobs that do not change the image (0 = default):
     * raster_tile: tile of the depth|id key buffer in pixels (8, 16, 32);
     * dice_group: sub-patches diced together per block (8, 11, 16 or 22
     * at reyes_patch_size 8; 2, 3, 4 or 6 at 16; 11 and 3 run 128-thread
     * blocks, the others 256) */
    int32_t raster_tile;
    int32_t dice_group;
    /* bound-and-split criterion (mp_bound_criterion) */
    int32_t bound_criterion;
} mp_options;

/* The reference's Projection(fovy, near, viewport) (src/base/Projection.h:144). */
typedef struct {
    float fovy_deg;
    float near_plane;
    int32_t viewport[2];            /* must equal window_size */
} mp_projection;

typedef struct {
    int64_t subpatches;             /* emitted sub-patches of the last frame */
    int64_t micropolygons;          /* reyes_patch_size^2 * subpatches (src/base/Statistics.cpp:175) */
    int64_t bounds;                 /* ranges bounded by bound&split */
    int64_t passes;                 /* plain path passes */
    int64_t fragments;              /* covered (micropolygon, pixel) pairs */
    int64_t big_quads;              /* quads on the exact slow raster path */
    double gpu_ms;                  /* device time of the last frame (CUDA events) */
    /* per-stage device times of the last frame (batched path: always, from
     * events inside its graph; plain path: with stage timing on,
     * mp_set_stage_timing); stages: 0 clear+reset, 1 bound&split, 2 dice+raster
     * (plain: dice), 3 exact slow raster, 4 resolve (plain: shade), 5 canonical
     * order sort (plain: sample), 6 plain pass resolve, 7 plain host readback gaps */
    double stage_ms[8];
    int64_t kernels;                /* kernel launches of the last frame (graph nodes included) */
} mp_stats;

typedef struct mp_ctx mp_ctx;

/* Fills the reyes.options defaults. */
void mp_options_default(mp_options* opts);

/* Creates a context on the current CUDA device (replaces RendererCL::RendererCL,
 * src/Reyes/RendererCL.cpp:21-106). */
mp_status mp_create(const mp_options* opts, mp_ctx** out);
void mp_destroy(mp_ctx* ctx);
const char* mp_last_error(const mp_ctx* ctx);
/* Uses `stream` (a cudaStream_t) for all further work; NULL restores the context's own. */
mp_status mp_set_stream(mp_ctx* ctx, void* stream);

/* Renderer::are_patches_loaded (Renderer.h:35, PatchIndex.cpp:50-53). */
mp_status mp_are_patches_loaded(mp_ctx* ctx, uint64_t handle, int32_t* loaded);
/* Renderer::load_patches (Renderer.h:36, PatchIndex.cpp:57-100): copies n_points xyz
 * points (16 per Bezier, 20 per Gregory patch) to the device, widened to (x,y,z,1).
 * handle is an opaque key chosen by the caller (the reference uses the mesh pointer).
 * Returns once xyz has been read (the buffer may then be reused); the widening is
 * ordered before the frames on the context's stream. */
mp_status mp_load_patches(mp_ctx* ctx, uint64_t handle, const float* xyz, size_t n_points, mp_patch_type type);
/* Same, from device memory (float4 x,y,z,1 per point), no host copy. */
mp_status mp_load_patches_device(mp_ctx* ctx, uint64_t handle, const void* dev_xyz1, size_t n_points,
                                 mp_patch_type type);
/* PatchIndex::delete_patches (PatchIndex.cpp:103-108). */
mp_status mp_delete_patches(mp_ctx* ctx, uint64_t handle);

/* Renderer::prepare (RendererCL.cpp:115-135): begins a frame (clear colour ^2.2,
 * alpha 1000, depth 0x7fffffff). */
mp_status mp_prepare(mp_ctx* ctx);
/* Renderer::draw_patches (RendererCL.cpp:170-200): modelview is column-major
 * (glm layout), colour the object colour.  Draws into framebuffer layer 0. */
mp_status mp_draw_patches(mp_ctx* ctx, uint64_t handle, const float modelview[16], const mp_projection* proj,
                          const float color[4]);
/* Same, into framebuffer layer `view` (batched independent views). */
mp_status mp_draw_patches_view(mp_ctx* ctx, uint64_t handle, const float modelview[16], const mp_projection* proj,
                               const float color[4], int32_t view);

/* One draw of a batch: mesh handle, modelview, projection, colour, layer. */
typedef struct {
    uint64_t handle;
    float modelview[16];
    mp_projection proj;
    float color[4];
    int32_t view;
} mp_view;
/* n draws at once (mp_draw_patches_view for each, in order); stops at the
 * first error and returns it. */
mp_status mp_draw_views(mp_ctx* ctx, int32_t n, const mp_view* views);
/* Renderer::finish (RendererCL.cpp:138-154): completes the frame; the framebuffer
 * is ready when this returns. */
mp_status mp_finish(mp_ctx* ctx);
/* Stage timing: when on, the batched frame runs its stages as separate
 * launches with CUDA events between them instead of one graph replay, and
 * mp_stats.stage_ms is filled (for profiling; the graph replay is faster). */
mp_status mp_set_stage_timing(mp_ctx* ctx, int32_t on);
/* Renderer::dump_trace (Renderer.h:43): the last frame's device commands as
 * `name@queue:queued:submit:start:end:id:deps` lines (src/CL/Device.cpp:275-289),
 * times in ns from the start of the frame, deps '|'-separated ids, named with
 * the reference's command names (those its tools/trace_summary.py maps).
 * Batched path: one line per stage.  Plain path: one line per command of each
 * pass, with stage timing on (mp_set_stage_timing); without it the plain path
 * records no times and the call returns MP_ERR_STATE.  NUL-terminated;
 * MP_ERR_OVERFLOW when the text did not fit in cap bytes (buf then holds the
 * lines that fit). */
mp_status mp_dump_trace(mp_ctx* ctx, char* buf, size_t cap);

/* Headless framebuffer (replaces OGLSharedFramebuffer, src/Reyes/Framebuffer.cpp:75-144):
 * tiled float4 colour and int32 depth, 8x8-pixel tiles, index
 * (tx + ceil(W/8)*ty)*64 + lx + 8*ly (kernels/reyes.cl:37-45), one layer per view. */
mp_status mp_framebuffer(mp_ctx* ctx, void** color_dev, void** depth_dev, int32_t* width, int32_t* height,
                         int32_t* views);
/* Copies layer `view` to host memory; linear != 0 converts to row-major (y up). */
mp_status mp_read_framebuffer(mp_ctx* ctx, int32_t view, float* color_rgba, int32_t* depth, int32_t linear);

/* Read-back of layer `view` (tiled colour float4, depth int32) that overlaps
 * the frames rendered after it: the layer is copied on the device into a
 * staging layer of the context (on the context's stream, after the frame),
 * then to `color` / `depth` in host memory on a copy stream of its own, and
 * the call returns at once.  The host buffers should be page-locked
 * (cudaMallocHost / cudaHostRegister) for the copy to run asynchronously;
 * either pointer may be NULL.  mp_wait_read_framebuffer returns when the last
 * requested read-back is in host memory; the host buffers must not be read
 * or reused before then.  A new request first waits, on the device, until the
 * previous one has left the staging layer.  The first call allocates the
 * staging layer (20 bytes per pixel) and the copy stream.  The reference
 * reads its framebuffer back synchronously (src/Reyes/Framebuffer.cpp:102-124). */
mp_status mp_read_framebuffer_async(mp_ctx* ctx, int32_t view, float* color_rgba, int32_t* depth);
mp_status mp_wait_read_framebuffer(mp_ctx* ctx);

/* Copies layer `view` (tiled colour float4, depth int32) into device buffers on
 * the context's stream; either pointer may be NULL. */
mp_status mp_copy_framebuffer_device(mp_ctx* ctx, int32_t view, void* color_dev, void* depth_dev);
/* Winning micropolygon of every tiled pixel of layer `view` in the last frame:
 * sub-patch index * reyes_patch_size^2 + nu + nv * reyes_patch_size, or -1. */
mp_status mp_read_visibility(mp_ctx* ctx, int32_t view, int64_t* ids);
/* Sub-patches of the last frame, for parity checks: count, then up to cap records
 * (draw index, patch id, range min.x min.y max.x max.y).  Any pointer may be NULL.
 * Record s owns the micropolygon numbers s * reyes_patch_size^2 + nu + nv *
 * reyes_patch_size (mp_read_visibility).  On the batched path the records
 * are in the canonical order: ascending root (the draw's first patch, counted
 * over the frame's draws in call order, + patch id), then split path (the
 * patch's split tree depth first, low half before high half), the same on
 * every run; the reference's CPU bound-and-split emits the same set in its
 * stack order (src/Reyes/BoundNSplitCLCPU.cpp:75-159).  On the plain path they
 * are in pass order. */
mp_status mp_subpatches(mp_ctx* ctx, int64_t* count, int32_t* draw, int32_t* pid, float* range, int64_t cap);
mp_status mp_stats_get(mp_ctx* ctx, mp_stats* stats);

/* Dice grids of explicit sub-patches of the last frame's draw 0 mesh list
 * (parity of the dicer): positions (float4), fixed-point pixels (int2), depth. */
mp_status mp_dice_subpatches(mp_ctx* ctx, int32_t draw, int64_t n, const int32_t* pid, const float* range,
                             float* pos, int32_t* pxl, float* depth);

/* Adjoint of the last frame of layer `view`: grad_color (device, tiled float4 per
 * pixel, dL/dcolour) -> dL/d control points of every draw whose gradient buffer is
 * registered, and dL/d displacement amplitude (device float, accumulated).
 * Visibility is the last frame's. */
mp_status mp_set_grad_buffer(mp_ctx* ctx, int32_t draw, void* grad_dev);
mp_status mp_backward(mp_ctx* ctx, int32_t view, const void* grad_color_dev, void* grad_amp_dev);
/* Sets the displacement amplitude multiplier (the 0.04/0.02/0.01 amplitudes of
 * kernels/dice.cl:52-54 are scaled by it) for the following frames. */
mp_status mp_set_displacement_amplitude(mp_ctx* ctx, float amplitude);
/* Same, from one float in device memory, copied on the context's stream
 * (no host synchronization): the differentiable path's amplitude stays on
 * the device.  The reference fixes the amplitudes in the dice kernel
 * (kernels/dice.cl:52-54); the multiplier is this core's parameter. */
mp_status mp_set_displacement_amplitude_device(mp_ctx* ctx, const void* amp_dev);
/* Replaces the control points of a loaded handle in place from device memory (same count). */
mp_status mp_update_patches_device(mp_ctx* ctx, uint64_t handle, const void* dev_xyz1);

/* Inclusive prefix sum on the device (the decoupled look-back scan used by the
 * plain path; the reference's CL::PrefixSum, src/CL/PrefixSum.cpp:33-80). */
mp_status mp_inclusive_scan(mp_ctx* ctx, const int32_t* host_in, int32_t* host_out, int64_t n);

/* Inclusive prefix sum of n int32 values already in device memory, for callers
 * that may not allocate device memory (e.g. a render loop with a fixed device
 * budget, where cudaFree would stall the device mid-frame, or a host whose own
 * allocator owns all device memory).  Has no counterpart in the reference.
 * It allocates nothing: the caller passes input and output, and the scan's
 * scratch (33 KB of look-back state) is a fixed __device__ array of the
 * library.  n may be at most 4,194,304 (MP_ERR_INVALID_ARG beyond).  The
 * first call on a device looks up that array's device address, so make it
 * before any stream capture.  All calls on a device share the array: calls
 * that overlap on the GPU race and must be serialized by the caller.  Every
 * call is blocking: it runs on `stream` (a cudaStream_t, NULL = default
 * stream), then waits for that stream (cudaStreamSynchronize) and copies the
 * scan's status word to host memory before it returns (MP_ERR_TIMEOUT when a
 * bounded wait gave up). */
mp_status mp_inclusive_scan_noalloc(const int32_t* in_dev, int32_t* out_dev, int64_t n, void* stream);

/* The image the reference shows for one layer (shaders/tex_draw.frag: gamma
 * 1/2.2 on RGB, 8-bit window): W*H*3 bytes, RGB, top row first.  Replaces the
 * OpenGL presentation of OGLSharedFramebuffer::show (src/Reyes/Framebuffer.cpp)
 * with a host buffer. */
mp_status mp_read_image(mp_ctx* ctx, int32_t view, uint8_t* rgb);

/* Statistics of the last frame in the format of Statistics::dump_stats
 * (src/base/Statistics.cpp:196-217): "key = value;" lines.  Writes at most
 * cap bytes including the terminating zero; MP_ERR_OVERFLOW when truncated. */
mp_status mp_dump_stats(mp_ctx* ctx, char* buf, size_t cap);

/* ---- .mscene scene files (src/micropolis/mscene.capnp, Scene.cpp:89-197) ----
 * A scene read from the reference's Cap'n Proto packed file: meshes (name,
 * patch type, xyz positions), objects (name, mesh, transform, colour),
 * cameras (name, transform, near, far, fovy) and the number of lights.
 * Host memory only; no CUDA call. */
typedef struct mp_scene mp_scene;
/* Reads and decodes a packed .mscene file (Scene::Scene, Scene.cpp:89-173);
 * MP_ERR_INVALID_ARG for a file that is not a well-formed scene. */
mp_status mp_scene_load(const char* path, mp_scene** out);
/* The same from bytes in memory. */
mp_status mp_scene_parse(const uint8_t* data, size_t size, mp_scene** out);
void mp_scene_free(mp_scene* scene);
mp_status mp_scene_counts(const mp_scene* scene, int32_t* meshes, int32_t* objects, int32_t* cameras,
                          int32_t* lights);
/* Mesh i: its name, mp_patch_type and the flattened positions (3 floats per
 * point, 16 or 20 points per patch); pointers stay valid until mp_scene_free. */
mp_status mp_scene_mesh(const mp_scene* scene, int32_t i, const char** name, int32_t* type, const float** xyz,
                        int64_t* n_floats);
/* Object i: name, mesh index (-1 when no mesh has its mesh name), the
 * column-major matrix translate(t) * mat4_cast(rotation), colour (rgb, 1). */
mp_status mp_scene_object(const mp_scene* scene, int32_t i, const char** name, int32_t* mesh, float matrix[16],
                          float color[4]);
mp_status mp_scene_camera(const mp_scene* scene, int32_t i, const char** name, float matrix[16], float* near_plane,
                          float* far_plane, float* fovy_deg);
/* inverse(camera matrix) * object matrix (Scene.cpp:190). */
mp_status mp_scene_modelview(const mp_scene* scene, int32_t camera, int32_t object, float mv[16]);
/* Scene::draw (Scene.cpp:179-197) with camera `camera`: prepare, load each
 * object's mesh on first use (one handle per mesh of this scene), draw every
 * object, finish. */
mp_status mp_scene_draw(mp_ctx* ctx, const mp_scene* scene, int32_t camera);

/* 64-bit atomicMin throughput probe (atomics per second): pattern 0 uniform
 * random slots, pattern 1 micropolygon-like locality. */
mp_status mp_atomic_bench(mp_ctx* ctx, int64_t n_slots, int64_t n_ops, int32_t pattern, double* atomics_per_s);

#ifdef __cplusplus
}
#endif

#endif /* MP_CORE_H */
