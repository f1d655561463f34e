/*
 * splatter.h — C ABI of libsplatter_cuda.so, the GB300 (sm_103a) implementation of splatter's
 * per-frame splat pipeline (Lichtso/splatter: src/renderer.rs, src/scene.rs, src/shaders.wgsl).
 *
 * The entry points mirror the reference's Rust API one to one; each declaration names the Rust item
 * it replaces (file:line in the reference).  Plain C types only: device buffers are raw pointers,
 * CUDA streams are passed as `void*` (a cudaStream_t; NULL = the legacy default stream), so a Rust
 * crate can bind this header with `extern "C"` + `#[repr(C)]` without CUDA headers.
 *
 * Errors: every call that can fail returns an SPL_* status (the reference panics via unwrap/assert);
 * spl_last_error_string() describes the last failure of the calling thread.  No C++ exception
 * crosses this boundary.
 *
 * Ownership and threading (renderer.rs:64-84, scene.rs:35-41): the caller owns every handle and
 * frees it with the matching *_destroy.  A renderer owns its sorting/binning scratch, so it renders
 * one frame at a time (calls on one renderer must not overlap on the GPU).  A scene may be rendered
 * by several renderers that were created on the same device.
 */
#ifndef SPLATTER_H
#define SPLATTER_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SPL_API __attribute__((visibility("default")))
#else
#define SPL_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------------ */
#define SPL_OK 0
#define SPL_ERR_INVALID 1          /* bad argument or configuration (reference: assert, renderer.rs:90) */
#define SPL_ERR_OOM 2              /* device or pinned allocation failed */
#define SPL_ERR_IO 3               /* file could not be read or parsed (reference: unwrap, scene.rs:202-224) */
#define SPL_ERR_LOOKBACK_TIMEOUT 4 /* a bounded decoupled look-back wait ran out (no hang, no trap) */
#define SPL_ERR_CUDA 5             /* a CUDA runtime call failed */
#define SPL_ERR_CAPACITY 6         /* the tile-binning pair list overflowed max_pair_count */

/* ---- configuration (renderer.rs:14-47) ----------------------------------------------------------- */
/* DepthSorting (renderer.rs:14-23). */
#define SPL_DEPTH_SORTING_NONE 0
#define SPL_DEPTH_SORTING_CPU 1
#define SPL_DEPTH_SORTING_GPU 2
#define SPL_DEPTH_SORTING_GPU_INDIRECT_DRAW 3

/* Blend target (extension): the reference blends into a Bgra8Unorm surface
 * (application_framework.rs:184); UNORM8 reproduces that with per-blend re-quantisation and writes
 * RGBA8 (A = final transmittance, i.e. the destination alpha the reference leaves behind).  FP32
 * blends in f32 and writes float4 (r, g, b, T). */
#define SPL_BLEND_UNORM8 0
#define SPL_BLEND_FP32 1

/* Configuration (renderer.rs:26-47) minus `surface_configuration` (no surface: output is a device
 * buffer), plus three documented extensions at the end. */
typedef struct spl_config {
    int32_t depth_sorting;              /* renderer.rs:29-30 */
    int32_t use_covariance_for_scale;   /* renderer.rs:31-32 (bool) */
    int32_t use_unaligned_rectangles;   /* renderer.rs:33-34 (bool) */
    uint32_t spherical_harmonics_order; /* renderer.rs:35-36, 0..=3 */
    uint64_t max_splat_count;           /* renderer.rs:37-38, 1 .. 2^30-1 */
    uint32_t radix_bits_per_digit;      /* renderer.rs:39-40, must divide 32 (renderer.rs:89-90); the
                                           device sort always ranks 8 bits per pass — the order is
                                           the same stable order for every valid value */
    float frustum_culling_tolerance;    /* renderer.rs:41-42 */
    float ellipse_margin;               /* renderer.rs:43-44 */
    float splat_scale;                  /* renderer.rs:45-46 */
    float field_of_view_y;              /* extension: the reference hard-codes pi/2 (renderer.rs:366) */
    int32_t blend_mode;                 /* extension: SPL_BLEND_* */
    uint64_t max_pair_count;            /* extension: capacity of the (tile, splat) list; 0 = 16 x
                                           max_splat_count (at least 2^20), at most 2^30-1 */
} spl_config;

typedef struct spl_renderer spl_renderer; /* Renderer, renderer.rs:64-84 */
typedef struct spl_scene spl_scene;       /* Scene, scene.rs:35-41 */

/* Counters of the last frame a renderer rendered (read back after the frame completes). */
typedef struct spl_frame_info {
    uint64_t splat_count;   /* N of the scene */
    uint64_t visible_count; /* V: splats inside the frustum (sorted / compacted entries) */
    uint64_t draw_count;    /* entries drawn: DrawIndirect.instance_count in GpuIndirectDraw mode
                               (shaders.wgsl:458-461); keys != 0xFFFFFFFF in Gpu mode; V otherwise */
    uint64_t pair_count;    /* (tile, splat) pairs the binning produced (may exceed capacity) */
    uint32_t device_error;  /* raw device error bits (1 = look-back timeout, 2 = pair overflow) */
    uint32_t width, height;
} spl_frame_info;

/* The `Configuration` literal of the reference's viewer (showcase.rs:39-50), with max_splat_count
 * 4Mi, field_of_view_y = pi/2 (the reference's fixed value), blend_mode UNORM8. */
SPL_API void spl_config_default(spl_config* cfg);

/* ---- renderer (renderer.rs:86-352) ---------------------------------------------------------------- */
/* Renderer::new (renderer.rs:88): validates the configuration (radix bits must divide 32,
 * renderer.rs:89-90) and allocates the sorting and binning scratch on the current CUDA device. */
SPL_API int spl_renderer_create(const spl_config* cfg, spl_renderer** out);
SPL_API void spl_renderer_destroy(spl_renderer* r);
/* Sizes the per-resolution scratch for frames up to width x height, so that later frames of that
 * size neither allocate nor synchronise (required before capturing render_frame into a CUDA graph). */
SPL_API int spl_renderer_reserve(spl_renderer* r, uint32_t width, uint32_t height);

/* Renderer::render_frame (renderer.rs:355-466): renders `scene` seen from `camera_to_world` (16
 * floats, column-major: right, up, forward, position — what motor3d_to_mat4 of the camera motor
 * gives, utils.rs:31-42) into `out_device` (width*height RGBA8 for SPL_BLEND_UNORM8, float4 for
 * SPL_BLEND_FP32, row-major, top row first).  Asynchronous on `stream`, like queue.submit
 * (renderer.rs:465); call spl_renderer_frame_info to wait and read the frame's counters/status. */
SPL_API int spl_render_frame(spl_renderer* r, const spl_scene* scene, const float camera_to_world[16], uint32_t width,
                     uint32_t height, void* out_device, void* stream);

/* Frame graphs inside render_frame (extension, on by default): when two frames in a row on a renderer
 * have the same viewport and scene size, the renderer captures the frame into a CUDA graph (grids
 * sized for that scene, as the direct launches) and replays it for later frames of that viewport and
 * size, any camera, any scene of that size and any output buffer — one graph launch instead of one
 * launch per kernel, the same results.  Frames are launched directly while profiling is on, while
 * the stream is being captured, and for other viewports and sizes.  enable = 0 turns it off (and
 * frees the graph). */
SPL_API int spl_renderer_set_frame_graphs(spl_renderer* r, int enable);

/* ---- camera motors (renderer.rs:355-366, utils.rs:31-42) -------------------------------------------
 * The reference's render_frame takes a projective-geometric-algebra motor.  Layout here (the crate
 * geometric_algebra 0.3.0 that defines the reference's is not available; built from the algebra
 * Cl(3,0,1) in double precision, rounded once to float):
 *   motor  [s, e23, e31, e12, e01, e02, e03, e0123],  moving points by the sandwich M P ~M
 *   rotor  [s, e23, e31, e12] ~ unit quaternion (w, x, y, z): a right-handed turn by 2 acos(s) about
 *          the axis (e23, e31, e12) / sin, like showcase.rs:16-19's rotate_around_axis
 * spl_motor_to_mat4 is motor3d_to_mat4: the images of the x, y, z directions and of the origin as
 * columns (column-major), i.e. camera_to_world.  spl_motor_inverse is Motor::inverse
 * (renderer.rs:365); spl_motor_product the geometric product (a applied after b);
 * spl_motor_from_rotor_translation builds translator(t) * rotor (showcase.rs:140).
 * spl_render_frame_motor renders with spl_motor_to_mat4 of the motor. */
SPL_API int spl_motor_to_mat4(const float motor[8], float camera_to_world[16]);
SPL_API int spl_motor_inverse(const float motor[8], float out[8]);
SPL_API int spl_motor_product(const float a[8], const float b[8], float out[8]);
SPL_API int spl_motor_from_rotor_translation(const float rotor[4], const float translation[3], float out[8]);
SPL_API int spl_render_frame_motor(spl_renderer* r, const spl_scene* scene, const float motor[8], uint32_t width,
                                   uint32_t height, void* out_device, void* stream);

/* Waits for the renderer's last frame and returns its counters; returns SPL_ERR_LOOKBACK_TIMEOUT or
 * SPL_ERR_CAPACITY when the device flagged one. */
SPL_API int spl_renderer_frame_info(spl_renderer* r, spl_frame_info* info);

/* Copies the last frame's visible entries — (depth key, splat index) in draw order: stable-sorted by
 * key for the sorting modes, index order for None — into device arrays of `capacity` entries (the
 * reference's debug readback of the entry buffer, renderer.rs:462-464).  Asynchronous on `stream`. */
SPL_API int spl_renderer_copy_entries(spl_renderer* r, uint32_t* keys_device, uint32_t* indices_device, uint64_t capacity,
                              void* stream);

/* Copies the last frame's per-splat screen-space records (16 floats per visible splat, in compaction
 * order = ascending splat index) into a device array of `capacity` records.  Asynchronous. */
SPL_API int spl_renderer_copy_records(spl_renderer* r, float* records_device, uint64_t capacity, void* stream);

/* Host math of render_frame (renderer.rs:364-409, utils.rs:45-70): the 224-byte uniform block for a
 * camera and viewport.  No GPU work. */
SPL_API int spl_compute_uniforms(const spl_config* cfg, const float camera_to_world[16], uint32_t width, uint32_t height,
                         void* uniforms_out_224);

/* ---- scene (scene.rs:43-264) ------------------------------------------------------------------ */
/* Scene::new (scene.rs:45): allocates resident SoA splat arrays for min(splat_count, max_splat_count)
 * splats (scene.rs:46); *clamped_count receives that number (may be NULL). */
SPL_API int spl_scene_create(spl_renderer* r, uint64_t splat_count, spl_scene** out, uint64_t* clamped_count);
SPL_API void spl_scene_destroy(spl_scene* s);
SPL_API uint64_t spl_scene_splat_count(const spl_scene* s);
/* Bytes of device memory the scene's arrays occupy (236 per splat). */
SPL_API uint64_t spl_scene_device_bytes(const spl_scene* s);

/* Scene::new_dev_test (scene.rs:158-192): three splats on the unit axes. */
SPL_API int spl_scene_create_dev_test(spl_renderer* r, spl_scene** out);

/* Scene::parse_file_header (scene.rs:197-213): header length in bytes and `element vertex` count.
 * The reference keeps the header length in a u16 (scene.rs:211); here it is a u32. */
SPL_API int spl_parse_file_header(const char* path, uint32_t* header_bytes, uint64_t* splat_count);

/* Scene::load_chunk (scene.rs:216-264) from host memory: `count` records of 62 floats (248 bytes,
 * scene.rs:15-24) for splats [start, start+count) (clamped to the scene, scene.rs:217).  The
 * records are staged through pinned memory and copied with cudaMemcpyAsync; the transform (rotor
 * normalisation, clamped exp of the log-scales, sigmoid opacity, SH copy) runs on the device.  The
 * host buffer may be reused when the call returns; the device work is asynchronous on `stream`. */
SPL_API int spl_scene_load_chunk(spl_scene* s, const void* records, uint64_t start, uint64_t count, void* stream);

/* Scene::load_chunk reading the records straight from a splat file (seek to header + start*248,
 * scene.rs:220-224) into the pinned staging buffers. */
SPL_API int spl_scene_load_chunk_file(spl_scene* s, const char* path, uint32_t header_bytes, uint64_t start, uint64_t count,
                              void* stream);

/* A validating splat-file header parser (no reference counterpart; the reference reads such files
 * unchecked, scene.rs:197-224): binary_little_endian 1.0 PLY, the vertex element first, exactly 62
 * 32-bit float vertex properties (with check_names, in the standard order x y z nx ny nz f_dc_0..2
 * f_rest_0..44 opacity scale_0..2 rot_0..3 — SerializedSplat, scene.rs:15-24), LF or CRLF lines, and
 * a body of at least 248 bytes per declared splat.  Same outputs as spl_parse_file_header; every
 * failure is SPL_ERR_IO with a message naming the line. */
SPL_API int spl_validate_file_header(const char* path, int check_names, uint32_t* header_bytes, uint64_t* splat_count);

/* Progressive loading as the reference's viewer does it (showcase.rs:13,54-59,98-103): a scene created
 * for the file's full count is filled one chunk per step, the last chunk first, so frames rendered in
 * between show the splats loaded so far (the others are still zero: no opacity, not drawn).
 * chunk_size 0 loads the whole scene in the first step.  Each step reads its chunk into the pinned
 * staging buffers and enqueues the copy and transform on `stream` (a frame rendered afterwards on
 * that stream sees it); *chunks_left (may be NULL) receives the number of chunks still to load.  The
 * file stays open until spl_progressive_loader_destroy.  (The reference's viewer also updates the
 * host positions of its CPU sort at the chunk-relative index, scene.rs:259-261, so chunked loading
 * with DepthSorting::Cpu sorts wrong positions there; here every mode reads the device arrays.) */
typedef struct spl_progressive_loader spl_progressive_loader;
SPL_API int spl_progressive_loader_create(spl_scene* s, const char* path, uint32_t header_bytes, uint64_t chunk_size,
                                          spl_progressive_loader** out);
SPL_API int spl_progressive_loader_step(spl_progressive_loader* l, void* stream, uint64_t* chunks_left);
SPL_API void spl_progressive_loader_destroy(spl_progressive_loader* l);

/* Writes splats already in the reference's device layout (60 floats: rotation[4], centre[3], pad,
 * scale[3], alpha, colourSH[48]; scene.rs:32, shaders.wgsl:28-35) from host memory — the write
 * new_dev_test does (scene.rs:178-182). */
SPL_API int spl_scene_write_splats(spl_scene* s, const float* splats60, uint64_t start, uint64_t count, void* stream);

/* Reads splats back in the same 60-float layout into host memory (synchronous). */
SPL_API int spl_scene_read_splats(const spl_scene* s, float* splats60, uint64_t start, uint64_t count);

/* A scene over caller-owned device arrays (no copy; the arrays must outlive the scene and are not
 * freed by spl_scene_destroy): planes x[n], y[n], z[n]; rotation[n][4] (scalar first, used as given —
 * the file loader normalises, scene.rs:227); scale_alpha[n][4] (scale xyz, opacity); sh[n][48].  The
 * last three must be 16-byte aligned.  This is how a training loop renders parameters it owns. */
SPL_API int spl_scene_wrap(spl_renderer* r, uint64_t splat_count, float* x, float* y, float* z, float* rotation,
                           float* scale_alpha, float* sh, spl_scene** out);

/* ---- backward pass (no reference counterpart) ------------------------------------------------------- */
/* Gradients of the renderer's LAST frame of `scene` (rendered with blend_mode SPL_BLEND_FP32) with
 * respect to the splat parameters, given the frame's float4 image (r, g, b, T) and dL/d(image)
 * (float4 per pixel).  Writes, for every splat that was drawn, grad_x/y/z[i], grad_rotation[i][4],
 * grad_scale_alpha[i][4] (scale xyz, opacity) and grad_sh[i][48]; splats that were not drawn are left
 * untouched (zero the arrays first).  grad_rotation, grad_scale_alpha and grad_sh must be 16-byte
 * aligned (SPL_ERR_INVALID otherwise).  Transmittance is recomputed per tile, not stored; depth order,
 * culling and the 1/255 discard are treated as constants.  Asynchronous on `stream`. */
SPL_API int spl_render_backward(spl_renderer* r, const spl_scene* scene, const float* image_device,
                                const float* grad_image_device, float* grad_x, float* grad_y, float* grad_z,
                                float* grad_rotation, float* grad_scale_alpha, float* grad_sh, void* stream);

/* spl_render_backward, adding the frame's gradients into the arrays instead of storing them: the
 * gradients of several frames (views) of one scene summed in place, frame after frame on one stream,
 * with no per-frame gradient arrays to zero and add up.  Zero the arrays once before the first frame. */
SPL_API int spl_render_backward_accumulate(spl_renderer* r, const spl_scene* scene, const float* image_device,
                                           const float* grad_image_device, float* grad_x, float* grad_y,
                                           float* grad_z, float* grad_rotation, float* grad_scale_alpha,
                                           float* grad_sh, void* stream);

/* The loader's activations (Scene::load_chunk, scene.rs:225-250) on device arrays of raw parameters,
 * for training: means (n x 3), quaternions (n x 4, scalar first), log-scales (n x 3) and opacity
 * logits (n) -> the arrays of a wrapped scene (x, y, z planes; unit rotations n x 4; scale + opacity
 * n x 4).  The arithmetic is the loader's, so a frame of these arrays equals the frame of a scene
 * loaded from the same file records.  Asynchronous on `stream`. */
SPL_API int spl_activate_splats(uint64_t n, const float* means, const float* quaternions, const float* log_scales,
                                const float* opacity_logits, float* x, float* y, float* z, float* rotation,
                                float* scale_alpha, void* stream);
/* Its backward: gradients of the activated arrays (x, y, z planes, rotation, scale_alpha) -> gradients
 * of the raw parameters (written, not accumulated).  Needs the raw quaternions and log-scales and the
 * activated rotation and scale_alpha. */
SPL_API int spl_activate_splats_backward(uint64_t n, const float* quaternions, const float* log_scales,
                                         const float* rotation, const float* scale_alpha, const float* grad_x,
                                         const float* grad_y, const float* grad_z, const float* grad_rotation,
                                         const float* grad_scale_alpha, float* grad_means, float* grad_quaternions,
                                         float* grad_log_scales, float* grad_opacity_logits, void* stream);

/* The L2 image loss of a training loop, sum over pixels and RGB of (image - target)^2, for `pixels`
 * float4 pixels (r, g, b, T; 16-byte aligned) against three floats per pixel: writes
 * spl_l2_image_loss_partials(pixels) partial sums to `partial` (their sum is the loss).  Its backward
 * writes grad_image[p] = (2 (image - target) * s, 0) with the scalar s (the loss's upstream gradient)
 * read from device memory: one pass each, the values torch's autograd forms for the same expression.
 * Asynchronous on `stream`. */
SPL_API uint32_t spl_l2_image_loss_partials(uint64_t pixels);
SPL_API int spl_l2_image_loss(const float* image, const float* target, uint64_t pixels, float* partial, void* stream);
SPL_API int spl_l2_image_loss_backward(const float* image, const float* target, uint64_t pixels,
                                       const float* scale_device, float* grad_image, void* stream);

/* Copies the last backward pass's per-record gradients (10 floats per visible splat, compaction
 * order: d/dA00, d/dA01, d/dB0, d/dA10, d/dA11, d/dB1 with A taken against pixel offsets from the
 * centre of the record's pixel box and B at that centre, then d/dopacity, d/dr, d/dg, d/db) into a
 * device array of `capacity` records.  Diagnostics.  Asynchronous on `stream`. */
SPL_API int spl_renderer_copy_record_gradients(spl_renderer* r, float* dst_device, uint64_t capacity, void* stream);

/* ---- device sort (radixSortB/radixSortC, shaders.wgsl:338-498) --------------------------------- */
/* Stable LSD radix sort of `count` (key, value) pairs on the device: keys_in/values_in are
 * sorted into keys_out/values_out by the low `key_bits` bits of the key (8, 16, 24 or 32), all
 * digit passes in one cooperative launch (the whole device; do not overlap it with a frame).
 * Uses the renderer's scratch (count <= max_splat_count).  Asynchronous on `stream`. */
SPL_API int spl_sort_pairs(spl_renderer* r, const uint32_t* keys_in, const uint32_t* values_in, uint32_t* keys_out,
                   uint32_t* values_out, uint64_t count, uint32_t key_bits, void* stream);

/* ---- sorting without allocation -------------------------------------------------------------------- */
/* No counterpart in the reference: an addition for callers that cannot allocate device memory when
 * they sort — hosts that give all device memory to their own pool up front (a cudaMalloc would fail
 * or bypass their accounting), plug-ins that may only touch the buffers they are handed, and loops
 * that must not take cudaMalloc's implicit device-wide synchronisation.
 * spl_sort_pairs_no_alloc gives the same stable result as spl_sort_pairs, through the onesweep passes
 * (spl_sort_pairs runs the cooperative sort), without a renderer: its scratch is a static device
 * array the library reserves on every device that loads it (2.6 MB, held until the process exits),
 * and it calls no allocator.  At most SPL_NO_ALLOC_MAX_PAIRS pairs per call (larger counts return
 * SPL_ERR_INVALID).  All calls on a device share that scratch and its contents persist between
 * calls: calls whose GPU work overlaps race and give wrong results, so order them on one stream.
 * The first call on a device looks up the scratch address (cudaGetSymbolAddress) with that device
 * current; make it before any stream capture.  Only the device's primary context is supported (the
 * address is cached per device ordinal; after cudaDeviceReset it is stale).  Inputs and outputs
 * must not overlap.  Asynchronous on `stream`. */
#define SPL_NO_ALLOC_MAX_PAIRS 262144u
SPL_API int spl_sort_pairs_no_alloc(const uint32_t* keys_in, const uint32_t* values_in, uint32_t* keys_out,
                                    uint32_t* values_out, uint64_t count, uint32_t key_bits, void* stream);
/* Status of the last spl_sort_pairs_no_alloc on the current device: waits for `stream` (the stream
 * that call used), then reads the scratch's device error word into *device_error (may be NULL;
 * bit 1 = a bounded look-back wait ran out, so the output is not sorted) and returns
 * SPL_ERR_LOOKBACK_TIMEOUT when it is set, SPL_OK otherwise.  Allocates nothing.  The word is
 * cleared by the next sort call with a non-zero count. */
SPL_API int spl_sort_pairs_no_alloc_status(void* stream, uint32_t* device_error);

/* ---- diagnostics ----------------------------------------------------------------------------------- */
/* Stage timing with CUDA events on the launching stream (off by default).  When enabled, each
 * render_frame records events between its stages; spl_renderer_stage_times waits for the last frame
 * and writes SPL_STAGE_COUNT durations in milliseconds, indexed by SPL_STAGE_*.  The stages run one
 * after another on the frame's stream, so they add up to the frame time. */
#define SPL_STAGE_CULL 0       /* frame start, cull + key + ordered compaction */
#define SPL_STAGE_PREPROCESS 1 /* vertex stage: colour, conic, rectangle records */
#define SPL_STAGE_DEPTH_SORT 2 /* the stable depth sort of the visible keys (one cooperative launch,
                                  or one onesweep launch per digit pass) */
#define SPL_STAGE_BIN 3        /* tile-range clear + tile binning */
#define SPL_STAGE_PAIR_SORT 4  /* the stable sort of the (tile, splat) pairs by tile id */
#define SPL_STAGE_RANGES 5     /* per-tile list ranges */
#define SPL_STAGE_RASTER 6     /* tile order + tile raster + blend */
#define SPL_STAGE_FRAME 7      /* whole frame on the main stream */
#define SPL_STAGE_COUNT 8
SPL_API int spl_renderer_set_profiling(spl_renderer* r, int enable);
SPL_API int spl_renderer_stage_times(spl_renderer* r, float* milliseconds, int count);
/* Number of kernel launches (plus memsets) one render_frame issues with this configuration at this
 * viewport. */
SPL_API int spl_renderer_launches_per_frame(const spl_renderer* r, uint32_t width, uint32_t height);

/* ---- sort algorithm (extension) -----------------------------------------------------------------
 * COOPERATIVE (default): each sort (the 4 depth passes, the <= 3 tile-id passes) is one cooperative
 * launch with grid-wide barriers; it assumes the whole device, so only one such frame may run at a
 * time.  ONESWEEP: one launch per pass with decoupled look-back over dynamically numbered tiles,
 * safe when several renderers run frames concurrently on different streams (the serving runtime
 * uses it).  Both are stable and give identical results. */
#define SPL_SORT_COOPERATIVE 0
#define SPL_SORT_ONESWEEP 1
SPL_API int spl_renderer_set_sort_mode(spl_renderer* r, int mode);

/* ---- captured frames (extension) ----------------------------------------------------------------
 * A frame at width x height into `out_device`, captured once into a CUDA graph with grids sized for
 * scenes of up to max_splats splats (0: the renderer's max_splat_count); each launch replays it for
 * any such scene and any camera (only the first kernel's parameters change: the kernels read the
 * scene and every count from device memory), on any stream.  The renderer's scratch is shared with
 * its other frames: one frame of a renderer in flight at a time.  Destroy the graph before the
 * renderer or the output buffer.  A later frame at a larger viewport reallocates the renderer's
 * per-viewport scratch; a graph captured before that refuses to launch (SPL_ERR_INVALID): capture
 * it again, or reserve the largest viewport first (spl_renderer_reserve). */
typedef struct spl_frame_graph spl_frame_graph;
SPL_API int spl_frame_graph_create(spl_renderer* r, uint32_t width, uint32_t height, uint64_t max_splats,
                                   void* out_device, spl_frame_graph** out);
SPL_API int spl_frame_graph_launch(spl_frame_graph* g, const spl_scene* scene, const float camera_to_world[16],
                                   void* stream);
SPL_API void spl_frame_graph_destroy(spl_frame_graph* g);

/* Scene::load_chunk from 62-float records already in device memory (no staging). */
SPL_API int spl_scene_load_chunk_device(spl_scene* s, const float* records_device, uint64_t start, uint64_t count,
                                        void* stream);

/* ---- serving runtime (extension; no reference counterpart) --------------------------------------
 * Many scenes resident on the device, admitted by their device footprint against a budget; scenes
 * beyond it are evicted least-recently-used (their page-locked host copies stay and are copied back
 * on the next request).  Requests of any scene, pose and viewport are admitted continuously as
 * slots free up: each slot owns a renderer's scratch, a stream and an output buffer, so the frames
 * of different slots overlap on the device; with use_graphs each slot replays a captured frame
 * graph per viewport and power-of-two scene-size class (grids at most twice the scene).  One scheduler thread per server issues all device work. */
typedef struct spl_server spl_server;
typedef struct spl_server_config {
    uint32_t slots;               /* frames in flight (>= 1) */
    uint32_t use_graphs;          /* 1: replay captured frame graphs; 0: launch each frame's kernels */
    uint64_t scene_memory_budget; /* device bytes for resident scenes; 0 = no limit */
    uint32_t max_width;           /* largest viewport a request may ask for */
    uint32_t max_height;
} spl_server_config;
typedef struct spl_request {
    uint64_t tag;                 /* returned in the completion */
    uint32_t scene_id;
    uint32_t width, height;
    float camera_to_world[16];
    void* host_out;               /* width*height*4 bytes (UNORM8) or *16 (FP32); page-locked lets it overlap */
} spl_request;
typedef struct spl_completion {
    uint64_t tag;
    int32_t status;               /* SPL_OK or an SPL_ERR_* code */
    uint32_t slot;
    uint64_t t_submit_ns, t_start_ns, t_done_ns; /* spl_server_now_ns clock */
    uint32_t restored;            /* 1 when this request copied its scene back to the device */
    uint32_t reserved;
} spl_completion;
typedef struct spl_server_stats {
    uint64_t submitted, completed, failed;
    uint64_t resident_scenes, resident_bytes, evictions, restores;
    uint64_t graphs_captured, graph_launches, direct_launches, max_in_flight;
} spl_server_stats;
SPL_API int spl_server_create(const spl_config* cfg, const spl_server_config* scfg, spl_server** out);
/* Waits for the requests in flight, then frees everything. */
SPL_API void spl_server_destroy(spl_server* s);
/* Adds a scene from `count` 62-float file records (host memory, or device memory when
 * records_on_device != 0); returns its id. */
SPL_API int spl_server_add_scene(spl_server* s, const float* records62, uint64_t count, int records_on_device,
                                 uint32_t* scene_id);
/* Queues a request (thread-safe, does not block on the device). */
SPL_API int spl_server_submit(spl_server* s, const spl_request* req);
/* Up to `capacity` completions; waits up to timeout_us (< 0: forever) for the first one. */
SPL_API int spl_server_poll(spl_server* s, spl_completion* out, uint32_t capacity, uint32_t* count,
                            int64_t timeout_us);
SPL_API int spl_server_get_stats(spl_server* s, spl_server_stats* out);
SPL_API uint64_t spl_server_now_ns(void);

SPL_API const char* spl_last_error_string(void);
/* Runs one bounded look-back wait against a predecessor that never publishes, with a wait limit of
 * `spin_limit` polls, and reports whether the kernel returned with the timeout flag set
 * (*timed_out = 1).  Used to check that waits end with an error status instead of hanging. */
SPL_API int spl_debug_lookback_timeout(uint32_t spin_limit, int* timed_out);

#ifdef __cplusplus
}
#endif
#endif /* SPLATTER_H */
