// Types shared by the host runtime and the kernels of the splat pipeline.
#pragma once
#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

namespace spl {

// Uniform block of one frame, byte-compatible with the reference's `Uniforms`
// (Lichtso/splatter src/renderer.rs:49-61, src/shaders.wgsl:1-11).  Passed to kernels by value.
struct Uniforms {
    float camera[16];  // camera-to-world, column-major
    float view[16];    // world-to-camera
    float vp[16];      // projection * view
    float view_size[2];
    uint32_t image_size[2];
    float tol;     // frustum_culling_tolerance
    float bias;    // ellipse_size_bias
    float margin;  // ellipse_margin
    float splat_scale;
};
static_assert(sizeof(Uniforms) == 224, "uniform block must stay 224 bytes");

// Device error bits (FrameCounters::err).
enum : uint32_t {
    SPL_DEV_ERR_LOOKBACK = 1u,       // a bounded look-back wait ran out
    SPL_DEV_ERR_PAIR_OVERFLOW = 2u,  // the tile-binning list exceeded its capacity
};

// Per-frame counters; zeroed by k_frame_begin at the start of every frame.
struct FrameCounters {
    uint32_t tile_counter[12];  // dynamic tile ids: 0 cull, 1..4 depth passes, 5..7 pair passes, 8 bin
    uint32_t visible;          // V: splats that pass the frustum test
    uint32_t keys_all_ones;    // visible splats whose composite key is 0xFFFFFFFF
    uint32_t keys_top_ff;      // visible splats whose key's top byte is 0xFF (not drawn in indirect mode)
    uint32_t pairs;            // (tile, splat) pairs the binning wanted to emit
    uint32_t err;              // SPL_DEV_ERR_* bits
    uint32_t draw;             // entries drawn (mode dependent)
    uint32_t epoch;            // copy of the frame epoch (for readback)
    uint32_t barrier[2];       // grid-barrier arrivals of the cooperative depth sort and pair sort
    uint32_t hist_depth[4][256];  // digit histograms of the visible depth keys (onesweep sort only)
    uint32_t hist_pairs[3][256];  // digit histograms of the tile ids of all pairs (onesweep sort only)
};

// Depth-sorting modes (renderer.rs:14-23).
enum DepthSorting : int32_t { DS_NONE = 0, DS_CPU = 1, DS_GPU = 2, DS_GPU_INDIRECT = 3 };

// Per-splat screen-space record written by the preprocess kernel (16 floats = 4 x float4):
//   q0 = (A00, A01, B0, A10)  q1 = (A11, B1, alpha, bbox_lo)  q2 = (r, g, b, bbox_hi)  q3 = (bx, by, R, 0)
// tc = (A00*X + A01*Y + B0, A10*X + A11*Y + B1) at pixel centre (X, Y); bbox_lo/hi = x | y << 16
// (inclusive pixel box, empty when lo > hi); (bx, by, R) is the axis-aligned-square coverage test.
constexpr int RECORD_FLOATS = 16;

constexpr int TILE_PIXELS = 16;        // raster tile edge
constexpr int CULL_TILE = 4096;        // splats per cull/compaction tile
constexpr int SORT_TILE = 4096;        // keys per onesweep tile (256 threads x 16)
constexpr int BIN_TILE = 1024;         // draw entries per binning tile (256 threads x 4)
constexpr float FP32_T_MIN = 1e-4f;    // fp32 blend mode stops a pixel below this transmittance

struct SceneView {
    const float* x;
    const float* y;
    const float* z;
    const float4* rot;          // (scalar, i, j, k)
    const float4* scale_alpha;  // (sx, sy, sz, alpha)
    const float* sh;            // 48 per splat
    uint32_t n;
};

// ---- launchers (defined in the .cu files) --------------------------------------------------------
// Streaming multiprocessors of the current device (queried once per device, then cached); grids of
// grid-stride kernels are capped at a multiple of it.
uint32_t device_sm_count();
void launch_frame_begin(FrameCounters* fc, uint32_t* epoch_word, cudaStream_t st);  // counters + epoch only
void launch_frame_begin(FrameCounters* fc, uint32_t* epoch_word, const Uniforms& u, Uniforms* d_u, const SceneView& sv,
                        SceneView* d_sv, cudaStream_t st);
const void* frame_begin_kernel();  // host handle of k_frame_begin (to find its node in a captured graph)
const void* raster_kernel(bool rect, int blend);  // host handle of the raster kernel (its output is re-targeted)
constexpr int RASTER_OUT_ARG = 10;                // index of the raster kernel's output-pointer argument
// grid_n: the splat count the grid is sized for (the scene's, or the renderer's maximum for a
// captured frame whose scene changes between launches); the kernels read the scene from d_sv.
// hist: also build the digit histograms of the keys (the onesweep passes need them).
void launch_cull_key(int mode, bool hist, uint32_t grid_n, const SceneView* d_sv, const Uniforms* d_u,
                     FrameCounters* fc, const uint32_t* epoch_word, uint64_t* status, uint32_t* keys_out,
                     uint32_t* idx_out, uint32_t spin_limit, cudaStream_t st);
void launch_preprocess(int sh_order, bool covariance, bool rect, const SceneView* d_sv, const Uniforms* d_u,
                       const uint32_t* idx, const FrameCounters* fc, float4* rec, uint2* boxes, uint32_t max_n,
                       cudaStream_t st);
// One LSD onesweep pass over 8 bits at `shift`.  n = min(*n_ptr, n_cap).  vals_in == nullptr means
// values are the input positions (0, 1, 2, ...).
void onesweep_prepare();  // runs the one-time occupancy query outside any stream capture
void launch_onesweep(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                     const uint32_t* n_ptr, uint32_t n_cap, const uint32_t* hist256, uint64_t* status,
                     uint32_t* tile_counter, const uint32_t* epoch_word, int shift, uint32_t spin_limit,
                     uint32_t* err, cudaStream_t st);
// hist: also build the digit histograms of the pairs' tile ids (the onesweep passes need them).
void launch_bin(int mode, bool hist, const uint32_t* order, const uint2* boxes, FrameCounters* fc,
                const uint32_t* epoch_word, uint64_t* status, uint32_t* pair_keys, uint32_t* pair_vals,
                uint32_t pair_cap, int tiles_x, uint32_t max_n, uint32_t spin_limit, cudaStream_t st);
void launch_tile_ranges(const uint32_t* pair_keys, const FrameCounters* fc, uint32_t pair_cap, uint2* ranges,
                        cudaStream_t st);
// Orders the tiles most pairs first (tile_order, one entry per tile), then rasterises them in that order;
// with tile_order == nullptr in row-major order.
void launch_raster(bool rect, int blend, const uint2* ranges, uint32_t* tile_order, const uint32_t* pair_vals,
                   const float4* rec, const Uniforms& u, void* out, cudaStream_t st);
void launch_load_records(const float* records62, uint32_t count, float* x, float* y, float* z, float4* rot,
                         float4* scale_alpha, float* sh, cudaStream_t st);
void launch_splats60_to_soa(const float* s60, uint32_t count, float* x, float* y, float* z, float4* rot,
                            float4* scale_alpha, float* sh, cudaStream_t st);
void launch_soa_to_splats60(const SceneView& s, uint32_t start, uint32_t count, float* s60, cudaStream_t st);
void launch_gather_entries(const uint32_t* keys, const uint32_t* slots, const uint32_t* idx, const FrameCounters* fc,
                           int mode, uint32_t* keys_out, uint32_t* idx_out, uint32_t cap, cudaStream_t st);
// All passes of a stable LSD radix sort in one cooperative launch (k_sort_coop.cu).  Pass p reads
// buffers (p even: 0, odd: 1) and writes the other; cnt holds 256 x sort_coop_grid() words; *bar (the
// grid barrier's arrival count) must be zero when the launch starts.
cudaError_t launch_sort_coop(uint32_t* keys0, uint32_t* keys1, uint32_t* vals0, uint32_t* vals1, bool iota_first,
                             const uint32_t* n_ptr, uint32_t n_cap, int passes, int shift0, uint32_t* cnt,
                             uint32_t* bar, uint32_t spin_limit, uint32_t* err, cudaStream_t st);
int sort_coop_grid();
// The loader's activations of raw parameters and their backward (k_activate.cu).
void launch_activate(uint32_t n, const float* means, const float* quats, const float* logs, const float* logits,
                     float* x, float* y, float* z, float* rot, float* scale_alpha, cudaStream_t st);
void launch_activate_backward(uint32_t n, const float* quats, const float* logs, const float* rot,
                              const float* scale_alpha, const float* gx, const float* gy, const float* gz,
                              const float* grot, const float* gsa, float* g_means, float* g_quats, float* g_logs,
                              float* g_logits, cudaStream_t st);
// The L2 image loss of float4 frames against RGB targets (k_activate.cu): l2_loss_partials(pixels)
// block partial sums, and its gradient (2 (image - target) * *scale, 0).
uint32_t l2_loss_partials(uint64_t pixels);
void launch_l2_loss(const float* image, const float* target, uint64_t pixels, float* partial, cudaStream_t st);
void launch_l2_loss_backward(const float* image, const float* target, uint64_t pixels, const float* scale,
                             float* grad, cudaStream_t st);
// Backward of the last frame (fp32 blend): raster backward into grad_rec (10 floats per record),
// then the vertex-stage backward into per-splat parameter gradients.  deferred: 1 + max_n words (the
// needles and discs whose vertex-stage sweep runs in double).
void launch_backward(int sh_order, bool covariance, bool rect, const SceneView& s, const Uniforms& u,
                     const uint32_t* idx, const FrameCounters* fc, const uint2* boxes, const uint2* ranges,
                     const uint32_t* tile_order, const uint32_t* pair_vals, const float4* rec, const float4* image,
                     const float4* grad_image,
                     float* grad_rec, uint32_t* deferred,
                     uint32_t max_n, float* gx, float* gy, float* gz, float4* grot, float4* gscale_alpha, float* gsh,
                     bool accumulate, cudaStream_t st);
void launch_histogram(const uint32_t* keys, const uint32_t* n_ptr, uint32_t n_cap, uint32_t* hist4x256,
                      cudaStream_t st);
void launch_set_count(uint32_t* dst, uint32_t value, cudaStream_t st);
void launch_lookback_probe(uint64_t* status, uint32_t* err, uint32_t spin_limit, uint32_t* out, cudaStream_t st);

}  // namespace spl
