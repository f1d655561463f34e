// Host runtime and C ABI of libsplatter_cuda.so (declared in include/splatter.h).
//
// Mirrors the reference's host side (Lichtso/splatter src/renderer.rs, src/scene.rs, src/utils.rs):
// Renderer owns the per-frame scratch (the reference's sorting buffer, entry buffers A/B and uniform
// buffer, renderer.rs:292-331), Scene owns resident splat arrays (scene.rs:45-155).  Instead of
// bind groups and compute/render passes, render_frame launches the sm_103a kernels on a CUDA stream;
// every per-frame size lives in device memory, so a frame never synchronises with the host and can
// be captured into a CUDA graph.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/splatter.h"
#include "spl_internal.h"

using namespace spl;

namespace {
thread_local std::string g_err;
}  // namespace

namespace spl {
int vfail(int code, const char* fmt, va_list ap) {
    char buf[512];
    vsnprintf(buf, sizeof(buf), fmt, ap);
    g_err = buf;
    return code;
}
}  // namespace spl

int spl_internal_fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    const int rc = spl::vfail(code, fmt, ap);
    va_end(ap);
    return rc;
}


// Frame uniforms (renderer.rs:364-409; utils.rs:45-70).  The camera is the camera-to-world matrix
// (motor3d_to_mat4 of the motor, utils.rs:31-42); the view matrix is its rigid inverse (the
// reference inverts the motor, renderer.rs:365).  field_of_view_y is a documented extension (the
// reference fixes pi/2, renderer.rs:366); view_width = aspect * view_height equals the reference's
// aspect / view_height there, because view_height == 1.
void spl::compute_uniforms(const spl_config& cfg, const float* cam, uint32_t W, uint32_t H, Uniforms& u) {
    std::memcpy(u.camera, cam, 64);
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) u.view[c * 4 + r] = cam[r * 4 + c];
    for (int r = 0; r < 3; ++r)
        u.view[12 + r] = -((cam[r * 4 + 0] * cam[12] + cam[r * 4 + 1] * cam[13]) + cam[r * 4 + 2] * cam[14]);
    u.view[3] = 0.0f;
    u.view[7] = 0.0f;
    u.view[11] = 0.0f;
    u.view[15] = 1.0f;
    const float half = cfg.field_of_view_y * 0.5f;
    const float vh = (float)std::tan((double)half);
    const float aspect = (float)W / (float)H;
    const float vw = aspect * vh;
    const float nearp = 1.0f, farp = 1000.0f;
    const float den = 1.0f / (nearp - farp);
    // perspective_projection (utils.rs:45-55), columns
    const float P[16] = {1.0f / vw, 0, 0, 0, 0, 1.0f / vh, 0, 0, 0, 0, -farp * den, 1.0f, 0, 0, nearp * farp * den, 0};
    // mat4_multiplication (utils.rs:58-65): column i = sum_k P[k] * V[i][k], in k order
    for (int i = 0; i < 4; ++i)
        for (int r = 0; r < 4; ++r)
            u.vp[i * 4 + r] = ((P[0 * 4 + r] * u.view[i * 4 + 0] + P[1 * 4 + r] * u.view[i * 4 + 1]) +
                               P[2 * 4 + r] * u.view[i * 4 + 2]) +
                              P[3 * 4 + r] * u.view[i * 4 + 3];
    u.view_size[0] = vw;
    u.view_size[1] = vh;
    u.image_size[0] = W;
    u.image_size[1] = H;
    u.tol = cfg.frustum_culling_tolerance;
    u.bias = (0.2f * vw) / (float)W;  // renderer.rs:404
    u.margin = cfg.ellipse_margin;
    u.splat_scale = cfg.splat_scale;
}


static int validate_config(const spl_config* c) {
    if (!c) return fail(SPL_ERR_INVALID, "config is NULL");
    if (c->depth_sorting < 0 || c->depth_sorting > 3) return fail(SPL_ERR_INVALID, "depth_sorting %d", c->depth_sorting);
    if (c->spherical_harmonics_order > 3)
        return fail(SPL_ERR_INVALID, "spherical_harmonics_order %u > 3", c->spherical_harmonics_order);
    const uint32_t b = c->radix_bits_per_digit;
    if (b == 0 || b > 32 || 32 % b != 0)  // renderer.rs:89-90
        return fail(SPL_ERR_INVALID, "radix_bits_per_digit %u does not divide 32", b);
    if (c->max_splat_count == 0 || c->max_splat_count > MAX_COUNT)
        return fail(SPL_ERR_INVALID, "max_splat_count %llu outside [1, 2^30-1]", (unsigned long long)c->max_splat_count);
    if (c->blend_mode != SPL_BLEND_UNORM8 && c->blend_mode != SPL_BLEND_FP32)
        return fail(SPL_ERR_INVALID, "blend_mode %d", c->blend_mode);
    if (!(c->field_of_view_y > 0.0f && c->field_of_view_y < 3.14159265f))
        return fail(SPL_ERR_INVALID, "field_of_view_y %f outside (0, pi)", (double)c->field_of_view_y);
    if (!std::isfinite(c->frustum_culling_tolerance) || !std::isfinite(c->ellipse_margin) ||
        !std::isfinite(c->splat_scale))
        return fail(SPL_ERR_INVALID, "non-finite configuration value");
    if (c->max_pair_count > MAX_COUNT) return fail(SPL_ERR_INVALID, "max_pair_count above 2^30-1");
    return SPL_OK;
}

extern "C" {
static void drop_own_graph(spl_renderer* r);  // defined with the frame graphs (C linkage there)
}

static int ensure_ranges(spl_renderer* r, uint64_t tiles) {
    if (tiles <= r->ranges_cap) return SPL_OK;
    cudaError_t e = cudaDeviceSynchronize();  // the old buffer may still be read by a frame in flight
    if (e != cudaSuccess) return fail(SPL_ERR_CUDA, "ranges resize: %s", cudaGetErrorString(e));
    // frame graphs captured with the old buffers must not run again
    drop_own_graph(r);
    ++r->scratch_generation;
    dfree(r->ranges);
    dfree(r->tile_order);
    r->ranges_cap = 0;
    int rc = dalloc(&r->ranges, tiles);
    if (!rc) rc = dalloc(&r->tile_order, tiles);
    if (rc) {
        dfree(r->ranges);
        return rc;
    }
    r->ranges_cap = tiles;
    return SPL_OK;
}

static int ensure_staging(spl_scene* s) {
    for (int i = 0; i < 2; ++i) {
        if (!s->stg.pinned[i]) {
            cudaError_t e = cudaMallocHost(reinterpret_cast<void**>(&s->stg.pinned[i]), CHUNK_RECORDS * 62 * 4);
            if (e != cudaSuccess) {
                s->stg.pinned[i] = nullptr;
                return fail(SPL_ERR_OOM, "pinned staging: %s", cudaGetErrorString(e));
            }
        }
        if (!s->stg.dev[i]) {
            int rc = dalloc(&s->stg.dev[i], CHUNK_RECORDS * 62);
            if (rc) return rc;
        }
        if (!s->stg.ev[i]) {
            cudaError_t e = cudaEventCreateWithFlags(&s->stg.ev[i], cudaEventDisableTiming);
            if (e != cudaSuccess) return fail(SPL_ERR_CUDA, "event: %s", cudaGetErrorString(e));
        }
    }
    return SPL_OK;
}

// Shared staging loop: fill(pinned, first, count) puts `count` items of `item_floats` floats into the
// pinned buffer; the items are copied to the device and converted by `convert`.
template <typename Fill, typename Convert>
static int staged_upload(spl_scene* s, uint64_t start, uint64_t count, size_t item_floats, cudaStream_t st, Fill fill,
                         Convert convert) {
    std::lock_guard<std::mutex> lk(s->stg_mu);
    int rc = ensure_staging(s);
    if (rc) return rc;
    uint64_t done = 0;
    while (done < count) {
        const uint64_t cnt = (count - done) < CHUNK_RECORDS ? (count - done) : CHUNK_RECORDS;
        const int slot = s->stg.next;
        s->stg.next ^= 1;
        CU(cudaEventSynchronize(s->stg.ev[slot]));
        rc = fill(s->stg.pinned[slot], start + done, cnt);
        if (rc) return rc;
        CU(cudaMemcpyAsync(s->stg.dev[slot], s->stg.pinned[slot], cnt * item_floats * 4, cudaMemcpyHostToDevice, st));
        convert(s->stg.dev[slot], start + done, cnt, st);
        CU(cudaGetLastError());
        CU(cudaEventRecord(s->stg.ev[slot], st));
        done += cnt;
    }
    return SPL_OK;
}

// Splats [start, start + count) of a splat file open as `f`: seek to header + start * 248
// (scene.rs:220-224), read through the pinned staging buffers, transform on the device.
static int load_file_range(spl_scene* s, FILE* f, const char* path, uint32_t header_bytes, uint64_t start,
                           uint64_t count, cudaStream_t st) {
    if (std::fseek(f, (long)(header_bytes + start * 248ull), SEEK_SET) != 0)
        return fail(SPL_ERR_IO, "seek failed in %s", path);
    return staged_upload(
        s, start, count, 62, st,
        [&](float* dst, uint64_t, uint64_t cnt) {
            if (std::fread(dst, 248, cnt, f) != cnt) return fail(SPL_ERR_IO, "short read in %s", path);
            return SPL_OK;
        },
        [&](float* dev, uint64_t first, uint64_t cnt, cudaStream_t stm) {
            launch_load_records(dev, (uint32_t)cnt, s->x + first, s->y + first, s->z + first, s->rot + first,
                                s->scale_alpha + first, s->sh + first * 48, stm);
        });
}

extern "C" {

void spl_config_default(spl_config* cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->depth_sorting = SPL_DEPTH_SORTING_GPU;  // showcase.rs:41
    cfg->use_covariance_for_scale = 1;           // showcase.rs:42
    cfg->use_unaligned_rectangles = 1;           // showcase.rs:43
    cfg->spherical_harmonics_order = 2;          // showcase.rs:44
    cfg->max_splat_count = 1024ull * 1024 * 4;   // showcase.rs:45
    cfg->radix_bits_per_digit = 8;               // showcase.rs:46
    cfg->frustum_culling_tolerance = 1.1f;       // showcase.rs:47
    cfg->ellipse_margin = 2.0f;                  // showcase.rs:48
    cfg->splat_scale = 1.0f;                     // showcase.rs:49
    cfg->field_of_view_y = 1.57079632679489661923f;  // renderer.rs:366
    cfg->blend_mode = SPL_BLEND_UNORM8;
    cfg->max_pair_count = 0;
}

const char* spl_last_error_string(void) { return g_err.c_str(); }

int spl_compute_uniforms(const spl_config* cfg, const float camera_to_world[16], uint32_t width, uint32_t height,
                         void* out) {
    int rc = validate_config(cfg);
    if (rc) return rc;
    if (!camera_to_world || !out || width == 0 || height == 0) return fail(SPL_ERR_INVALID, "bad uniform arguments");
    Uniforms u;
    compute_uniforms(*cfg, camera_to_world, width, height, u);
    std::memcpy(out, &u, sizeof(u));
    return SPL_OK;
}

int spl_renderer_create(const spl_config* cfg, spl_renderer** out) {
    if (!out) return fail(SPL_ERR_INVALID, "out is NULL");
    *out = nullptr;
    int rc = validate_config(cfg);
    if (rc) return rc;
    spl_renderer* r = new (std::nothrow) spl_renderer();
    if (!r) return fail(SPL_ERR_OOM, "host allocation failed");
    r->cfg = *cfg;
    cudaGetDevice(&r->device);
    r->max_n = cfg->max_splat_count;
    uint64_t pc = cfg->max_pair_count;
    if (pc == 0) {
        pc = r->max_n * 16;
        if (pc < (1ull << 20)) pc = 1ull << 20;
        if (pc > MAX_COUNT) pc = MAX_COUNT;
    }
    r->pair_cap = pc;
    const uint64_t n = r->max_n;
#define TRY(x)           \
    do {                 \
        rc = (x);        \
        if (rc) {        \
            r->release(); \
            delete r;    \
            return rc;   \
        }                \
    } while (0)
    TRY(dalloc(&r->keys_a, n));
    TRY(dalloc(&r->keys_b, n));
    TRY(dalloc(&r->vals_a, n));
    TRY(dalloc(&r->vals_b, n));
    TRY(dalloc(&r->idx, n));
    TRY(dalloc(&r->rec, n * 4));
    TRY(dalloc(&r->boxes, n));
    TRY(dalloc(&r->st_cull, ceil_div(n, CULL_TILE)));
    TRY(dalloc(&r->st_bin, ceil_div(n, BIN_TILE)));
    TRY(dalloc(&r->pk_a, pc));
    TRY(dalloc(&r->pk_b, pc));
    TRY(dalloc(&r->pv_a, pc));
    TRY(dalloc(&r->pv_b, pc));
    TRY(dalloc(&r->fc, 1));
    TRY(dalloc(&r->fc_sort, 1));
    TRY(dalloc(&r->epoch, 1));
    TRY(dalloc(&r->d_u, 1));
    TRY(dalloc(&r->d_sv, 1));
    TRY(dalloc(&r->coop_cnt, 256 * (((size_t)sort_coop_grid() + 3) & ~(size_t)3) + 256));
#undef TRY
    cudaError_t e = cudaSuccess;
    // status words start at epoch 0, which no frame uses
    if (e == cudaSuccess) e = cudaMemset(r->st_cull, 0, ceil_div(n, CULL_TILE) * 8);
    if (e == cudaSuccess) e = cudaMemset(r->st_bin, 0, ceil_div(n, BIN_TILE) * 8);
    if (e == cudaSuccess) e = cudaMemset(r->fc, 0, sizeof(FrameCounters));
    if (e == cudaSuccess) e = cudaMemset(r->fc_sort, 0, sizeof(FrameCounters));
    if (e == cudaSuccess)
        e = cudaMemset(r->coop_cnt, 0, (256 * (((size_t)sort_coop_grid() + 3) & ~(size_t)3) + 256) * 4);
    if (e == cudaSuccess) e = cudaMemset(r->epoch, 0, 4);
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&r->host_fc), sizeof(FrameCounters));
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        cudaGetLastError();
        r->release();
        delete r;
        return fail(e == cudaErrorMemoryAllocation ? SPL_ERR_OOM : SPL_ERR_CUDA, "renderer setup: %s",
                    cudaGetErrorString(e));
    }
    *out = r;
    return SPL_OK;
}

void spl_renderer_destroy(spl_renderer* r) {
    if (!r) return;
    cudaDeviceSynchronize();
    drop_own_graph(r);
    r->release();
    delete r;
}

int spl_renderer_reserve(spl_renderer* r, uint32_t width, uint32_t height) {
    if (!r || width == 0 || height == 0 || width > 65535 || height > 65535)
        return fail(SPL_ERR_INVALID, "bad reserve arguments");
    const uint64_t tiles = ceil_div(width, TILE_PIXELS) * ceil_div(height, TILE_PIXELS);
    return ensure_ranges(r, tiles);
}

// One frame on `st`.  grid_n sizes the grids (the scene's count, or the renderer's maximum for a
// captured frame whose scene changes between launches: the kernels read the scene and every count
// from device memory).
static int render_frame_impl(spl_renderer* r, const SceneView& sv, const Uniforms& u, uint32_t width, uint32_t height,
                             void* out_device, cudaStream_t st, uint32_t grid_n) {
    const spl_config& cfg = r->cfg;
    const uint64_t tiles_x = ceil_div(width, TILE_PIXELS), tiles_y = ceil_div(height, TILE_PIXELS);
    const uint64_t tiles = tiles_x * tiles_y;
    if (tiles > r->ranges_cap) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
            return fail(SPL_ERR_INVALID, "call spl_renderer_reserve(%u, %u) before capturing a frame", width, height);
        int rc = ensure_ranges(r, tiles);
        if (rc) return rc;
    }
    const uint32_t N = grid_n;
    const int mode = cfg.depth_sorting;
    const uint32_t sl = r->spin_limit;

    const bool coop = r->sort_mode == SPL_SORT_COOPERATIVE;
    r->mark(0, st);
    launch_frame_begin(r->fc, r->epoch, u, r->d_u, sv, r->d_sv, st);
    launch_cull_key(mode, !coop, N, r->d_sv, r->d_u, r->fc, r->epoch, r->st_cull, r->keys_a, r->idx, sl, st);
    r->mark(1, st);
    launch_preprocess((int)cfg.spherical_harmonics_order, cfg.use_covariance_for_scale != 0,
                      cfg.use_unaligned_rectangles != 0, r->d_sv, r->d_u, r->idx, r->fc, r->rec, r->boxes, N, st);
    r->mark(2, st);
    const uint32_t* order = nullptr;
    if (mode != DS_NONE && N > 0) {
        // four stable 8-bit passes a -> b -> a -> b -> a; pass 0 takes the compaction slot as the value
        if (coop) {
            CU(launch_sort_coop(r->keys_a, r->keys_b, r->vals_a, r->vals_b, true, &r->fc->visible, N, 4, 0,
                                r->coop_cnt, r->fc->barrier, sl, &r->fc->err, st));
        } else {
            // digit histograms from the cull kernel; one launch per pass
            uint32_t *src_k = r->keys_a, *dst_k = r->keys_b, *dst_v = r->vals_b;
            const uint32_t* src_v = nullptr;
            const uint64_t stride = r->sort_tiles() * 256;
            for (int p = 0; p < 4; ++p) {
                launch_onesweep(src_k, src_v, dst_k, dst_v, &r->fc->visible, N, r->fc->hist_depth[p],
                                r->st_sort + p * stride, &r->fc->tile_counter[1 + p], r->epoch, 8 * p, sl,
                                &r->fc->err, st);
                uint32_t* next_k = dst_k == r->keys_b ? r->keys_a : r->keys_b;
                uint32_t* next_v = dst_v == r->vals_b ? r->vals_a : r->vals_b;
                src_k = dst_k;
                src_v = dst_v;
                dst_k = next_k;
                dst_v = next_v;
            }
        }
        order = r->vals_a;  // keys in keys_a
    }
    r->mark(3, st);
    CU(cudaMemsetAsync(r->ranges, 0, tiles * sizeof(uint2), st));
    launch_bin(mode, !coop, order, r->boxes, r->fc, r->epoch, r->st_bin, r->pk_a, r->pv_a, (uint32_t)r->pair_cap,
               (int)tiles_x, N, sl, st);
    r->mark(4, st);
    // stable sort of the pairs by tile id keeps each tile's list in depth order
    const int passes = tiles <= 256 ? 1 : (tiles <= 65536 ? 2 : 3);
    if (coop) {
        CU(launch_sort_coop(r->pk_a, r->pk_b, r->pv_a, r->pv_b, false, &r->fc->pairs, (uint32_t)r->pair_cap, passes,
                            0, r->coop_cnt, r->fc->barrier + 1, sl, &r->fc->err, st));
    } else {
        // tile-id histograms from the binning kernel
        uint32_t *ak = r->pk_a, *av = r->pv_a, *bk = r->pk_b, *bv = r->pv_b;
        const uint64_t pstride = r->pair_tiles() * 256;
        for (int p = 0; p < passes; ++p) {
            launch_onesweep(ak, av, bk, bv, &r->fc->pairs, (uint32_t)r->pair_cap, r->fc->hist_pairs[p],
                            r->st_pairs + p * pstride, &r->fc->tile_counter[5 + p], r->epoch, 8 * p, sl, &r->fc->err,
                            st);
            std::swap(ak, bk);
            std::swap(av, bv);
        }
    }
    const uint32_t* pk = (passes & 1) ? r->pk_b : r->pk_a;
    const uint32_t* pv = (passes & 1) ? r->pv_b : r->pv_a;
    r->mark(5, st);
    launch_tile_ranges(pk, r->fc, (uint32_t)r->pair_cap, r->ranges, st);
    r->mark(6, st);
    launch_raster(cfg.use_unaligned_rectangles != 0, cfg.blend_mode, r->ranges, r->order_tiles ? r->tile_order : nullptr,
                  pv, r->rec, u, out_device, st);
    r->mark(7, st);
    CU(cudaGetLastError());
    r->final_pair_vals = pv;
    return SPL_OK;
}

int spl_render_frame_motor(spl_renderer* r, const spl_scene* scene, const float motor[8], uint32_t width,
                           uint32_t height, void* out_device, void* stream) {
    if (!motor) return fail(SPL_ERR_INVALID, "NULL argument");
    float cam[16];
    const int rc = spl_motor_to_mat4(motor, cam);  // renderer.rs:364
    if (rc) return rc;
    return spl_render_frame(r, scene, cam, width, height, out_device, stream);
}

static int frame_graph_replay(spl_frame_graph* g, const spl_scene* scene, const float camera_to_world[16],
                              void* out_device, cudaStream_t st);
static bool own_graph_matches(const spl_renderer* r, uint32_t w, uint32_t h, uint64_t n);

int spl_render_frame(spl_renderer* r, const spl_scene* scene, const float camera_to_world[16], uint32_t width,
                     uint32_t height, void* out_device, void* stream) {
    if (!r || !scene || !camera_to_world || !out_device) return fail(SPL_ERR_INVALID, "NULL argument");
    if (width == 0 || height == 0 || width > 65535 || height > 65535)
        return fail(SPL_ERR_INVALID, "viewport %ux%u outside [1, 65535]", width, height);
    if (scene->n > r->max_n) return fail(SPL_ERR_INVALID, "scene larger than the renderer's max_splat_count");
    cudaStream_t st = (cudaStream_t)stream;
    // The second frame in a row of the same viewport and scene size is captured into a frame graph
    // (grids sized for the scene, exactly as the direct launches), and frames of that key replay it:
    // one graph launch instead of a launch per kernel.  Not while profiling (the stage events are
    // direct launches) or while the caller's stream is being captured.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const bool capturing = cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone;
    if (r->frame_graphs && !r->profiling && !capturing && scene->n > 0) {
        if (!own_graph_matches(r, width, height, scene->n) && r->seen_w == width && r->seen_h == height &&
            r->seen_n == scene->n) {
            drop_own_graph(r);
            spl_frame_graph* g = nullptr;
            const int rc = spl_frame_graph_create(r, width, height, scene->n, out_device, &g);
            if (rc) return rc;
            r->own_graph = g;
        }
        if (own_graph_matches(r, width, height, scene->n))
            return frame_graph_replay(r->own_graph, scene, camera_to_world, out_device, st);
    }
    Uniforms u;
    compute_uniforms(r->cfg, camera_to_world, width, height, u);
    const int rc = render_frame_impl(r, scene->view(), u, width, height, out_device, st, (uint32_t)scene->n);
    if (rc) return rc;
    r->seen_w = width;
    r->seen_h = height;
    r->seen_n = scene->n;
    r->last_stream = st;
    r->last_scene = scene;
    r->last_u = u;
    r->has_frame = true;
    r->last_w = width;
    r->last_h = height;
    r->last_n = scene->n;
    return SPL_OK;
}

int spl_renderer_set_frame_graphs(spl_renderer* r, int enable) {
    if (!r) return fail(SPL_ERR_INVALID, "NULL argument");
    r->frame_graphs = enable != 0;
    if (!r->frame_graphs) drop_own_graph(r);
    return SPL_OK;
}

int spl_renderer_set_sort_mode(spl_renderer* r, int mode) {
    if (!r) return fail(SPL_ERR_INVALID, "NULL argument");
    if (mode != SPL_SORT_COOPERATIVE && mode != SPL_SORT_ONESWEEP) return fail(SPL_ERR_INVALID, "sort mode %d", mode);
    if (mode == SPL_SORT_ONESWEEP && !r->st_sort) {
        const uint64_t ns = r->sort_tiles() * 256 * 4, np = r->pair_tiles() * 256 * 3;
        int rc = dalloc(&r->st_sort, ns);
        if (rc) return rc;
        rc = dalloc(&r->st_pairs, np);
        if (rc) {
            dfree(r->st_sort);
            return rc;
        }
        // status words start at epoch 0, which no frame uses
        CU(cudaMemset(r->st_sort, 0, ns * 8));
        CU(cudaMemset(r->st_pairs, 0, np * 8));
        CU(cudaDeviceSynchronize());
        onesweep_prepare();
    }
    if (mode != r->sort_mode) drop_own_graph(r);  // its sorts are the other algorithm's
    r->sort_mode = mode;
    return SPL_OK;
}

int spl_renderer_set_profiling(spl_renderer* r, int enable) {
    if (!r) return fail(SPL_ERR_INVALID, "NULL argument");
    if (enable) {
        for (auto& e : r->ev_prof)
            if (!e) CU(cudaEventCreate(&e));
    }
    r->profiling = enable != 0;
    return SPL_OK;
}

int spl_renderer_stage_times(spl_renderer* r, float* ms, int count) {
    if (!r || !ms || count < SPL_STAGE_COUNT) return fail(SPL_ERR_INVALID, "need %d outputs", SPL_STAGE_COUNT);
    if (!r->profiling || !r->has_frame) return fail(SPL_ERR_INVALID, "profiling is off or no frame rendered");
    CU(cudaEventSynchronize(r->ev_prof[7]));
    auto el = [&](int a, int b, float* out) -> cudaError_t { return cudaEventElapsedTime(out, r->ev_prof[a], r->ev_prof[b]); };
    CU(el(0, 1, &ms[SPL_STAGE_CULL]));
    CU(el(1, 2, &ms[SPL_STAGE_PREPROCESS]));
    CU(el(2, 3, &ms[SPL_STAGE_DEPTH_SORT]));
    CU(el(3, 4, &ms[SPL_STAGE_BIN]));
    CU(el(4, 5, &ms[SPL_STAGE_PAIR_SORT]));
    CU(el(5, 6, &ms[SPL_STAGE_RANGES]));
    CU(el(6, 7, &ms[SPL_STAGE_RASTER]));
    CU(el(0, 7, &ms[SPL_STAGE_FRAME]));
    return SPL_OK;
}

int spl_renderer_launches_per_frame(const spl_renderer* r, uint32_t width, uint32_t height) {
    if (!r) return 0;
    const uint64_t tiles = ceil_div(width, TILE_PIXELS) * ceil_div(height, TILE_PIXELS);
    const int pair_passes = tiles <= 256 ? 1 : (tiles <= 65536 ? 2 : 3);
    const bool coop = r->sort_mode == SPL_SORT_COOPERATIVE;
    const int depth_sort = r->cfg.depth_sorting == DS_NONE ? 0 : (coop ? 1 : 4);
    // frame_begin, cull, preprocess, depth sort (one cooperative launch or 4 onesweep passes),
    // ranges memset, bin, pair sort (one cooperative launch or one launch per pass), ranges, tile
    // order, raster
    return 1 + 1 + 1 + depth_sort + 1 + 1 + (coop ? 1 : pair_passes) + 1 + (r->order_tiles ? 1 : 0) + 1;
}

static int render_backward(spl_renderer* r, const spl_scene* scene, const float* image_device,
                           const float* grad_image_device, float* grad_x, float* grad_y, float* grad_z,
                           float* grad_rotation, float* grad_scale_alpha, float* grad_sh, void* stream, bool accumulate) {
    if (!r || !scene || !image_device || !grad_image_device || !grad_x || !grad_y || !grad_z || !grad_rotation ||
        !grad_scale_alpha || !grad_sh)
        return fail(SPL_ERR_INVALID, "NULL argument");
    if ((reinterpret_cast<uintptr_t>(grad_rotation) | reinterpret_cast<uintptr_t>(grad_scale_alpha) |
         reinterpret_cast<uintptr_t>(grad_sh)) & 15u)
        return fail(SPL_ERR_INVALID, "grad_rotation, grad_scale_alpha and grad_sh must be 16-byte aligned");
    if (r->cfg.blend_mode != SPL_BLEND_FP32) return fail(SPL_ERR_INVALID, "the backward pass needs blend_mode FP32");
    if (!r->has_frame || r->last_scene != scene)
        return fail(SPL_ERR_INVALID, "render this scene with spl_render_frame first (the backward reuses that frame)");
    if (!r->grad_rec) {
        int rc = dalloc(&r->grad_rec, r->max_n * 10);
        if (!rc) rc = dalloc(&r->grad_deferred, r->max_n + 1);
        if (rc) {
            dfree(r->grad_rec);
            return rc;
        }
    }
    cudaStream_t st = (cudaStream_t)stream;
    const spl_config& cfg = r->cfg;
    launch_backward((int)cfg.spherical_harmonics_order, cfg.use_covariance_for_scale != 0,
                    cfg.use_unaligned_rectangles != 0, scene->view(), r->last_u, r->idx, r->fc, r->boxes, r->ranges,
                    r->order_tiles ? r->tile_order : nullptr, r->final_pair_vals, r->rec, reinterpret_cast<const float4*>(image_device),
                    reinterpret_cast<const float4*>(grad_image_device), r->grad_rec, r->grad_deferred, (uint32_t)scene->n, grad_x,
                    grad_y, grad_z, reinterpret_cast<float4*>(grad_rotation), reinterpret_cast<float4*>(grad_scale_alpha),
                    grad_sh, accumulate, st);
    CU(cudaGetLastError());
    return SPL_OK;
}

int spl_render_backward(spl_renderer* r, const spl_scene* scene, const float* image_device,
                        const float* grad_image_device, float* grad_x, float* grad_y, float* grad_z, float* grad_rotation,
                        float* grad_scale_alpha, float* grad_sh, void* stream) {
    return render_backward(r, scene, image_device, grad_image_device, grad_x, grad_y, grad_z, grad_rotation,
                           grad_scale_alpha, grad_sh, stream, false);
}

int spl_render_backward_accumulate(spl_renderer* r, const spl_scene* scene, const float* image_device,
                                   const float* grad_image_device, float* grad_x, float* grad_y, float* grad_z,
                                   float* grad_rotation, float* grad_scale_alpha, float* grad_sh, void* stream) {
    return render_backward(r, scene, image_device, grad_image_device, grad_x, grad_y, grad_z, grad_rotation,
                           grad_scale_alpha, grad_sh, stream, true);
}

int spl_renderer_copy_record_gradients(spl_renderer* r, float* dst_device, uint64_t capacity, void* stream) {
    if (!r || !dst_device) return fail(SPL_ERR_INVALID, "NULL argument");
    if (!r->grad_rec) return fail(SPL_ERR_INVALID, "no backward pass has run on this renderer");
    if (capacity > r->max_n) capacity = r->max_n;
    if (capacity == 0) return SPL_OK;
    CU(cudaMemcpyAsync(dst_device, r->grad_rec, capacity * 40, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return SPL_OK;
}

int spl_renderer_frame_info(spl_renderer* r, spl_frame_info* info) {
    if (!r || !info) return fail(SPL_ERR_INVALID, "NULL argument");
    std::memset(info, 0, sizeof(*info));
    if (!r->has_frame) return fail(SPL_ERR_INVALID, "no frame rendered yet");
    CU(cudaMemcpyAsync(r->host_fc, r->fc, sizeof(FrameCounters), cudaMemcpyDeviceToHost, r->last_stream));
    CU(cudaStreamSynchronize(r->last_stream));
    const FrameCounters& f = *r->host_fc;
    info->splat_count = r->last_n;
    info->visible_count = f.visible;
    info->draw_count = f.draw;
    info->pair_count = f.pairs;
    info->device_error = f.err;
    info->width = r->last_w;
    info->height = r->last_h;
    if (f.err & SPL_DEV_ERR_LOOKBACK) return fail(SPL_ERR_LOOKBACK_TIMEOUT, "a decoupled look-back wait timed out");
    if (f.err & SPL_DEV_ERR_PAIR_OVERFLOW)
        return fail(SPL_ERR_CAPACITY, "tile binning needs %u pairs, capacity %llu", f.pairs,
                    (unsigned long long)r->pair_cap);
    return SPL_OK;
}

int spl_renderer_copy_entries(spl_renderer* r, uint32_t* keys_device, uint32_t* indices_device, uint64_t capacity,
                              void* stream) {
    if (!r || !keys_device || !indices_device) return fail(SPL_ERR_INVALID, "NULL argument");
    if (!r->has_frame) return fail(SPL_ERR_INVALID, "no frame rendered yet");
    if (capacity > r->max_n) capacity = r->max_n;
    const bool sorted = r->cfg.depth_sorting != DS_NONE;
    launch_gather_entries(r->keys_a, sorted ? r->vals_a : nullptr, r->idx, r->fc, r->cfg.depth_sorting, keys_device,
                          indices_device, (uint32_t)capacity, (cudaStream_t)stream);
    CU(cudaGetLastError());
    return SPL_OK;
}

int spl_renderer_copy_records(spl_renderer* r, float* records_device, uint64_t capacity, void* stream) {
    if (!r || !records_device) return fail(SPL_ERR_INVALID, "NULL argument");
    if (capacity > r->max_n) capacity = r->max_n;
    if (capacity == 0) return SPL_OK;
    CU(cudaMemcpyAsync(records_device, r->rec, capacity * 64, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return SPL_OK;
}

int spl_sort_pairs(spl_renderer* r, const uint32_t* keys_in, const uint32_t* values_in, uint32_t* keys_out,
                   uint32_t* values_out, uint64_t count, uint32_t key_bits, void* stream) {
    if (!r || !keys_in || !values_in || !keys_out || !values_out) return fail(SPL_ERR_INVALID, "NULL argument");
    if (count > r->max_n) return fail(SPL_ERR_INVALID, "count %llu above max_splat_count", (unsigned long long)count);
    if (key_bits == 0 || key_bits > 32 || key_bits % 8 != 0) return fail(SPL_ERR_INVALID, "key_bits %u", key_bits);
    cudaStream_t st = (cudaStream_t)stream;
    if (count == 0) return SPL_OK;
    const int passes = (int)(key_bits / 8);
    launch_frame_begin(r->fc_sort, r->epoch, st);
    launch_set_count(&r->fc_sort->visible, (uint32_t)count, st);
    CU(cudaMemcpyAsync(r->keys_a, keys_in, count * 4, cudaMemcpyDeviceToDevice, st));
    CU(cudaMemcpyAsync(r->vals_a, values_in, count * 4, cudaMemcpyDeviceToDevice, st));
    CU(launch_sort_coop(r->keys_a, r->keys_b, r->vals_a, r->vals_b, false, &r->fc_sort->visible, (uint32_t)count,
                        passes, 0, r->coop_cnt, r->fc_sort->barrier, r->spin_limit, &r->fc_sort->err, st));
    const uint32_t* kr = (passes & 1) ? r->keys_b : r->keys_a;
    const uint32_t* vr = (passes & 1) ? r->vals_b : r->vals_a;
    CU(cudaMemcpyAsync(keys_out, kr, count * 4, cudaMemcpyDeviceToDevice, st));
    CU(cudaMemcpyAsync(values_out, vr, count * 4, cudaMemcpyDeviceToDevice, st));
    return SPL_OK;
}

int spl_debug_lookback_timeout(uint32_t spin_limit, int* timed_out) {
    if (!timed_out) return fail(SPL_ERR_INVALID, "NULL argument");
    *timed_out = 0;
    uint64_t* status = nullptr;
    uint32_t* words = nullptr;
    int rc = dalloc(&status, 64);
    if (rc) return rc;
    rc = dalloc(&words, 4);
    if (rc) {
        dfree(status);
        return rc;
    }
    uint32_t host[4] = {0, 0, 0, 0};
    cudaError_t e = cudaMemset(status, 0, 64 * 8);
    if (e == cudaSuccess) e = cudaMemset(words, 0, 16);
    if (e == cudaSuccess) {
        launch_lookback_probe(status, words, spin_limit, words + 2, nullptr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(host, words, 16, cudaMemcpyDeviceToHost);
    dfree(status);
    dfree(words);
    if (e != cudaSuccess) return fail(SPL_ERR_CUDA, "look-back probe: %s", cudaGetErrorString(e));
    *timed_out = (host[3] & SPL_DEV_ERR_LOOKBACK) ? 1 : 0;
    return SPL_OK;
}

// ---- scenes ----------------------------------------------------------------------------------------

int spl_scene_create(spl_renderer* r, uint64_t splat_count, spl_scene** out, uint64_t* clamped_count) {
    if (!r || !out) return fail(SPL_ERR_INVALID, "NULL argument");
    *out = nullptr;
    spl_scene* s = new (std::nothrow) spl_scene();
    if (!s) return fail(SPL_ERR_OOM, "host allocation failed");
    s->renderer = r;
    cudaGetDevice(&s->device);
    s->n = splat_count < r->max_n ? splat_count : r->max_n;  // scene.rs:46
    const uint64_t n = s->n;
    int rc = SPL_OK;
    if (!rc) rc = dalloc(&s->x, n);
    if (!rc) rc = dalloc(&s->y, n);
    if (!rc) rc = dalloc(&s->z, n);
    if (!rc) rc = dalloc(&s->rot, n);
    if (!rc) rc = dalloc(&s->scale_alpha, n);
    if (!rc) rc = dalloc(&s->sh, n * 48);
    if (rc) {
        s->release();
        delete s;
        return rc;
    }
    // zeroed like a fresh wgpu buffer
    cudaError_t e = cudaSuccess;
    if (n) {
        e = cudaMemset(s->x, 0, n * 4);
        if (e == cudaSuccess) e = cudaMemset(s->y, 0, n * 4);
        if (e == cudaSuccess) e = cudaMemset(s->z, 0, n * 4);
        if (e == cudaSuccess) e = cudaMemset(s->rot, 0, n * 16);
        if (e == cudaSuccess) e = cudaMemset(s->scale_alpha, 0, n * 16);
        if (e == cudaSuccess) e = cudaMemset(s->sh, 0, n * 192);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) {
        s->release();
        delete s;
        return fail(SPL_ERR_CUDA, "scene setup: %s", cudaGetErrorString(e));
    }
    *out = s;
    if (clamped_count) *clamped_count = n;
    return SPL_OK;
}

void spl_scene_destroy(spl_scene* s) {
    if (!s) return;
    cudaDeviceSynchronize();
    s->release();
    delete s;
}

uint64_t spl_scene_splat_count(const spl_scene* s) { return s ? s->n : 0; }

int spl_scene_wrap(spl_renderer* r, uint64_t splat_count, float* x, float* y, float* z, float* rotation,
                   float* scale_alpha, float* sh, spl_scene** out) {
    if (!r || !out || !x || !y || !z || !rotation || !scale_alpha || !sh) return fail(SPL_ERR_INVALID, "NULL argument");
    if (splat_count > r->max_n) return fail(SPL_ERR_INVALID, "splat_count above max_splat_count");
    if ((reinterpret_cast<uintptr_t>(rotation) | reinterpret_cast<uintptr_t>(scale_alpha) |
         reinterpret_cast<uintptr_t>(sh)) & 15u)
        return fail(SPL_ERR_INVALID, "rotation, scale_alpha and sh must be 16-byte aligned");
    spl_scene* s = new (std::nothrow) spl_scene();
    if (!s) return fail(SPL_ERR_OOM, "host allocation failed");
    s->renderer = r;
    cudaGetDevice(&s->device);
    s->n = splat_count;
    s->owns = false;
    s->x = x;
    s->y = y;
    s->z = z;
    s->rot = reinterpret_cast<float4*>(rotation);
    s->scale_alpha = reinterpret_cast<float4*>(scale_alpha);
    s->sh = sh;
    *out = s;
    return SPL_OK;
}
uint64_t spl_scene_device_bytes(const spl_scene* s) { return s ? s->n * 236ull : 0; }

int spl_scene_load_chunk(spl_scene* s, const void* records, uint64_t start, uint64_t count, void* stream) {
    if (!s || (!records && count)) return fail(SPL_ERR_INVALID, "NULL argument");
    if (start >= s->n) return SPL_OK;
    if (count > s->n - start) count = s->n - start;  // scene.rs:217
    const float* src = static_cast<const float*>(records);
    return staged_upload(
        s, start, count, 62, (cudaStream_t)stream,
        [&](float* dst, uint64_t first, uint64_t cnt) {
            std::memcpy(dst, src + (first - start) * 62, cnt * 248);
            return SPL_OK;
        },
        [&](float* dev, uint64_t first, uint64_t cnt, cudaStream_t st) {
            launch_load_records(dev, (uint32_t)cnt, s->x + first, s->y + first, s->z + first, s->rot + first,
                                s->scale_alpha + first, s->sh + first * 48, st);
        });
}

int spl_scene_load_chunk_file(spl_scene* s, const char* path, uint32_t header_bytes, uint64_t start, uint64_t count,
                              void* stream) {
    if (!s || !path) return fail(SPL_ERR_INVALID, "NULL argument");
    if (start >= s->n) return SPL_OK;
    if (count > s->n - start) count = s->n - start;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(SPL_ERR_IO, "cannot open %s", path);
    const int rc = load_file_range(s, f, path, header_bytes, start, count, (cudaStream_t)stream);
    std::fclose(f);
    return rc;
}

// ---- progressive loading (showcase.rs:13,54-59,98-103) ----------------------------------------------
struct spl_progressive_loader {
    spl_scene* s = nullptr;
    FILE* f = nullptr;
    std::string path;
    uint32_t header_bytes = 0;
    uint64_t chunk = 0;       // splats per step (0: the whole scene in one step)
    uint64_t chunks_left = 0;
};

int spl_progressive_loader_create(spl_scene* s, const char* path, uint32_t header_bytes, uint64_t chunk_size,
                                  spl_progressive_loader** out) {
    if (!s || !path || !out) return fail(SPL_ERR_INVALID, "NULL argument");
    *out = nullptr;
    auto* l = new (std::nothrow) spl_progressive_loader();
    if (!l) return fail(SPL_ERR_OOM, "host allocation failed");
    l->f = std::fopen(path, "rb");
    if (!l->f) {
        delete l;
        return fail(SPL_ERR_IO, "cannot open %s", path);
    }
    l->s = s;
    l->path = path;
    l->header_bytes = header_bytes;
    l->chunk = chunk_size == 0 ? s->n : chunk_size;
    l->chunks_left = l->chunk == 0 ? 0 : (s->n + l->chunk - 1) / l->chunk;  // showcase.rs:54-59
    *out = l;
    return SPL_OK;
}

int spl_progressive_loader_step(spl_progressive_loader* l, void* stream, uint64_t* chunks_left) {
    if (!l) return fail(SPL_ERR_INVALID, "NULL argument");
    if (l->chunks_left > 0) {
        // the last chunk not yet loaded (showcase.rs:98-101), clamped to the scene (scene.rs:217)
        const uint64_t k = l->chunks_left - 1;
        const uint64_t start = k * l->chunk;
        const uint64_t count = std::min(l->chunk, l->s->n - start);
        const int rc = load_file_range(l->s, l->f, l->path.c_str(), l->header_bytes, start, count, (cudaStream_t)stream);
        if (rc) return rc;
        l->chunks_left = k;
    }
    if (chunks_left) *chunks_left = l->chunks_left;
    return SPL_OK;
}

void spl_progressive_loader_destroy(spl_progressive_loader* l) {
    if (!l) return;
    if (l->f) std::fclose(l->f);
    delete l;
}

int spl_scene_write_splats(spl_scene* s, const float* splats60, uint64_t start, uint64_t count, void* stream) {
    if (!s || (!splats60 && count)) return fail(SPL_ERR_INVALID, "NULL argument");
    if (start >= s->n) return SPL_OK;
    if (count > s->n - start) count = s->n - start;
    return staged_upload(
        s, start, count, 60, (cudaStream_t)stream,
        [&](float* dst, uint64_t first, uint64_t cnt) {
            std::memcpy(dst, splats60 + (first - start) * 60, cnt * 240);
            return SPL_OK;
        },
        [&](float* dev, uint64_t first, uint64_t cnt, cudaStream_t st) {
            launch_splats60_to_soa(dev, (uint32_t)cnt, s->x + first, s->y + first, s->z + first, s->rot + first,
                                   s->scale_alpha + first, s->sh + first * 48, st);
        });
}

int spl_scene_read_splats(const spl_scene* cs, float* splats60, uint64_t start, uint64_t count) {
    spl_scene* s = const_cast<spl_scene*>(cs);
    if (!s || (!splats60 && count)) return fail(SPL_ERR_INVALID, "NULL argument");
    if (start > s->n || count > s->n - start) return fail(SPL_ERR_INVALID, "range outside the scene");
    std::lock_guard<std::mutex> lk(s->stg_mu);
    int rc = ensure_staging(s);
    if (rc) return rc;
    CU(cudaDeviceSynchronize());
    uint64_t done = 0;
    while (done < count) {
        const uint64_t cnt = (count - done) < CHUNK_RECORDS ? (count - done) : CHUNK_RECORDS;
        launch_soa_to_splats60(s->view(), (uint32_t)(start + done), (uint32_t)cnt, s->stg.dev[0], nullptr);
        CU(cudaGetLastError());
        CU(cudaMemcpy(splats60 + done * 60, s->stg.dev[0], cnt * 240, cudaMemcpyDeviceToHost));
        done += cnt;
    }
    return SPL_OK;
}

int spl_scene_create_dev_test(spl_renderer* r, spl_scene** out) {
    int rc = spl_scene_create(r, 3, out, nullptr);
    if (rc) return rc;
    float d[3][60];
    std::memset(d, 0, sizeof(d));
    for (int i = 0; i < 3; ++i) {  // scene.rs:162-177
        d[i][0] = 1.0f;
        d[i][4] = i == 0 ? 1.0f : 0.0f;
        d[i][5] = i == 1 ? 1.0f : 0.0f;
        d[i][6] = i == 2 ? 1.0f : 0.0f;
        d[i][8] = 0.2f;
        d[i][9] = 0.1f;
        d[i][10] = 0.05f;
        d[i][11] = 1.0f;
        d[i][12] = i == 0 ? 1.0f : 0.0f;
        d[i][13] = i == 1 ? 1.0f : 0.0f;
        d[i][14] = i == 2 ? 1.0f : 0.0f;
    }
    const uint64_t n = (*out)->n < 3 ? (*out)->n : 3;
    rc = spl_scene_write_splats(*out, &d[0][0], 0, n, nullptr);
    if (rc == SPL_OK) {
        cudaError_t e = cudaStreamSynchronize(nullptr);
        if (e != cudaSuccess) rc = fail(SPL_ERR_CUDA, "dev test upload: %s", cudaGetErrorString(e));
    }
    if (rc) {
        spl_scene_destroy(*out);
        *out = nullptr;
    }
    return rc;
}

int spl_parse_file_header(const char* path, uint32_t* header_bytes, uint64_t* splat_count) {
    if (!path || !header_bytes || !splat_count) return fail(SPL_ERR_INVALID, "NULL argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(SPL_ERR_IO, "cannot open %s", path);
    char line[4096];
    uint64_t count = 0;
    bool ended = false;
    uint64_t pos = 0;
    while (std::fgets(line, sizeof(line), f)) {  // scene.rs:201-210
        pos += std::strlen(line);
        if (std::strcmp(line, "end_header\n") == 0) {
            ended = true;
            break;
        }
        if (std::strncmp(line, "element vertex ", 15) == 0) {
            char* endp = nullptr;
            const unsigned long long v = std::strtoull(line + 15, &endp, 10);
            if (endp == line + 15 || (*endp != '\n' && *endp != '\0')) {
                std::fclose(f);
                return fail(SPL_ERR_IO, "malformed element vertex line in %s", path);
            }
            count = v;
        }
    }
    std::fclose(f);
    if (!ended) return fail(SPL_ERR_IO, "no end_header in %s", path);
    if (pos > 0xFFFFFFFFull) return fail(SPL_ERR_IO, "header too long in %s", path);
    *header_bytes = (uint32_t)pos;
    *splat_count = count;
    return SPL_OK;
}

// ---- captured frames ----------------------------------------------------------------------------
struct spl_frame_graph {
    spl_renderer* r = nullptr;
    uint32_t w = 0, h = 0;
    uint64_t max_splats = 0;  // the grids' bound
    uint32_t generation = 0;  // the renderer's scratch generation the graph was captured with
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t begin_node = nullptr;  // k_frame_begin: the node whose parameters carry camera and scene
    cudaKernelNodeParams begin_params{};
    cudaGraphNode_t raster_node = nullptr;  // the raster: its output pointer can be re-targeted
    cudaKernelNodeParams raster_params{};
    void* out = nullptr;  // the output the raster node writes now
    const uint32_t* final_pair_vals = nullptr;
};

static void drop_own_graph(spl_renderer* r) {
    if (r->own_graph) spl_frame_graph_destroy(r->own_graph);  // an exec in flight is freed when it completes
    r->own_graph = nullptr;
}

static bool own_graph_matches(const spl_renderer* r, uint32_t w, uint32_t h, uint64_t n) {
    const spl_frame_graph* g = r->own_graph;
    return g && g->w == w && g->h == h && g->max_splats == n && g->generation == r->scratch_generation;
}

void spl_frame_graph_destroy(spl_frame_graph* g) {
    if (!g) return;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
}

int spl_frame_graph_create(spl_renderer* r, uint32_t width, uint32_t height, uint64_t max_splats, void* out_device,
                           spl_frame_graph** out) {
    if (!r || !out_device || !out) return fail(SPL_ERR_INVALID, "NULL argument");
    *out = nullptr;
    if (max_splats == 0 || max_splats > r->max_n) max_splats = r->max_n;
    if (width == 0 || height == 0 || width > 65535 || height > 65535)
        return fail(SPL_ERR_INVALID, "viewport %ux%u outside [1, 65535]", width, height);
    if (r->profiling) return fail(SPL_ERR_INVALID, "turn profiling off before capturing a frame");
    int rc = spl_renderer_reserve(r, width, height);
    if (rc) return rc;
    spl_frame_graph* g = new (std::nothrow) spl_frame_graph();
    if (!g) return fail(SPL_ERR_OOM, "host allocation failed");
    g->r = r;
    g->w = width;
    g->h = height;
    g->max_splats = max_splats;
    g->generation = r->scratch_generation;
    g->out = out_device;
    cudaStream_t cs = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete g;
        return fail(SPL_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    // The uniform block of this viewport with a placeholder pose: the raster's parameters (viewport,
    // pixel size, margin) are taken from it on the host and baked into the graph; every launch
    // replaces the whole block on the device (camera included) and the scene view.
    const float pose[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, -5, 1};
    Uniforms u;
    compute_uniforms(r->cfg, pose, width, height, u);
    const SceneView sv{};
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        rc = render_frame_impl(r, sv, u, width, height, out_device, cs, (uint32_t)max_splats);
        const cudaError_t e2 = cudaStreamEndCapture(cs, &g->graph);
        if (!rc && e2 != cudaSuccess) rc = fail(SPL_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e2));
    } else {
        rc = fail(SPL_ERR_CUDA, "cudaStreamBeginCapture: %s", cudaGetErrorString(e));
    }
    cudaStreamDestroy(cs);
    if (!rc) {
        g->final_pair_vals = r->final_pair_vals;
        size_t nn = 0;
        e = cudaGraphGetNodes(g->graph, nullptr, &nn);
        std::vector<cudaGraphNode_t> nodes(nn);
        if (e == cudaSuccess && nn) e = cudaGraphGetNodes(g->graph, nodes.data(), &nn);
        const void* raster = raster_kernel(r->cfg.use_unaligned_rectangles != 0, r->cfg.blend_mode);
        for (size_t i = 0; e == cudaSuccess && i < nn; ++i) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[i], &t) != cudaSuccess || t != cudaGraphNodeTypeKernel) continue;
            cudaKernelNodeParams kp{};
            if (cudaGraphKernelNodeGetParams(nodes[i], &kp) != cudaSuccess) continue;
            if (kp.func == frame_begin_kernel()) {
                g->begin_node = nodes[i];
                g->begin_params = kp;
            } else if (kp.func == raster) {
                g->raster_node = nodes[i];
                g->raster_params = kp;
            }
        }
        if (e != cudaSuccess) rc = fail(SPL_ERR_CUDA, "cudaGraphGetNodes: %s", cudaGetErrorString(e));
        else if (!g->begin_node) rc = fail(SPL_ERR_CUDA, "captured frame has no frame-begin node");
        else if (!g->raster_node) rc = fail(SPL_ERR_CUDA, "captured frame has no raster node");
    }
    if (!rc) {
        e = cudaGraphInstantiate(&g->exec, g->graph, 0);
        if (e != cudaSuccess) rc = fail(SPL_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    }
    cudaGetLastError();
    if (rc) {
        spl_frame_graph_destroy(g);
        return rc;
    }
    *out = g;
    return SPL_OK;
}

// One replay of a captured frame: the first node takes the camera and the scene, the raster node
// the output when it differs from the one it writes now.
static int frame_graph_replay(spl_frame_graph* g, const spl_scene* scene, const float camera_to_world[16],
                              void* out_device, cudaStream_t st) {
    spl_renderer* r = g->r;
    if (g->generation != r->scratch_generation)
        return fail(SPL_ERR_INVALID, "the renderer's viewport scratch was reallocated (a larger frame): recreate the graph");
    Uniforms u;
    compute_uniforms(r->cfg, camera_to_world, g->w, g->h, u);
    SceneView sv = scene->view();
    FrameCounters* fc = r->fc;
    uint32_t* ep = r->epoch;
    Uniforms* du = r->d_u;
    SceneView* dsv = r->d_sv;
    void* args[6] = {&fc, &ep, &u, &du, &sv, &dsv};
    cudaKernelNodeParams kp = g->begin_params;
    kp.kernelParams = args;
    kp.extra = nullptr;
    CU(cudaGraphExecKernelNodeSetParams(g->exec, g->begin_node, &kp));
    if (out_device != g->out) {
        // the other arguments keep their captured values (the graph node holds them)
        void* rargs[RASTER_OUT_ARG + 1];
        for (int i = 0; i < RASTER_OUT_ARG; ++i) rargs[i] = g->raster_params.kernelParams[i];
        void* out = out_device;
        rargs[RASTER_OUT_ARG] = &out;
        cudaKernelNodeParams rp = g->raster_params;
        rp.kernelParams = rargs;
        rp.extra = nullptr;
        CU(cudaGraphExecKernelNodeSetParams(g->exec, g->raster_node, &rp));
        g->out = out_device;
    }
    CU(cudaGraphLaunch(g->exec, st));
    r->last_stream = st;
    r->last_scene = scene;
    r->last_u = u;
    r->has_frame = true;
    r->last_w = g->w;
    r->last_h = g->h;
    r->last_n = scene->n;
    r->final_pair_vals = g->final_pair_vals;
    return SPL_OK;
}

int spl_frame_graph_launch(spl_frame_graph* g, const spl_scene* scene, const float camera_to_world[16], void* stream) {
    if (!g || !scene || !camera_to_world) return fail(SPL_ERR_INVALID, "NULL argument");
    if (scene->n > g->max_splats)
        return fail(SPL_ERR_INVALID, "scene of %llu splats exceeds the graph's bound %llu",
                    (unsigned long long)scene->n, (unsigned long long)g->max_splats);
    return frame_graph_replay(g, scene, camera_to_world, g->out, (cudaStream_t)stream);
}

int spl_scene_load_chunk_device(spl_scene* s, const float* records_device, uint64_t start, uint64_t count,
                                void* stream) {
    if (!s || (!records_device && count)) return fail(SPL_ERR_INVALID, "NULL argument");
    if (start >= s->n) return SPL_OK;
    if (count > s->n - start) count = s->n - start;
    for (uint64_t first = 0; first < count; first += 0x40000000ull) {
        const uint64_t cnt = count - first < 0x40000000ull ? count - first : 0x40000000ull;
        const uint64_t at = start + first;
        launch_load_records(records_device + first * 62, (uint32_t)cnt, s->x + at, s->y + at, s->z + at, s->rot + at,
                            s->scale_alpha + at, s->sh + at * 48, (cudaStream_t)stream);
    }
    CU(cudaGetLastError());
    return SPL_OK;
}

int spl_activate_splats(uint64_t n, const float* means, const float* quaternions, const float* log_scales,
                        const float* opacity_logits, float* x, float* y, float* z, float* rotation, float* scale_alpha,
                        void* stream) {
    if (n == 0) return SPL_OK;
    if (!means || !quaternions || !log_scales || !opacity_logits || !x || !y || !z || !rotation || !scale_alpha)
        return fail(SPL_ERR_INVALID, "NULL argument");
    if (n > MAX_COUNT) return fail(SPL_ERR_INVALID, "%llu splats", (unsigned long long)n);
    launch_activate((uint32_t)n, means, quaternions, log_scales, opacity_logits, x, y, z, rotation, scale_alpha,
                    (cudaStream_t)stream);
    CU(cudaGetLastError());
    return SPL_OK;
}

uint32_t spl_l2_image_loss_partials(uint64_t pixels) { return l2_loss_partials(pixels); }

int spl_l2_image_loss(const float* image, const float* target, uint64_t pixels, float* partial, void* stream) {
    if (!image || !target || !partial) return fail(SPL_ERR_INVALID, "NULL argument");
    if (reinterpret_cast<uintptr_t>(image) & 15u) return fail(SPL_ERR_INVALID, "image must be 16-byte aligned");
    if (pixels == 0) return SPL_OK;
    launch_l2_loss(image, target, pixels, partial, (cudaStream_t)stream);
    CU(cudaGetLastError());
    return SPL_OK;
}

int spl_l2_image_loss_backward(const float* image, const float* target, uint64_t pixels, const float* scale_device,
                               float* grad_image, void* stream) {
    if (!image || !target || !scale_device || !grad_image) return fail(SPL_ERR_INVALID, "NULL argument");
    if ((reinterpret_cast<uintptr_t>(image) | reinterpret_cast<uintptr_t>(grad_image)) & 15u)
        return fail(SPL_ERR_INVALID, "image and grad_image must be 16-byte aligned");
    if (pixels == 0) return SPL_OK;
    launch_l2_loss_backward(image, target, pixels, scale_device, grad_image, (cudaStream_t)stream);
    CU(cudaGetLastError());
    return SPL_OK;
}

int spl_activate_splats_backward(uint64_t n, const float* quaternions, const float* log_scales, const float* rotation,
                                 const float* scale_alpha, const float* grad_x, const float* grad_y,
                                 const float* grad_z, const float* grad_rotation, const float* grad_scale_alpha,
                                 float* grad_means, float* grad_quaternions, float* grad_log_scales,
                                 float* grad_opacity_logits, void* stream) {
    if (n == 0) return SPL_OK;
    if (!quaternions || !log_scales || !rotation || !scale_alpha || !grad_x || !grad_y || !grad_z || !grad_rotation ||
        !grad_scale_alpha || !grad_means || !grad_quaternions || !grad_log_scales || !grad_opacity_logits)
        return fail(SPL_ERR_INVALID, "NULL argument");
    if (n > MAX_COUNT) return fail(SPL_ERR_INVALID, "%llu splats", (unsigned long long)n);
    launch_activate_backward((uint32_t)n, quaternions, log_scales, rotation, scale_alpha, grad_x, grad_y, grad_z,
                             grad_rotation, grad_scale_alpha, grad_means, grad_quaternions, grad_log_scales,
                             grad_opacity_logits, (cudaStream_t)stream);
    CU(cudaGetLastError());
    return SPL_OK;
}

}  // extern "C"
