// Internal host-side definitions of libsplatter_cuda.so shared by its C++ translation units (the
// C ABI in abi.cpp, the serving runtime in server.cpp).  Not installed: callers use
// include/splatter.h.
#pragma once
#include <cstdarg>
#include <cstdint>
#include <mutex>
#include <string>

#include <nvtx3/nvToolsExt.h>  // header-only NVTX v3: no-op calls unless a profiler is attached

#include "../../include/splatter.h"
#include "spl_types.h"

// Records an error message for spl_last_error_string and returns `code`.
int spl_internal_fail(int code, const char* fmt, ...);

namespace spl {

int vfail(int code, const char* fmt, va_list ap);

inline int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    const int rc = vfail(code, fmt, ap);
    va_end(ap);
    return rc;
}

#define CU(call)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return ::spl::fail(SPL_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                                                  __FILE__, __LINE__);                               \
    } while (0)

constexpr uint64_t MAX_COUNT = (1ull << 30) - 1;  // look-back status words carry 30-bit counts
constexpr uint32_t DEFAULT_SPIN_LIMIT = 1u << 20;
constexpr uint64_t CHUNK_RECORDS = 1u << 16;  // staging ring piece (16.25 MB of 248-byte records)

template <typename T>
int dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return SPL_OK;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(SPL_ERR_OOM, "cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
    }
    return SPL_OK;
}

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

inline uint64_t ceil_div(uint64_t a, uint64_t b) { return (a + b - 1) / b; }

// Frame uniforms (renderer.rs:364-409) from the camera-to-world matrix.
void compute_uniforms(const spl_config& cfg, const float* cam, uint32_t W, uint32_t H, Uniforms& u);

}  // namespace spl

using namespace spl;  // the structs below use the device-side types

struct spl_frame_graph;

struct spl_renderer {
    spl_config cfg{};
    int device = 0;
    uint64_t max_n = 0;
    uint64_t pair_cap = 0;
    uint32_t spin_limit = DEFAULT_SPIN_LIMIT;
    // depth sort: K1 writes keys_a/idx; 4 passes a->b->a->b->a leave (key, slot) in keys_a/vals_a
    uint32_t *keys_a = nullptr, *keys_b = nullptr, *vals_a = nullptr, *vals_b = nullptr, *idx = nullptr;
    float4* rec = nullptr;
    uint2* boxes = nullptr;  // pixel box of each record, for the binning kernel
    uint64_t* st_cull = nullptr;  // [ceil(max_n/4096)]
    uint64_t* st_bin = nullptr;   // [ceil(max_n/1024)]
    uint32_t *pk_a = nullptr, *pk_b = nullptr, *pv_a = nullptr, *pv_b = nullptr;
    FrameCounters* fc = nullptr;
    FrameCounters* fc_sort = nullptr;  // counters of spl_sort_pairs
    uint32_t* coop_cnt = nullptr;      // [256][grid, padded to 4] digit counts + [256] totals (cooperative sort)
    uint32_t* epoch = nullptr;
    Uniforms* d_u = nullptr;           // the frame's uniform block in device memory (k_frame_begin writes it)
    SceneView* d_sv = nullptr;         // the frame's scene view in device memory (k_frame_begin writes it)
    int sort_mode = SPL_SORT_COOPERATIVE;
    uint64_t* st_sort = nullptr;       // onesweep mode: look-back status of the 4 depth passes
    uint64_t* st_pairs = nullptr;      // onesweep mode: look-back status of the <= 3 pair passes
    FrameCounters* host_fc = nullptr;  // pinned
    uint2* ranges = nullptr;
    uint32_t* tile_order = nullptr;  // the raster's tile order, most pairs first (ranges_cap entries)
    bool order_tiles = true;         // off where concurrent frames already hide the raster's tail (serving)
    // render_frame replays a frame graph it captured itself once a viewport and scene size repeat
    bool frame_graphs = true;
    spl_frame_graph* own_graph = nullptr;  // the captured frame of (own_w, own_h, own_n)
    uint32_t seen_w = 0, seen_h = 0;       // the previous direct frame's key
    uint64_t seen_n = 0;
    uint64_t ranges_cap = 0;
    uint32_t scratch_generation = 0;  // bumped when the per-viewport scratch is reallocated (graphs hold it)
    // last frame
    cudaStream_t last_stream = nullptr;
    bool has_frame = false;
    uint32_t last_w = 0, last_h = 0;
    uint64_t last_n = 0;
    const uint32_t* final_pair_vals = nullptr;
    const spl_scene* last_scene = nullptr;
    Uniforms last_u{};
    float* grad_rec = nullptr;  // [max_n][10] record gradients of the backward pass (allocated on first use)
    uint32_t* grad_deferred = nullptr;  // [1 + max_n] count, then the slots swept in double (same)
    // stage profiling: events 0..7 on the frame's stream
    bool profiling = false;
    cudaEvent_t ev_prof[8] = {};
    nvtxRangeId_t nvtx_stage = 0;  // the open stage range of the frame being enqueued


    void release() {
        dfree(keys_a); dfree(keys_b); dfree(vals_a); dfree(vals_b); dfree(idx); dfree(rec); dfree(boxes); dfree(grad_rec); dfree(grad_deferred);
        dfree(st_cull); dfree(st_bin);
        dfree(pk_a); dfree(pk_b); dfree(pv_a); dfree(pv_b);
        dfree(fc); dfree(fc_sort); dfree(coop_cnt); dfree(epoch); dfree(ranges); dfree(tile_order); dfree(d_u); dfree(d_sv);
        dfree(st_sort); dfree(st_pairs);
        if (host_fc) cudaFreeHost(host_fc);
        host_fc = nullptr;
        for (auto& e : ev_prof) {
            if (e) cudaEventDestroy(e);
            e = nullptr;
        }
    }
    uint64_t sort_tiles() const { return (max_n + SORT_TILE - 1) / SORT_TILE; }
    uint64_t pair_tiles() const { return (pair_cap + SORT_TILE - 1) / SORT_TILE; }
    // Stage boundary i of a frame (0: before the cull ... 7: after the raster): a CUDA event when
    // profiling, and an NVTX range per stage around its launches, so that a system profiler shows
    // the stages on the host timeline and their kernels under them.
    void mark(int i, cudaStream_t s) {
        static const char* const stage[7] = {"spl cull", "spl vertex", "spl depth sort", "spl binning",
                                             "spl pair sort", "spl tile ranges", "spl raster"};
        if (profiling) cudaEventRecord(ev_prof[i], s);
        if (i > 0 && nvtx_stage) nvtxRangeEnd(nvtx_stage);
        nvtx_stage = i < 7 ? nvtxRangeStartA(stage[i]) : 0;
    }
};

struct Staging {
    float* pinned[2] = {nullptr, nullptr};
    float* dev[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int next = 0;
};

struct spl_scene {
    spl_renderer* renderer = nullptr;
    int device = 0;
    uint64_t n = 0;
    bool owns = true;  // false for scenes wrapping caller-owned arrays (spl_scene_wrap)
    float *x = nullptr, *y = nullptr, *z = nullptr, *sh = nullptr;
    float4 *rot = nullptr, *scale_alpha = nullptr;
    Staging stg;
    std::mutex stg_mu;

    SceneView view() const { return SceneView{x, y, z, rot, scale_alpha, sh, (uint32_t)n}; }
    void release() {
        if (owns) {
            dfree(x); dfree(y); dfree(z); dfree(sh); dfree(rot); dfree(scale_alpha);
        }
        for (int i = 0; i < 2; ++i) {
            if (stg.pinned[i]) cudaFreeHost(stg.pinned[i]);
            dfree(stg.dev[i]);
            if (stg.ev[i]) cudaEventDestroy(stg.ev[i]);
            stg.pinned[i] = nullptr;
            stg.ev[i] = nullptr;
        }
    }
};
