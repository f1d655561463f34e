// Projection side of the splat pipeline (sm_103a):
//   k_frame_begin   - per-frame counter reset + epoch bump (replaces buffer clears, renderer.rs:412,422-427)
//   k_cull_key      - worldToClipSpace + isInFrustum + depth key + digit histograms (radixSortA,
//                     shaders.wgsl:298-336) fused with ORDERED stream compaction of the visible splats
//                     (warp ballots + decoupled look-back), so only visible keys are sorted
//   k_preprocess    - the vertex stage (shaders.wgsl:507-573): SH colour, exact perspective conic of the
//                     ellipsoid, its decomposition and the rotated rectangle, emitted once per visible
//                     splat as a 64-byte screen-space record for the compute rasteriser
//   k_load_records  - Scene::load_chunk transform (scene.rs:225-250) on the device
//
// Compiled with -fmad=false: all FP32 expressions follow the WGSL operation order and are
// bit-identical to the oracle's FP32 restatement.
#include <cstdio>

#include "spl_vertex.cuh"

namespace spl {

// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ void counters_begin(FrameCounters* fc, uint32_t* epoch_word) {
    uint32_t* w = reinterpret_cast<uint32_t*>(fc);
    const uint32_t nwords = sizeof(FrameCounters) / 4;
    for (uint32_t i = threadIdx.x; i < nwords; i += blockDim.x) w[i] = 0u;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t e = *epoch_word + 1u;
        if (e == 0u) e = 1u;  // epoch 0 marks never-written status words
        *epoch_word = e;
        fc->epoch = e;
    }
}

__global__ void k_counters_begin(FrameCounters* fc, uint32_t* epoch_word) { counters_begin(fc, epoch_word); }

// A frame's first kernel: the counters as above, and the frame's uniform block and scene view
// (kernel parameters here, so that a captured frame graph takes a new camera and scene by updating
// this one node) published to device memory for the kernels that follow.
__global__ void k_frame_begin(FrameCounters* fc, uint32_t* epoch_word, Uniforms u, Uniforms* d_u, SceneView sv,
                              SceneView* d_sv) {
    if (threadIdx.x < sizeof(Uniforms) / 4)
        reinterpret_cast<uint32_t*>(d_u)[threadIdx.x] = reinterpret_cast<const uint32_t*>(&u)[threadIdx.x];
    if (threadIdx.x < sizeof(SceneView) / 4)
        reinterpret_cast<uint32_t*>(d_sv)[threadIdx.x] = reinterpret_cast<const uint32_t*>(&sv)[threadIdx.x];
    counters_begin(fc, epoch_word);
}

void launch_frame_begin(FrameCounters* fc, uint32_t* epoch_word, cudaStream_t st) {
    k_counters_begin<<<1, 256, 0, st>>>(fc, epoch_word);
}

void launch_frame_begin(FrameCounters* fc, uint32_t* epoch_word, const Uniforms& u, Uniforms* d_u, const SceneView& sv,
                        SceneView* d_sv, cudaStream_t st) {
    k_frame_begin<<<1, 256, 0, st>>>(fc, epoch_word, u, d_u, sv, d_sv);
}

const void* frame_begin_kernel() { return reinterpret_cast<const void*>(&k_frame_begin); }

// The frame's uniform block and scene view staged in shared memory (one word per thread of the
// first warps; the caller synchronises).
__device__ __forceinline__ void stage_frame(const Uniforms* __restrict__ d_u, Uniforms& s_u,
                                            const SceneView* __restrict__ d_sv, SceneView& s_sv) {
    if (threadIdx.x < sizeof(Uniforms) / 4)
        reinterpret_cast<uint32_t*>(&s_u)[threadIdx.x] = __ldg(reinterpret_cast<const uint32_t*>(d_u) + threadIdx.x);
    if (threadIdx.x < sizeof(SceneView) / 4)
        reinterpret_cast<uint32_t*>(&s_sv)[threadIdx.x] = __ldg(reinterpret_cast<const uint32_t*>(d_sv) + threadIdx.x);
}

// ------------------------------------------------------------------------------------------------
// Cull + key + histogram + ordered compaction.  One CTA handles 4096 consecutive splats; warp w owns
// splats [w*512, w*512+512) of the tile and lane l handles elements w*512 + 32*j + l, so loads are
// coalesced and the ballot order is the index order.
template <int MODE, bool HIST>
__global__ void __launch_bounds__(256, 3) k_cull_key(const SceneView* __restrict__ d_sv, const Uniforms* __restrict__ d_u,
                                                  FrameCounters* fc,
                                                  const uint32_t* __restrict__ epoch_word, uint64_t* status,
                                                  uint32_t* __restrict__ keys_out, uint32_t* __restrict__ idx_out,
                                                  uint32_t spin_limit) {
    __shared__ uint32_t s_hist[HIST ? 1024 : 1];
    __shared__ uint32_t s_wcnt[8];
    __shared__ uint32_t s_tile, s_epoch, s_base;
    __shared__ Uniforms s_u;
    __shared__ SceneView s_sv;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
    if (HIST)
        for (uint32_t i = tid; i < 1024u; i += 256u) s_hist[i] = 0u;
    stage_frame(d_u, s_u, d_sv, s_sv);
    if (tid == 0) {
        s_tile = atomicAdd(&fc->tile_counter[0], 1u);
        s_epoch = *epoch_word;
    }
    __syncthreads();
    const Uniforms& u = s_u;
    const SceneView& s = s_sv;
    const uint32_t tile = s_tile, epoch = s_epoch, n = s.n;
    const uint32_t ntiles = (n + CULL_TILE - 1) / CULL_TILE;
    if (tile >= ntiles) return;  // a grid sized for a larger scene (captured frames)
    const uint32_t base = tile * CULL_TILE + w * (CULL_TILE / 8u) + lane;

    constexpr int PER_LANE = CULL_TILE / 256;
    float px[PER_LANE], py[PER_LANE], pz[PER_LANE];
#pragma unroll
    for (int j = 0; j < PER_LANE; ++j) {
        const uint32_t e = base + 32u * j;
        if (e < n) {
            px[j] = __ldg(s.x + e);
            py[j] = __ldg(s.y + e);
            pz[j] = __ldg(s.z + e);
        } else {
            px[j] = py[j] = pz[j] = 0.0f;
        }
    }
    uint32_t key[PER_LANE], pos[PER_LANE];
    uint32_t vis_bits = 0u, wtotal = 0u, all_ones = 0u, top_ff = 0u;
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int j = 0; j < PER_LANE; ++j) {
        const uint32_t e = base + 32u * j;
        float h[4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
            h[r] = ((u.vp[0 * 4 + r] * px[j] + u.vp[1 * 4 + r] * py[j]) + u.vp[2 * 4 + r] * pz[j]) + u.vp[3 * 4 + r] * 1.0f;
        bool vis;
        uint32_t k;
        if (MODE == DS_CPU) {
            // renderer.rs:381-387: reciprocal multiply, no epsilon, key = bits(z)
            const float rw = 1.0f / h[3];
            const float cx = h[0] * rw, cy = h[1] * rw, cz = h[2] * rw;
            vis = fabsf(cx) < u.tol && fabsf(cy) < u.tol && fabsf(cz - 0.5f) < 0.5f;
            k = __float_as_uint(cz);
        } else {
            // shaders.wgsl:54-61, 318-324
            const float den = h[3] + 1e-7f;
            const float cx = h[0] / den, cy = h[1] / den, cz = h[2] / den;
            vis = fabsf(cx) < u.tol && fabsf(cy) < u.tol && fabsf(cz - 0.5f) < 0.5f;
            k = sat_u32(cz * 65535.0f) << 16;
            k |= sat_u32((cx * 0.5f + 0.5f) * 255.0f) << 8;
            k |= sat_u32((cy * 0.5f + 0.5f) * 255.0f);
        }
        vis = vis && e < n;
        const uint32_t b = __ballot_sync(FULL_MASK, vis);
        pos[j] = wtotal + __popc(b & lt);
        wtotal += __popc(b);
        key[j] = k;
        if (vis) {
            vis_bits |= 1u << j;
            if (HIST) {
                atomicAdd(&s_hist[k & 255u], 1u);
                atomicAdd(&s_hist[256u + ((k >> 8) & 255u)], 1u);
                atomicAdd(&s_hist[512u + ((k >> 16) & 255u)], 1u);
                atomicAdd(&s_hist[768u + (k >> 24)], 1u);
            }
            all_ones += k == 0xFFFFFFFFu;
            top_ff += (k >> 24) == 0xFFu;
        }
    }
    if (lane == 0) s_wcnt[w] = wtotal;
    __syncthreads();
    uint32_t wpre = 0, ttot = 0;
#pragma unroll
    for (uint32_t i = 0; i < 8; ++i) {
        const uint32_t c = s_wcnt[i];
        wpre += i < w ? c : 0u;
        ttot += c;
    }
    if (w == 0) {
        if (lane == 0) lb_store(status + tile, lb_pack(epoch, tile == 0 ? LB_INC : LB_AGG, ttot));
        const uint32_t excl = tile == 0 ? 0u : lookback_single(status, tile, epoch, spin_limit, &fc->err);
        if (lane == 0) {
            if (tile != 0) lb_store(status + tile, lb_pack(epoch, LB_INC, excl + ttot));
            s_base = excl;
            if (tile == ntiles - 1) fc->visible = excl + ttot;
        }
    }
    __syncthreads();
    const uint32_t out0 = s_base + wpre;
#pragma unroll
    for (int j = 0; j < PER_LANE; ++j) {
        if (vis_bits & (1u << j)) {
            keys_out[out0 + pos[j]] = key[j];
            idx_out[out0 + pos[j]] = base + 32u * j;
        }
    }
    if (HIST) {
        for (uint32_t i = tid; i < 1024u; i += 256u) {
            const uint32_t v = s_hist[i];
            if (v) atomicAdd(&fc->hist_depth[0][0] + i, v);
        }
    }
    if (MODE != DS_CPU) {
        const uint32_t a = __reduce_add_sync(FULL_MASK, all_ones), t = __reduce_add_sync(FULL_MASK, top_ff);
        if (lane == 0 && a) atomicAdd(&fc->keys_all_ones, a);
        if (lane == 0 && t) atomicAdd(&fc->keys_top_ff, t);
    }
}

void launch_cull_key(int mode, bool hist, uint32_t grid_n, const SceneView* d_sv, const Uniforms* u,
                     FrameCounters* fc, const uint32_t* epoch_word, uint64_t* status, uint32_t* keys_out,
                     uint32_t* idx_out, uint32_t spin_limit, cudaStream_t st) {
    if (grid_n == 0) return;
    const uint32_t grid = (grid_n + CULL_TILE - 1) / CULL_TILE;
    auto k = mode == DS_CPU ? (hist ? k_cull_key<DS_CPU, true> : k_cull_key<DS_CPU, false>)
                            : (hist ? k_cull_key<DS_GPU, true> : k_cull_key<DS_GPU, false>);
    k<<<grid, 256, 0, st>>>(d_sv, u, fc, epoch_word, status, keys_out, idx_out, spin_limit);
}

// ------------------------------------------------------------------------------------------------
template <int SHO>
__device__ __forceinline__ void load_sh(const float* __restrict__ sh, uint32_t i, float* out) {
    constexpr int NF = 3 * (SHO + 1) * (SHO + 1);
    constexpr int NV = (NF + 3) / 4;
    const float4* p = reinterpret_cast<const float4*>(sh + (size_t)i * 48);
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const float4 v = __ldg(p + k);
        out[4 * k + 0] = v.x;
        if (4 * k + 1 < 48) out[4 * k + 1] = v.y;
        if (4 * k + 2 < 48) out[4 * k + 2] = v.z;
        if (4 * k + 3 < 48) out[4 * k + 3] = v.w;
    }
}

template <int SHO, bool COV, bool RECT>
__global__ void __launch_bounds__(256) k_preprocess(const SceneView* __restrict__ d_sv,
                                                    const Uniforms* __restrict__ d_u,
                                                    const uint32_t* __restrict__ idx,
                                                    const FrameCounters* __restrict__ fc, float4* __restrict__ rec,
                                                    uint2* __restrict__ boxes) {
    __shared__ Uniforms s_u;
    __shared__ SceneView s_sv;
    stage_frame(d_u, s_u, d_sv, s_sv);
    __syncthreads();
    const Uniforms& u = s_u;
    const SceneView& s = s_sv;
    const uint32_t V = fc->visible;
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < V; slot += gridDim.x * blockDim.x) {
        const uint32_t i = __ldg(idx + slot);
        const float cx = __ldg(s.x + i), cy = __ldg(s.y + i), cz = __ldg(s.z + i);
        const float4 rot = __ldg(s.rot + i);
        const float4 sca = __ldg(s.scale_alpha + i);
        float sh[48];
        load_sh<SHO>(s.sh, i, sh);
        VertexOut<float> o;
        vertex_math<SHO, COV, float>(u, cx, cy, cz, rot.x, rot.y, rot.z, rot.w, sca.x, sca.y, sca.z, sh, o);
        // pixel box of the rectangle (or AA square) and validity
        const float vw = u.view_size[0], vh = u.view_size[1];
        const float Wf = (float)u.image_size[0], Hf = (float)u.image_size[1];
        const float psx = (2.0f * vw) / Wf, psy = -((2.0f * vh) / Hf);
        const float m = u.margin;
        float ex, ey, R = 0.0f;
        if (RECT) {
            ex = m * (fabsf(o.Xx) + fabsf(o.Yx));
            ey = m * (fabsf(o.Xy) + fabsf(o.Yy));
        } else {
            R = sqrtf(fmaxf(o.Xx * o.Xx + o.Xy * o.Xy, o.Yx * o.Yx + o.Yy * o.Yy)) * m;
            ex = R;
            ey = R;
        }
        const float cxp = (o.t0 + vw) / psx, exq = ex / psx;
        const float cyp = (o.t1 - vh) / psy, eyq = ey / (-psy);
        // pixels whose centre (p + 0.5) lies in the exact box, widened by 1/64 px against rounding
        const float eps = 0.015625f;
        const float fx0 = ceilf(((cxp - exq) - eps) - 0.5f), fx1 = floorf(((cxp + exq) + eps) - 0.5f);
        const float fy0 = ceilf(((cyp - eyq) - eps) - 0.5f), fy1 = floorf(((cyp + eyq) + eps) - 0.5f);
        const float al = sca.w;
        bool ok = isfinite(o.A00) && isfinite(o.A01) && isfinite(o.B0) && isfinite(o.A10) && isfinite(o.A11) &&
                  isfinite(o.B1) && isfinite(o.cr) && isfinite(o.cg) && isfinite(o.cb) && isfinite(fx0) &&
                  isfinite(fx1) && isfinite(fy0) && isfinite(fy1) && isfinite(R) && isfinite(o.bx) && isfinite(o.by) &&
                  (al >= 1.0f / 255.0f);
        uint32_t lo = 0xFFFFFFFFu, hi = 0u;
        if (ok) {
            const float cx0 = fmaxf(fx0, 0.0f), cx1 = fminf(fx1, Wf - 1.0f);
            const float cy0 = fmaxf(fy0, 0.0f), cy1 = fminf(fy1, Hf - 1.0f);
            if (cx0 <= cx1 && cy0 <= cy1) {
                lo = (uint32_t)(int)cx0 | ((uint32_t)(int)cy0 << 16);
                hi = (uint32_t)(int)cx1 | ((uint32_t)(int)cy1 << 16);
            }
        }
        float4* q = rec + (size_t)slot * 4;
        q[0] = make_float4(o.A00, o.A01, o.B0, o.A10);
        q[1] = make_float4(o.A11, o.B1, al, __uint_as_float(lo));
        q[2] = make_float4(o.cr, o.cg, o.cb, __uint_as_float(hi));
        q[3] = RECT ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : make_float4(o.bx, o.by, R, 0.0f);
        boxes[slot] = make_uint2(lo, hi);  // compact copy for the binning kernel
    }
}

template <int SHO, bool COV>
static void launch_pre2(bool rect, dim3 g, const SceneView* s, const Uniforms* u, const uint32_t* idx,
                        const FrameCounters* fc, float4* rec, uint2* boxes, cudaStream_t st) {
    if (rect)
        k_preprocess<SHO, COV, true><<<g, 256, 0, st>>>(s, u, idx, fc, rec, boxes);
    else
        k_preprocess<SHO, COV, false><<<g, 256, 0, st>>>(s, u, idx, fc, rec, boxes);
}
template <int SHO>
static void launch_pre1(bool cov, bool rect, dim3 g, const SceneView* s, const Uniforms* u, const uint32_t* idx,
                        const FrameCounters* fc, float4* rec, uint2* boxes, cudaStream_t st) {
    if (cov)
        launch_pre2<SHO, true>(rect, g, s, u, idx, fc, rec, boxes, st);
    else
        launch_pre2<SHO, false>(rect, g, s, u, idx, fc, rec, boxes, st);
}

void launch_preprocess(int sh_order, bool covariance, bool rect, const SceneView* s, const Uniforms* u,
                       const uint32_t* idx, const FrameCounters* fc, float4* rec, uint2* boxes, uint32_t max_n,
                       cudaStream_t st) {
    if (max_n == 0) return;
    uint32_t blocks = (max_n + 255) / 256;
    if (blocks > device_sm_count() * 16u) blocks = device_sm_count() * 16u;
    const dim3 g(blocks);
    switch (sh_order) {
        case 0: launch_pre1<0>(covariance, rect, g, s, u, idx, fc, rec, boxes, st); break;
        case 1: launch_pre1<1>(covariance, rect, g, s, u, idx, fc, rec, boxes, st); break;
        case 2: launch_pre1<2>(covariance, rect, g, s, u, idx, fc, rec, boxes, st); break;
        default: launch_pre1<3>(covariance, rect, g, s, u, idx, fc, rec, boxes, st); break;
    }
}

// ------------------------------------------------------------------------------------------------
// Loader: 62-float PLY records -> SoA (scene.rs:225-250).  A block stages 256 records in shared
// memory with coalesced 16-byte loads, transforms one record per thread, and writes the 48 SH
// floats of its 256 splats back as one contiguous, coalesced range.
constexpr int LOAD_BLOCK = 256;

__global__ void __launch_bounds__(LOAD_BLOCK) k_load_records(const float* __restrict__ recs, uint32_t count,
                                                             float* x, float* y, float* z, float4* rot,
                                                             float4* scale_alpha, float* sh) {
    extern __shared__ float4 s_buf4[];
    float* s_buf = reinterpret_cast<float*>(s_buf4);
    const uint32_t first = blockIdx.x * LOAD_BLOCK;
    const uint32_t nrec = min((uint32_t)LOAD_BLOCK, count - first);
    const uint32_t nflt = nrec * 62u;
    const float* src = recs + (size_t)first * 62u;  // 256*62*4 bytes per block: 16-byte aligned
    const uint32_t nvec = nflt / 4u;
    for (uint32_t k = threadIdx.x; k < nvec; k += LOAD_BLOCK) s_buf4[k] = __ldg(reinterpret_cast<const float4*>(src) + k);
    for (uint32_t k = nvec * 4u + threadIdx.x; k < nflt; k += LOAD_BLOCK) s_buf[k] = __ldg(src + k);
    __syncthreads();
    const uint32_t t = threadIdx.x;
    if (t < nrec) {
        const float* r = s_buf + t * 62u;
        const uint32_t i = first + t;
        float4 q, sa;
        activate_splat(r[58], r[59], r[60], r[61], r[55], r[56], r[57], r[54], q, sa);
        rot[i] = q;
        scale_alpha[i] = sa;
        x[i] = r[0];
        y[i] = r[1];
        z[i] = r[2];
    }
    float* dst = sh + (size_t)first * 48u;
    for (uint32_t k = threadIdx.x; k < nrec * 48u; k += LOAD_BLOCK) {
        const uint32_t rr = k / 48u, c = k - rr * 48u;
        dst[k] = s_buf[rr * 62u + 6u + c];
    }
}

void launch_load_records(const float* records62, uint32_t count, float* x, float* y, float* z, float4* rot,
                         float4* scale_alpha, float* sh, cudaStream_t st) {
    if (count == 0) return;
    static bool attr = false;
    const int smem = LOAD_BLOCK * 62 * 4;
    if (!attr) {
        cudaFuncSetAttribute(k_load_records, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr = true;
    }
    const uint32_t grid = (count + LOAD_BLOCK - 1) / LOAD_BLOCK;
    k_load_records<<<grid, LOAD_BLOCK, smem, st>>>(records62, count, x, y, z, rot, scale_alpha, sh);
}

// 60-float device splats of the reference (scene.rs:32, shaders.wgsl:28-35) <-> SoA.
__global__ void k_splats60_to_soa(const float* __restrict__ s60, uint32_t count, float* x, float* y, float* z,
                                  float4* rot, float4* scale_alpha, float* sh) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const float4* r = reinterpret_cast<const float4*>(s60 + (size_t)i * 60);
        const float4 a = r[0], b = r[1], c = r[2];
        rot[i] = a;
        x[i] = b.x;
        y[i] = b.y;
        z[i] = b.z;
        scale_alpha[i] = c;
        float4* d = reinterpret_cast<float4*>(sh + (size_t)i * 48);
#pragma unroll
        for (int k = 0; k < 12; ++k) d[k] = r[3 + k];
    }
}

__global__ void k_soa_to_splats60(SceneView s, uint32_t start, uint32_t count, float* s60) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
        const uint32_t i = start + t;
        float4* r = reinterpret_cast<float4*>(s60 + (size_t)t * 60);
        r[0] = s.rot[i];
        r[1] = make_float4(s.x[i], s.y[i], s.z[i], 0.0f);
        r[2] = s.scale_alpha[i];
        const float4* q = reinterpret_cast<const float4*>(s.sh + (size_t)i * 48);
#pragma unroll
        for (int k = 0; k < 12; ++k) r[3 + k] = q[k];
    }
}

void launch_splats60_to_soa(const float* s60, uint32_t count, float* x, float* y, float* z, float4* rot,
                            float4* scale_alpha, float* sh, cudaStream_t st) {
    if (count == 0) return;
    uint32_t grid = (count + 255) / 256;
    if (grid > 4096) grid = 4096;
    k_splats60_to_soa<<<grid, 256, 0, st>>>(s60, count, x, y, z, rot, scale_alpha, sh);
}

void launch_soa_to_splats60(const SceneView& s, uint32_t start, uint32_t count, float* s60, cudaStream_t st) {
    if (count == 0) return;
    uint32_t grid = (count + 255) / 256;
    if (grid > 4096) grid = 4096;
    k_soa_to_splats60<<<grid, 256, 0, st>>>(s, start, count, s60);
}

// Sorted entries (key, splat index) for readback (the reference's commented debug readback,
// renderer.rs:456-464).  slots == nullptr for the unsorted (None) mode.
__global__ void k_gather_entries(const uint32_t* keys, const uint32_t* slots, const uint32_t* idx,
                                 const FrameCounters* fc, uint32_t* keys_out, uint32_t* idx_out, uint32_t cap) {
    const uint32_t V = min(fc->visible, cap);
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < V; r += gridDim.x * blockDim.x) {
        if (slots) {
            keys_out[r] = keys[r];
            idx_out[r] = idx[slots[r]];
        } else {
            keys_out[r] = keys[r];
            idx_out[r] = idx[r];
        }
    }
}

void launch_gather_entries(const uint32_t* keys, const uint32_t* slots, const uint32_t* idx, const FrameCounters* fc,
                           int mode, uint32_t* keys_out, uint32_t* idx_out, uint32_t cap, cudaStream_t st) {
    (void)mode;
    if (cap == 0) return;
    uint32_t grid = (cap + 255) / 256;
    if (grid > 4096) grid = 4096;
    k_gather_entries<<<grid, 256, 0, st>>>(keys, slots, idx, fc, keys_out, idx_out, cap);
}

// Fault-free check of the bounded look-back: one warp acts as tile 1 of a scan whose tile 0 never
// publishes (status[0] is never written).  The wait runs out after spin_limit polls, raises the
// error bit and returns; out[0] = prefix it gave up with, out[1] = error word.
__global__ void k_lookback_probe(uint64_t* status, uint32_t* err, uint32_t spin_limit, uint32_t* out) {
    const uint32_t excl = lookback_single(status, 1u, 7u, spin_limit, err);
    __syncwarp();
    if (threadIdx.x == 0) {
        out[0] = excl;
        out[1] = ld_relaxed_u32(err);
    }
}

void launch_lookback_probe(uint64_t* status, uint32_t* err, uint32_t spin_limit, uint32_t* out, cudaStream_t st) {
    k_lookback_probe<<<1, 32, 0, st>>>(status, err, spin_limit, out);
}

}  // namespace spl
