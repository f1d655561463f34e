// Backward pass of the splat pipeline (sm_103a), fp32 blend mode.  No reference counterpart: the
// reference only renders.  The forward it differentiates is the one k_raster/k_preprocess compute:
//
//   per pixel, front to back over the tile's depth-ordered list:
//     alpha = a * exp(-|tc|^2 / 2)            (skipped when alpha < 1/255)
//     s_c = sat(rgb_c * alpha), sa = sat(alpha)
//     C_c += s_c * T,  T *= (1 - sa)          (stops once T < 1e-4)
//
// k_raster_backward re-walks each tile front to back, RECOMPUTING the transmittance instead of
// storing it.  With C_final and T_final from the forward image, the colour still to come after
// splat i is S = C_final - C_(<=i), so
//     dL/ds_c  = dL/dC_c * T_i
//     dL/dsa   = -(dL/dC . S + dL/dT * T_final) / (1 - sa)
// and the chain through sat(), the falloff and tc = A (X, Y) + B gives per-splat gradients of the
// record (A00, A01, B0, A10, A11, B1, a, r, g, b), reduced over each 8-lane pixel group before one
// set of global float atomics per (splat, group).  A is accumulated against pixel offsets from the
// centre of the splat's pixel box and B at that centre (well conditioned; see vertex_vjp_t).
//
// k_preprocess_backward maps those record gradients to the splat parameters (centre, rotation,
// scale, opacity, SH) in reverse mode (vertex_vjp_t): one sweep of the vertex stage's values, one
// sweep of adjoints back through the same formulas, in float; needles and discs (needs_double_sweep)
// are left to k_preprocess_backward_double, which sweeps them in double.  SH coefficient gradients
// are the basis values times the colour gradients.
#include "spl_vertex.cuh"

namespace spl {

constexpr int GR = 10;  // gradient words per record

__global__ void k_zero_grad_rec(float* grad_rec, const FrameCounters* fc, uint32_t* deferred) {
    if (blockIdx.x == 0 && threadIdx.x == 0) deferred[0] = 0u;
    const uint32_t n = fc->visible * GR;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) grad_rec[i] = 0.0f;
}

// Sums 10 values over the 8 lanes of a lane group (lane index li = lane & 7) in three exchange steps
// that halve the values each lane carries (5 + 3 + 2 shuffles instead of 3 per value): afterwards lane
// li holds the group sum of value k0 in v0 and, for li = 0 and 4, of value k0 + 1 in v1.
//   li: 0 -> 0, 1   1 -> 2   2 -> 3   3 -> 4   4 -> 5, 6   5 -> 7   6 -> 8   7 -> 9
__device__ __forceinline__ uint32_t reduce10_over8(const float* g, uint32_t li, float& v0, float& v1) {
    const bool h4 = (li & 4u) != 0u, h2 = (li & 2u) != 0u, h1 = (li & 1u) != 0u;
    float a[5], b[3];
#pragma unroll
    for (int i = 0; i < 5; ++i) {  // keep values 5..9 (h4) or 0..4
        const float send = h4 ? g[i] : g[i + 5], keep = h4 ? g[i + 5] : g[i];
        a[i] = keep + __shfl_xor_sync(FULL_MASK, send, 4);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {  // keep a[3..4] (h2) or a[0..2]
        const float hi = i < 2 ? a[i + 3] : 0.0f;
        const float send = h2 ? a[i] : hi, keep = h2 ? hi : a[i];
        b[i] = keep + __shfl_xor_sync(FULL_MASK, send, 2);
    }
    // h2 lanes carry two values (b0, b1): keep b1 (h1) or b0; the others three: keep b2 (h1) or b0, b1
    const float send0 = h1 ? b[0] : (h2 ? b[1] : b[2]);
    const float keep0 = h1 ? (h2 ? b[1] : b[2]) : b[0];
    const float send1 = (h1 && !h2) ? b[1] : 0.0f;
    const float keep1 = (!h1 && !h2) ? b[1] : 0.0f;
    v0 = keep0 + __shfl_xor_sync(FULL_MASK, send0, 1);
    v1 = keep1 + __shfl_xor_sync(FULL_MASK, send1, 1);
    return (h4 ? 5u : 0u) + (h2 ? (h1 ? 4u : 3u) : (h1 ? 2u : 0u));
}

template <bool RECT>
__global__ void __launch_bounds__(256) k_raster_backward(const uint2* __restrict__ ranges,
                                                         const uint32_t* __restrict__ tile_order,
                                                         const uint32_t* __restrict__ pair_vals,
                                                         const float4* __restrict__ rec, int W, int H, int tiles_x,
                                                         float margin, float psx, float psy,
                                                         const float4* __restrict__ image,
                                                         const float4* __restrict__ grad_image,
                                                         float* __restrict__ grad_rec) {
    __shared__ float4 s_q0[256], s_q1[256], s_q2[256];
    __shared__ float4 s_q3[RECT ? 1 : 256];
    __shared__ uint32_t s_slot[256];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
    const uint32_t grp = lane >> 3, li = lane & 7u;
    // the forward's most-pairs-first order of this frame's tiles, when it made one
    const int tile = tile_order ? (int)__ldg(tile_order + blockIdx.x) : (int)blockIdx.x;
    const int tx = tile % tiles_x, ty = tile / tiles_x;
    const int bx0 = tx * TILE_PIXELS + 4 * (int)grp;
    const int by0 = ty * TILE_PIXELS + 2 * (int)w;
    const int px = bx0 + (int)(li & 3u), py = by0 + (int)(li >> 2);
    const float X = (float)px + 0.5f, Y = (float)py + 0.5f;
    const uint2 rg = ranges[tile];
    const bool inside = px < W && py < H;
    float Cf[3] = {0.0f, 0.0f, 0.0f}, gC[3] = {0.0f, 0.0f, 0.0f}, Tf = 1.0f, gT = 0.0f;
    if (inside) {
        const size_t pix = (size_t)py * (size_t)W + (size_t)px;
        const float4 im = image[pix], gi = grad_image[pix];
        Cf[0] = im.x; Cf[1] = im.y; Cf[2] = im.z; Tf = im.w;
        gC[0] = gi.x; gC[1] = gi.y; gC[2] = gi.z; gT = gi.w;
    }
    const float kT = gT * Tf;
    bool done = !inside;
    float T = 1.0f, Ca[3] = {0.0f, 0.0f, 0.0f};
    const float alpha_min = 1.0f / 255.0f;
    const int wx0 = tx * TILE_PIXELS;
    for (uint32_t b = rg.x; b < rg.y; b += 256) {
        __syncthreads();
        const uint32_t i = b + tid;
        if (i < rg.y) {
            const uint32_t slot = __ldg(pair_vals + i);
            s_slot[tid] = slot;
            const float4* r = rec + (size_t)slot * 4;
            s_q0[tid] = __ldg(r + 0);
            s_q1[tid] = __ldg(r + 1);
            s_q2[tid] = __ldg(r + 2);
            if (!RECT) s_q3[tid] = __ldg(r + 3);
        }
        __syncthreads();
        const uint32_t cnt = min(256u, rg.y - b);
        if (__any_sync(FULL_MASK, !done)) {
            for (uint32_t j0 = 0; j0 < cnt; j0 += 32) {
                uint32_t m0, m1, m2, m3;
                {
                    const uint32_t jl = j0 + lane;
                    int x0 = 1, x1 = 0, y0 = 1, y1 = 0;
                    if (jl < cnt) {
                        const uint32_t lo = __float_as_uint(s_q1[jl].w), hi = __float_as_uint(s_q2[jl].w);
                        x0 = (int)(lo & 0xFFFFu);
                        y0 = (int)(lo >> 16);
                        x1 = (int)(hi & 0xFFFFu);
                        y1 = (int)(hi >> 16);
                    }
                    const bool rows = !(y1 < by0 || y0 > by0 + 1) && x0 <= x1;
                    m0 = __ballot_sync(FULL_MASK, rows && !(x1 < wx0 + 0 || x0 > wx0 + 3));
                    m1 = __ballot_sync(FULL_MASK, rows && !(x1 < wx0 + 4 || x0 > wx0 + 7));
                    m2 = __ballot_sync(FULL_MASK, rows && !(x1 < wx0 + 8 || x0 > wx0 + 11));
                    m3 = __ballot_sync(FULL_MASK, rows && !(x1 < wx0 + 12 || x0 > wx0 + 15));
                }
                uint32_t mine = grp == 0 ? m0 : (grp == 1 ? m1 : (grp == 2 ? m2 : m3));
                // every lane runs every iteration (no early exits) so the group reductions are legal
                while (__any_sync(FULL_MASK, mine != 0u)) {
                    const bool have = mine != 0u;
                    const uint32_t j = have ? j0 + (uint32_t)(__ffs(mine) - 1) : 0u;
                    if (have) mine &= mine - 1u;
                    float g[GR];
#pragma unroll
                    for (int k = 0; k < GR; ++k) g[k] = 0.0f;
                    bool contrib = false;
                    if (have && !done) {
                        const float4 q1 = s_q1[j], q2 = s_q2[j];
                        const uint32_t lo = __float_as_uint(q1.w), hi = __float_as_uint(q2.w);
                        const int x0 = (int)(lo & 0xFFFFu), y0 = (int)(lo >> 16);
                        const int x1 = (int)(hi & 0xFFFFu), y1 = (int)(hi >> 16);
                        if ((unsigned)(px - x0) <= (unsigned)(x1 - x0) && (unsigned)(py - y0) <= (unsigned)(y1 - y0)) {
                            const float4 q0 = s_q0[j];
                            const float tcx = fmaf(q0.y, Y, fmaf(q0.x, X, q0.z));
                            const float tcy = fmaf(q1.x, Y, fmaf(q0.w, X, q1.y));
                            bool cov;
                            if (RECT) {
                                cov = fabsf(tcx) <= margin && fabsf(tcy) <= margin;
                            } else {
                                const float4 q3 = s_q3[j];
                                const float dx = fmaf(psx, X, q3.x), dy = fmaf(psy, Y, q3.y);
                                cov = fabsf(dx) <= q3.z && fabsf(dy) <= q3.z;
                            }
                            if (cov) {
                                const float power = fmaf(tcx, tcx, tcy * tcy);
                                const float E = spl_expf_nonpos(-0.5f * power);
                                const float a = q1.z;
                                const float alpha = a * E;
                                if (!(alpha < alpha_min)) {
                                    contrib = true;
                                    const float rgb[3] = {q2.x, q2.y, q2.z};
                                    float s[3], dS[3];
                                    const float sa = __saturatef(alpha);
#pragma unroll
                                    for (int c = 0; c < 3; ++c) {
                                        s[c] = __saturatef(rgb[c] * alpha);
                                        dS[c] = gC[c] * T;
                                        Ca[c] = s[c] * T + Ca[c];  // the forward's operation order
                                    }
                                    const float om = 1.0f - sa;
                                    float dsa = 0.0f;
                                    if (om > 0.0f) {  // om in (0, 1]: the fast divide is within 2 ulp
                                        const float Sdot =
                                            (gC[0] * (Cf[0] - Ca[0]) + gC[1] * (Cf[1] - Ca[1])) + gC[2] * (Cf[2] - Ca[2]);
                                        dsa = __fdividef(-(Sdot + kT), om);
                                    }
                                    T = T * om;
                                    done = T < FP32_T_MIN;
                                    float dalpha = alpha < 1.0f ? dsa : 0.0f;
#pragma unroll
                                    for (int c = 0; c < 3; ++c) {
                                        const float v = rgb[c] * alpha;
                                        if (v > 0.0f && v < 1.0f) {
                                            dalpha += dS[c] * rgb[c];
                                            g[7 + c] = dS[c] * alpha;
                                        }
                                    }
                                    g[6] = dalpha * E;
                                    const float dpow = -0.5f * (dalpha * a * E);
                                    const float dtx = 2.0f * dpow * tcx, dty = 2.0f * dpow * tcy;
                                    // A against offsets from the box centre (Xr, Yr), B at that centre
                                    const float ox = X - 0.5f * (float)(x0 + x1 + 1);
                                    const float oy = Y - 0.5f * (float)(y0 + y1 + 1);
                                    g[0] = dtx * ox;
                                    g[1] = dtx * oy;
                                    g[2] = dtx;
                                    g[3] = dty * ox;
                                    g[4] = dty * oy;
                                    g[5] = dty;
                                }
                            }
                        }
                    }
                    // reduce over the 8 lanes of the group (all hold the same record this iteration)
                    const uint32_t gm = __ballot_sync(FULL_MASK, contrib);
                    if (gm != 0u) {
                        float v0, v1;
                        const uint32_t k0 = reduce10_over8(g, li, v0, v1);
                        if ((gm >> (grp * 8u)) & 0xFFu) {
                            float* dst = grad_rec + (size_t)s_slot[j] * GR;
                            atomicAdd(dst + k0, v0);
                            if ((li & 3u) == 0u) atomicAdd(dst + k0 + 1u, v1);
                        }
                    }
                }
            }
        }
        if (__syncthreads_and(done)) break;
    }
}

// One splat's inputs to the vertex-stage backward: its parameters and SH coefficients, and the view-plane
// position of its record's reference pixel (the centre of the record's pixel box).
template <int SHO>
struct VjpInputs {
    float cx, cy, cz, rx, ry;
    float4 rot, sca;
    float sh[48];
    __device__ __forceinline__ void load(const SceneView& s, const Uniforms& u, uint32_t i, uint2 bb) {
        cx = __ldg(s.x + i);
        cy = __ldg(s.y + i);
        cz = __ldg(s.z + i);
        rot = __ldg(s.rot + i);
        sca = __ldg(s.scale_alpha + i);
        // 16-byte loads of the row's first NF coefficients (rows are 192 bytes, 16-byte aligned; the
        // last load of SH degree 2 also reads coefficient 27, inside the row)
        constexpr int NF4 = (3 * (SHO + 1) * (SHO + 1) + 3) / 4;
        const float4* p = reinterpret_cast<const float4*>(s.sh + (size_t)i * 48);
#pragma unroll
        for (int k = 0; k < NF4; ++k) {
            const float4 v = __ldg(p + k);
            sh[4 * k + 0] = v.x;
            sh[4 * k + 1] = v.y;
            sh[4 * k + 2] = v.z;
            sh[4 * k + 3] = v.w;
        }
        const float Xr = 0.5f * (float)((bb.x & 0xFFFFu) + (bb.y & 0xFFFFu) + 1u);
        const float Yr = 0.5f * (float)((bb.x >> 16) + (bb.y >> 16) + 1u);
        const float vw = u.view_size[0], vh = u.view_size[1];
        rx = Xr * ((2.0f * vw) / (float)u.image_size[0]) - vw;
        ry = vh - Yr * ((2.0f * vh) / (float)u.image_size[1]);
    }
};

__device__ __forceinline__ bool load_record_gradient(const float* grad_rec, uint32_t slot, float* g) {
    const float2* gr = reinterpret_cast<const float2*>(grad_rec + (size_t)slot * GR);  // 40-byte rows
    bool any = false;
#pragma unroll
    for (int k = 0; k < GR / 2; ++k) {
        const float2 v = gr[k];
        g[2 * k] = v.x;
        g[2 * k + 1] = v.y;
        any = any || v.x != 0.0f || v.y != 0.0f;
    }
    return any;  // false: not drawn, or no gradient reached it
}

// The centre, rotation, scale and opacity gradients of splat i (set, or added to what is there).
__device__ __forceinline__ void store_splat_gradient(uint32_t i, const float* gin, float galpha, float* gx, float* gy,
                                                     float* gz, float4* grot, float4* gscale_alpha, bool accumulate) {
    if (accumulate) {  // several frames' gradients summed in place, one frame after another
        const float4 r0 = grot[i], s0 = gscale_alpha[i];
        gx[i] += gin[0];
        gy[i] += gin[1];
        gz[i] += gin[2];
        grot[i] = make_float4(r0.x + gin[3], r0.y + gin[4], r0.z + gin[5], r0.w + gin[6]);
        gscale_alpha[i] = make_float4(s0.x + gin[7], s0.y + gin[8], s0.z + gin[9], s0.w + galpha);
    } else {
        gx[i] = gin[0];
        gy[i] = gin[1];
        gz[i] = gin[2];
        grot[i] = make_float4(gin[3], gin[4], gin[5], gin[6]);
        gscale_alpha[i] = make_float4(gin[7], gin[8], gin[9], galpha);
    }
}

// Float sweep of every drawn splat but the needles and discs (needs_double_sweep), whose slots go to
// `deferred` ([0] the count, then the slots) for k_preprocess_backward_double; SH gradients of all.
template <int SHO, bool COV>
__global__ void __launch_bounds__(128, 4) k_preprocess_backward(SceneView s, Uniforms u, const uint32_t* __restrict__ idx,
                                                             const FrameCounters* __restrict__ fc,
                                                             const uint2* __restrict__ boxes,
                                                             const float* __restrict__ grad_rec, float* gx, float* gy,
                                                             float* gz, float4* grot, float4* gscale_alpha,
                                                             float* gsh, uint32_t* deferred, uint32_t deferred_cap,
                                                             bool accumulate) {
    const uint32_t V = fc->visible;
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < V; slot += gridDim.x * blockDim.x) {
        float g[GR];
        if (!load_record_gradient(grad_rec, slot, g)) continue;
        const uint32_t i = __ldg(idx + slot);
        VjpInputs<SHO> in;
        in.load(s, u, i, __ldg(boxes + slot));
        if (needs_double_sweep(in.sca.x, in.sca.y, in.sca.z)) {
            const uint32_t pos = atomicAdd(deferred, 1u);
            if (pos < deferred_cap) deferred[1 + pos] = slot;
        } else {
            float gin[10];
            vertex_vjp_t<float, SHO, COV>(u, in.cx, in.cy, in.cz, in.rot.x, in.rot.y, in.rot.z, in.rot.w, in.sca.x,
                                          in.sca.y, in.sca.z, in.sh, in.rx, in.ry, g, gin);
            store_splat_gradient(i, gin, g[6], gx, gy, gz, grot, gscale_alpha, accumulate);
        }
        // SH: rgb_c = 0.5 + sum_k B_k(d) sh[3k + c]
        const float vx = in.cx - u.camera[12], vy = in.cy - u.camera[13], vz = in.cz - u.camera[14];
        const float len = sqrtf((vx * vx + vy * vy) + vz * vz);
        float B[16];
        sh_basis<SHO>(vx / len, vy / len, vz / len, B);
        // coefficient m = 3 k + c gets B[k] g[7 + c]: whole 16-byte groups, then the tail
        constexpr int NF = 3 * (SHO + 1) * (SHO + 1), NV = NF / 4;
        float v[NF];
#pragma unroll
        for (int m = 0; m < NF; ++m) v[m] = B[m / 3] * g[7 + m % 3];
        float* o = gsh + (size_t)i * 48;
        float4* o4 = reinterpret_cast<float4*>(o);
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            float4 x = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
            if (accumulate) {
                const float4 y = o4[k];
                x = make_float4(y.x + x.x, y.y + x.y, y.z + x.z, y.w + x.w);
            }
            o4[k] = x;
        }
#pragma unroll
        for (int m = 4 * NV; m < NF; ++m) o[m] = accumulate ? o[m] + v[m] : v[m];
    }
}

// The deferred needles and discs, swept in double (same formulas, same float forward values).
template <int SHO, bool COV>
__global__ void __launch_bounds__(128) k_preprocess_backward_double(SceneView s, Uniforms u,
                                                                    const uint32_t* __restrict__ idx,
                                                                    const uint2* __restrict__ boxes,
                                                                    const float* __restrict__ grad_rec, float* gx,
                                                                    float* gy, float* gz, float4* grot,
                                                                    float4* gscale_alpha,
                                                                    const uint32_t* __restrict__ deferred,
                                                                    uint32_t deferred_cap, bool accumulate) {
    const uint32_t n = min(deferred[0], deferred_cap);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t slot = deferred[1 + k];
        float g[GR];
        load_record_gradient(grad_rec, slot, g);
        const uint32_t i = __ldg(idx + slot);
        VjpInputs<SHO> in;
        in.load(s, u, i, __ldg(boxes + slot));
        float gin[10];
        vertex_vjp_t<double, SHO, COV>(u, in.cx, in.cy, in.cz, in.rot.x, in.rot.y, in.rot.z, in.rot.w, in.sca.x,
                                       in.sca.y, in.sca.z, in.sh, in.rx, in.ry, g, gin);
        store_splat_gradient(i, gin, g[6], gx, gy, gz, grot, gscale_alpha, accumulate);
    }
}

void launch_backward(int sh_order, bool covariance, bool rect, const SceneView& s, const Uniforms& u,
                     const uint32_t* idx, const FrameCounters* fc, const uint2* boxes, const uint2* ranges,
                     const uint32_t* tile_order, const uint32_t* pair_vals, const float4* rec, const float4* image,
                     const float4* grad_image, float* grad_rec, uint32_t* deferred,
                     uint32_t max_n, float* gx, float* gy, float* gz, float4* grot, float4* gscale_alpha, float* gsh,
                     bool accumulate, cudaStream_t st) {
    const int W = (int)u.image_size[0], H = (int)u.image_size[1];
    const int tiles_x = (W + TILE_PIXELS - 1) / TILE_PIXELS, tiles_y = (H + TILE_PIXELS - 1) / TILE_PIXELS;
    const float psx = (2.0f * u.view_size[0]) / (float)W;
    const float psy = -((2.0f * u.view_size[1]) / (float)H);
    uint32_t zg = (max_n * GR + 255) / 256;
    if (zg > device_sm_count() * 8u) zg = device_sm_count() * 8u;
    if (zg == 0) zg = 1;
    k_zero_grad_rec<<<zg, 256, 0, st>>>(grad_rec, fc, deferred);
    const int grid = tiles_x * tiles_y;
    if (grid > 0) {
        if (rect)
            k_raster_backward<true><<<grid, 256, 0, st>>>(ranges, tile_order, pair_vals, rec, W, H, tiles_x, u.margin,
                                                          psx, psy, image, grad_image, grad_rec);
        else
            k_raster_backward<false><<<grid, 256, 0, st>>>(ranges, tile_order, pair_vals, rec, W, H, tiles_x,
                                                           u.margin, psx, psy, image, grad_image, grad_rec);
    }
    if (max_n == 0) return;
    uint32_t blocks = (max_n + 127) / 128;
    if (blocks > device_sm_count() * 16u) blocks = device_sm_count() * 16u;
    // the double sweep's grid: a few blocks per SM (needles and discs are few; the count is on the device)
    const uint32_t dblocks = device_sm_count() * 2u;
#define PB(SHO, COV)                                                                                          \
    do {                                                                                                      \
        k_preprocess_backward<SHO, COV><<<blocks, 128, 0, st>>>(s, u, idx, fc, boxes, grad_rec, gx, gy, gz, grot, \
                                                                gscale_alpha, gsh, deferred, max_n, accumulate); \
        k_preprocess_backward_double<SHO, COV><<<dblocks, 128, 0, st>>>(s, u, idx, boxes, grad_rec, gx, gy, gz,   \
                                                                        grot, gscale_alpha, deferred, max_n,      \
                                                                        accumulate);                              \
    } while (0)
    switch (sh_order * 2 + (covariance ? 1 : 0)) {
        case 0: PB(0, false); break;
        case 1: PB(0, true); break;
        case 2: PB(1, false); break;
        case 3: PB(1, true); break;
        case 4: PB(2, false); break;
        case 5: PB(2, true); break;
        case 6: PB(3, false); break;
        default: PB(3, true); break;
    }
#undef PB
}

}  // namespace spl
