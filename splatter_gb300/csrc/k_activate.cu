// The loader's activations on device arrays of raw parameters, and their backward, for training:
//   k_activate           raw (positions, quaternions, log-scales, opacity logits) -> the scene's
//                        arrays (x, y, z planes, unit rotations, scale + opacity), with the exact
//                        arithmetic of Scene::load_chunk (scene.rs:225-250; activate_splat)
//   k_activate_backward  gradients of the scene's arrays -> gradients of the raw parameters
//   k_l2_loss            the L2 image loss of float4 frames against RGB targets (block partial sums)
//   k_l2_loss_backward   its gradient, 2 (image - target) times the upstream gradient, in one pass
#include "spl_device.cuh"

namespace spl {

__global__ void __launch_bounds__(256) k_activate(uint32_t n, const float* __restrict__ means,
                                                  const float4* __restrict__ quats, const float* __restrict__ logs,
                                                  const float* __restrict__ logits, float* __restrict__ x,
                                                  float* __restrict__ y, float* __restrict__ z,
                                                  float4* __restrict__ rot, float4* __restrict__ scale_alpha) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 q = __ldg(quats + i);
        float4 r, sa;
        activate_splat(q.x, q.y, q.z, q.w, __ldg(logs + 3 * (size_t)i), __ldg(logs + 3 * (size_t)i + 1),
                       __ldg(logs + 3 * (size_t)i + 2), __ldg(logits + i), r, sa);
        rot[i] = r;
        scale_alpha[i] = sa;
        x[i] = __ldg(means + 3 * (size_t)i);
        y[i] = __ldg(means + 3 * (size_t)i + 1);
        z[i] = __ldg(means + 3 * (size_t)i + 2);
    }
}

// Chain rule through activate_splat, from the activated values it produced:
//   rotation r = q / |q|:            dL/dq = (g_r - (g_r . r) r) / |q|
//   scale s_k = exp(clamp(l_k, m - 5, m + 5)), m = mean(l): an unclamped s_k depends on l_k alone
//                                    (ds_k/dl_k = s_k); a clamped one on m (ds_k/dl_j = s_k / 3)
//   opacity a = sigmoid(t):          dL/dt = g_a a (1 - a)
__global__ void __launch_bounds__(256) k_activate_backward(
    uint32_t n, const float4* __restrict__ quats, const float* __restrict__ logs, const float4* __restrict__ rot,
    const float4* __restrict__ scale_alpha, const float* __restrict__ gx, const float* __restrict__ gy,
    const float* __restrict__ gz, const float4* __restrict__ grot, const float4* __restrict__ gsa,
    float* __restrict__ g_means, float4* __restrict__ g_quats, float* __restrict__ g_logs,
    float* __restrict__ g_logits) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        g_means[3 * (size_t)i] = __ldg(gx + i);
        g_means[3 * (size_t)i + 1] = __ldg(gy + i);
        g_means[3 * (size_t)i + 2] = __ldg(gz + i);
        const float4 q = __ldg(quats + i), r = __ldg(rot + i), g = __ldg(grot + i);
        const float inv = 1.0f / sqrtf(((q.x * q.x + q.y * q.y) + q.z * q.z) + q.w * q.w);
        const float d = ((g.x * r.x + g.y * r.y) + g.z * r.z) + g.w * r.w;
        g_quats[i] = make_float4((g.x - d * r.x) * inv, (g.y - d * r.y) * inv, (g.z - d * r.z) * inv,
                                 (g.w - d * r.w) * inv);
        const float l[3] = {__ldg(logs + 3 * (size_t)i), __ldg(logs + 3 * (size_t)i + 1), __ldg(logs + 3 * (size_t)i + 2)};
        const float4 sa = __ldg(scale_alpha + i), gs = __ldg(gsa + i);
        const float s[3] = {sa.x, sa.y, sa.z}, gsk[3] = {gs.x, gs.y, gs.z};
        const float avg = ((l[0] + l[1]) + l[2]) / 3.0f;
        const float lo = avg - 5.0f, hi = avg + 5.0f;
        float via_mean = 0.0f, out[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const bool clamped = l[k] < lo || l[k] > hi;
            out[k] = clamped ? 0.0f : gsk[k] * s[k];
            if (clamped) via_mean += gsk[k] * s[k];
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) g_logs[3 * (size_t)i + k] = out[k] + via_mean / 3.0f;
        g_logits[i] = gs.w * sa.w * (1.0f - sa.w);
    }
}

// sum over pixels and RGB of (image - target)^2; image: float4 (r, g, b, T) per pixel, target: three
// floats per pixel.  Each block writes its partial sum to partial[blockIdx.x].
__global__ void __launch_bounds__(256) k_l2_loss(const float4* __restrict__ image, const float* __restrict__ target,
                                                 uint64_t pixels, float* __restrict__ partial) {
    __shared__ float s_w[8];
    float acc = 0.0f;
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < pixels; p += gridDim.x * (uint64_t)blockDim.x) {
        const float4 c = __ldg(image + p);
        const float* t = target + 3 * p;
        const float dr = c.x - __ldg(t), dg = c.y - __ldg(t + 1), db = c.z - __ldg(t + 2);
        acc += (dr * dr + dg * dg) + db * db;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(FULL_MASK, acc, o);
    if ((threadIdx.x & 31u) == 0u) s_w[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float sum = 0.0f;
#pragma unroll
        for (int w = 0; w < 8; ++w) sum += s_w[w];
        partial[blockIdx.x] = sum;
    }
}

// grad = (2 (image - target) * scale, 0) per pixel, scale read from device memory (the upstream
// gradient of the loss, with no host round trip): the products torch's autograd forms for the same
// expression, so the result is the same bit for bit.
__global__ void __launch_bounds__(256) k_l2_loss_backward(const float4* __restrict__ image,
                                                          const float* __restrict__ target, uint64_t pixels,
                                                          const float* __restrict__ scale, float4* __restrict__ grad) {
    const float sc = __ldg(scale);
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < pixels; p += gridDim.x * (uint64_t)blockDim.x) {
        const float4 c = __ldg(image + p);
        const float* t = target + 3 * p;
        const float dr = c.x - __ldg(t), dg = c.y - __ldg(t + 1), db = c.z - __ldg(t + 2);
        grad[p] = make_float4(sc * (2.0f * dr), sc * (2.0f * dg), sc * (2.0f * db), 0.0f);
    }
}

static uint32_t grid_for(uint64_t n) {
    const uint64_t b = (n + 255) / 256, cap = (uint64_t)device_sm_count() * 16u;
    return (uint32_t)(b < cap ? (b ? b : 1) : cap);
}

void launch_activate(uint32_t n, const float* means, const float* quats, const float* logs, const float* logits,
                     float* x, float* y, float* z, float* rot, float* scale_alpha, cudaStream_t st) {
    if (n == 0) return;
    k_activate<<<grid_for(n), 256, 0, st>>>(n, means, reinterpret_cast<const float4*>(quats), logs, logits, x, y, z,
                                             reinterpret_cast<float4*>(rot), reinterpret_cast<float4*>(scale_alpha));
}

uint32_t l2_loss_partials(uint64_t pixels) { return grid_for(pixels); }

void launch_l2_loss(const float* image, const float* target, uint64_t pixels, float* partial, cudaStream_t st) {
    k_l2_loss<<<grid_for(pixels), 256, 0, st>>>(reinterpret_cast<const float4*>(image), target, pixels, partial);
}

void launch_l2_loss_backward(const float* image, const float* target, uint64_t pixels, const float* scale,
                             float* grad, cudaStream_t st) {
    k_l2_loss_backward<<<grid_for(pixels), 256, 0, st>>>(reinterpret_cast<const float4*>(image), target, pixels, scale,
                                                         reinterpret_cast<float4*>(grad));
}

void launch_activate_backward(uint32_t n, const float* quats, const float* logs, const float* rot,
                              const float* scale_alpha, const float* gx, const float* gy, const float* gz,
                              const float* grot, const float* gsa, float* g_means, float* g_quats, float* g_logs,
                              float* g_logits, cudaStream_t st) {
    if (n == 0) return;
    k_activate_backward<<<grid_for(n), 256, 0, st>>>(
        n, reinterpret_cast<const float4*>(quats), logs, reinterpret_cast<const float4*>(rot),
        reinterpret_cast<const float4*>(scale_alpha), gx, gy, gz, reinterpret_cast<const float4*>(grot),
        reinterpret_cast<const float4*>(gsa), g_means, reinterpret_cast<float4*>(g_quats), g_logs, g_logits);
}

}  // namespace spl
