// Device-side building blocks shared by the splat-pipeline kernels (sm_103a).
//
// Floating point: every translation unit is compiled with -fmad=false and IEEE division/sqrt, so
// the FP32 results follow the written operation order exactly (the WGSL order of
// Lichtso/splatter src/shaders.wgsl).  Where a fused multiply-add is wanted it is written as
// fmaf() explicitly.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "spl_types.h"

namespace spl {

constexpr uint32_t FULL_MASK = 0xFFFFFFFFu;

// ------------------------------------------------------------------------------------------------
// Decoupled look-back status words: [epoch:32 | INC:1 | AGG:1 | value:30].  A word is only valid
// when its epoch equals the frame's epoch, so status arrays never need clearing between frames.
// ------------------------------------------------------------------------------------------------
constexpr uint32_t LB_AGG = 0x40000000u;
constexpr uint32_t LB_INC = 0x80000000u;
constexpr uint32_t LB_VAL = 0x3FFFFFFFu;

__device__ __forceinline__ uint64_t lb_pack(uint32_t epoch, uint32_t flags, uint32_t value) {
    return ((uint64_t)epoch << 32) | (uint64_t)(flags | (value & LB_VAL));
}
__device__ __forceinline__ void lb_store(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t lb_load(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Warp-cooperative look-back for a single running total (stream compaction, bin offsets).
// Called by all 32 lanes of one warp; returns the exclusive prefix of `tile` (sum of all earlier
// tiles).  Every wait is bounded: after spin_limit polls the error flag is raised and the missing
// predecessors count as zero, so the kernel always terminates.
__device__ __forceinline__ uint32_t lookback_single(const uint64_t* status, uint32_t tile, uint32_t epoch,
                                                    uint32_t spin_limit, uint32_t* err) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t excl = 0;
    int64_t window = (int64_t)tile - 1;
    while (window >= 0) {
        const int64_t idx = window - (int64_t)lane;
        uint64_t s = 0;
        uint32_t ready_mask = 0, inc_mask = 0, need = 0;
        uint32_t spins = 0;
        bool timed_out = false;
        for (;;) {
            s = idx >= 0 ? lb_load(status + idx) : lb_pack(epoch, LB_INC, 0);
            const bool ready = (uint32_t)(s >> 32) == epoch && ((uint32_t)s & (LB_AGG | LB_INC)) != 0;
            const bool inc = ready && ((uint32_t)s & LB_INC) != 0;
            ready_mask = __ballot_sync(FULL_MASK, ready);
            inc_mask = __ballot_sync(FULL_MASK, inc);
            const int stop = inc_mask ? __ffs(inc_mask) - 1 : 31;
            need = stop == 31 ? FULL_MASK : ((2u << stop) - 1u);
            if ((ready_mask & need) == need) break;
            if (++spins > spin_limit) {
                timed_out = true;
                break;
            }
            if (spins > 16) __nanosleep(64);
        }
        if (timed_out) {
            if (lane == 0) atomicOr(err, SPL_DEV_ERR_LOOKBACK);
            return excl;
        }
        const uint32_t v = (need >> lane) & 1u ? ((uint32_t)s & LB_VAL) : 0u;
        excl += __reduce_add_sync(FULL_MASK, v);
        if (inc_mask) break;
        window -= 32;
    }
    return excl;
}

// Per-thread look-back for one digit of a onesweep pass (status has 256 words per tile).
__device__ __forceinline__ uint32_t lookback_digit(const uint64_t* status, uint32_t tile, uint32_t digit,
                                                   uint32_t epoch, uint32_t spin_limit, uint32_t* err) {
    uint32_t excl = 0;
    int64_t p = (int64_t)tile - 1;
    while (p >= 0) {
        uint64_t s;
        uint32_t spins = 0;
        for (;;) {
            s = lb_load(status + (size_t)p * 256u + digit);
            if ((uint32_t)(s >> 32) == epoch && ((uint32_t)s & (LB_AGG | LB_INC)) != 0) break;
            if (++spins > spin_limit) {
                atomicOr(err, SPL_DEV_ERR_LOOKBACK);
                return excl;
            }
            if (spins > 16) __nanosleep(64);
        }
        excl += (uint32_t)s & LB_VAL;
        if ((uint32_t)s & LB_INC) break;
        --p;
    }
    return excl;
}

// ------------------------------------------------------------------------------------------------
// exp: Cody–Waite range reduction (x = n*ln2 + r with ln2 split into a 16-bit head and a tail),
// degree-7 Taylor polynomial of e^r on |r| <= ln2/2 in Horner form with fused multiply-adds, and a
// two-factor scaling by 2^n that keeps both factors normal.  Bit-identical to the oracle's exp.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ float spl_expf(float x) {
    if (x != x) return x;
    if (x > 88.72283935546875f) return __int_as_float(0x7f800000);
    if (x < -103.97208404541015625f) return 0.0f;
    const float n = rintf(__fmul_rn(x, 1.44269502162933349609375f));
    float r = fmaf(n, -0.693145751953125f, x);
    r = fmaf(n, -1.428606765330187045e-06f, r);
    float p = 1.98412698412698412e-04f;
    p = fmaf(p, r, 1.38888888888888889e-03f);
    p = fmaf(p, r, 8.33333333333333333e-03f);
    p = fmaf(p, r, 4.16666666666666667e-02f);
    p = fmaf(p, r, 1.66666666666666667e-01f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    const int ni = (int)n;
    const int h = ni / 2;
    const float s1 = __int_as_float((h + 127) << 23);
    const float s2 = __int_as_float((ni - h + 127) << 23);
    return __fmul_rn(__fmul_rn(p, s1), s2);
}

// spl_expf restricted to finite x <= 0 (the fragment falloff): the same result bit for bit.  For
// n >= -125 the two-factor scaling reduces to one multiply by 2^n, exact because p * 2^n is normal.
__device__ __forceinline__ float spl_expf_nonpos(float x) {
    if (x < -87.0f) return spl_expf(x);
    const float n = rintf(__fmul_rn(x, 1.44269502162933349609375f));
    float r = fmaf(n, -0.693145751953125f, x);
    r = fmaf(n, -1.428606765330187045e-06f, r);
    float p = 1.98412698412698412e-04f;
    p = fmaf(p, r, 1.38888888888888889e-03f);
    p = fmaf(p, r, 8.33333333333333333e-03f);
    p = fmaf(p, r, 4.16666666666666667e-02f);
    p = fmaf(p, r, 1.66666666666666667e-01f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    return __fmul_rn(p, __int_as_float(((int)n + 127) << 23));
}

// The loader's transform of one splat (Scene::load_chunk, scene.rs:225-250): quaternion normalised,
// log-scales clamped to their mean +- 5 and exponentiated, opacity logit through the sigmoid.
__device__ __forceinline__ void activate_splat(float q0, float q1, float q2, float q3, float l0, float l1, float l2,
                                               float logit, float4& rot, float4& scale_alpha) {
    const float inv = 1.0f / sqrtf(((q0 * q0 + q1 * q1) + q2 * q2) + q3 * q3);
    rot = make_float4(q0 * inv, q1 * inv, q2 * inv, q3 * inv);
    const float avg = ((l0 + l1) + l2) / 3.0f;
    const float lo = avg - 5.0f, hi = avg + 5.0f;
    const float s0 = spl_expf(fminf(fmaxf(l0, lo), hi));
    const float s1 = spl_expf(fminf(fmaxf(l1, lo), hi));
    const float s2 = spl_expf(fminf(fmaxf(l2, lo), hi));
    const float a = 1.0f / (1.0f + spl_expf(-logit));
    scale_alpha = make_float4(s0, s1, s2, a);
}

__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }

// WGSL u32(f32): truncate, saturate, NaN -> 0.
__device__ __forceinline__ uint32_t sat_u32(float x) { return __float2uint_rz(x); }

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Lanes whose 8-bit digit equals this lane's (valid lanes only), from eight ballots: the warp-level
// multisplit match without MATCH.ANY, whose latency dominated the ranking.
__device__ __forceinline__ uint32_t match_digit(uint32_t d, bool valid) {
    uint32_t peers = __ballot_sync(FULL_MASK, valid);
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const bool bit = (d >> b) & 1u;
        const uint32_t m = __ballot_sync(FULL_MASK, bit);
        peers &= bit ? m : ~m;
    }
    return peers;
}

// Block-wide exclusive scan of one u32 per thread (blockDim.x == 256).  `scratch` holds 8 words.
__device__ __forceinline__ uint32_t block_exclusive_scan_256(uint32_t v, uint32_t* scratch, uint32_t* total) {
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL_MASK, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) scratch[w] = x;
    __syncthreads();
    uint32_t wpre = 0, tot = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const uint32_t s = scratch[i];
        wpre += (uint32_t)i < w ? s : 0u;
        tot += s;
    }
    __syncthreads();
    *total = tot;
    return wpre + x - v;
}

}  // namespace spl
