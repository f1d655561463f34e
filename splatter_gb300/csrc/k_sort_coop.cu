// All passes of a stable LSD radix sort in ONE cooperative launch (sm_103a).
//
// The reference's GPU depth sort (radixSortA/B/C, Lichtso/splatter src/shaders.wgsl:298-498) is a
// onesweep sort whose tiles learn their global digit offsets through a decoupled look-back chain.
// At splat-pipeline sizes (a few million keys, L2-resident) that chain — one L2 round trip per
// tile — dominates.  Here every CTA is resident (cooperative launch, one 1024-thread CTA per SM) and
// owns one contiguous segment of the input; each 8-bit pass is:
//   1. count: the segment's digit histogram -> cnt[digit][cta]                       (global)
//   2. bounded grid barrier
//   3. offsets: for each digit, the exclusive prefix over earlier CTAs plus the global digit base,
//      from one sweep over cnt[digit][*] (vector loads)
//   4. scatter, sub-tile by sub-tile (8192 keys): warp-level multisplit ranking (__match_any_sync),
//      per-digit warp prefixes, keys then values staged through shared memory and written as runs
//   5. bounded grid barrier (the next pass reads this pass's output)
// The ranking keeps equal digits in input order, so every pass is stable, like the onesweep passes.
// Every barrier wait is bounded: on timeout the error bit is raised and the kernel runs to its end
// (writes stay in bounds), so a missing CTA can never hang the GPU.
#include <cooperative_groups.h>

#include "spl_device.cuh"

namespace spl {

constexpr int CS_THREADS = 1024;
constexpr int CS_WARPS = CS_THREADS / 32;
constexpr int CS_KPT = 8;
constexpr int CS_TILE = CS_THREADS * CS_KPT;  // 8192 keys per sub-tile

struct CoopSmem {
    uint32_t buf[CS_TILE];             // 32 KB staging for keys, then values
    uint32_t wcnt[CS_WARPS][256];      // per-warp digit counts -> exclusive prefixes (32 KB)
    uint32_t part[4][256];             // partial sums of 8 warps each / of CTA quarters
    uint32_t base[256];                // global output base of each digit for this CTA
    uint32_t running[256];             // keys of each digit already written by this CTA
    uint32_t dstart[256];              // tile-local exclusive digit offsets
    uint32_t tcount[256];              // tile digit counts
    uint32_t scan[32];
};

__device__ __forceinline__ void grid_barrier(uint32_t* bar, uint32_t nblocks, uint32_t spin_limit, uint32_t* err) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile uint32_t* vgen = bar + 1;
        const uint32_t gen = *vgen;
        __threadfence();
        const uint32_t arrived = atomicAdd(bar, 1u);
        if (arrived == nblocks - 1u) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            uint32_t spins = 0;
            while (*vgen == gen) {
                if (++spins > spin_limit) {
                    atomicOr(err, SPL_DEV_ERR_LOOKBACK);
                    break;
                }
                if (spins > 32) __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// Block-wide exclusive scan over 256 values held by threads 0..255 (other threads pass 0 and ignore
// the result).  Uses sm->scan; all 1024 threads must call it.
__device__ __forceinline__ uint32_t scan256(uint32_t v, uint32_t* scan, uint32_t* total) {
    const uint32_t tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL_MASK, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31 && w < 8) scan[w] = x;
    __syncthreads();
    uint32_t pre = 0, tot = 0;
#pragma unroll
    for (uint32_t i = 0; i < 8; ++i) {
        const uint32_t s = scan[i];
        pre += i < w ? s : 0u;
        tot += s;
    }
    __syncthreads();
    *total = tot;
    return pre + x - v;
}

// keys0 -> keys1 -> keys0 ... for `passes` passes starting at bit `shift0`; vals likewise (both value
// buffers are real; with iota_first the values read by pass 0 are the input positions instead of
// vals0).  The result of pass p is in keys1/vals1 for even p and keys0/vals0 for odd p.
__global__ void __launch_bounds__(CS_THREADS, 1)
    k_sort_coop(uint32_t* keys0, uint32_t* keys1, uint32_t* vals0, uint32_t* vals1, int iota_first,
                const uint32_t* n_ptr, uint32_t n_cap, int passes, int shift0, uint32_t* cnt /*[256][gridDim]*/,
                uint32_t* bar, uint32_t spin_limit, uint32_t* err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CoopSmem& sm = *reinterpret_cast<CoopSmem*>(smem_raw);
    const uint32_t tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
    const uint32_t G = gridDim.x, c = blockIdx.x;
    const uint32_t n = min(*n_ptr, n_cap);
    // contiguous segments, 256-aligned
    uint32_t seg = (n + G - 1) / G;
    seg = (seg + 255u) & ~255u;
    const uint32_t s_begin = min(c * seg, n), s_end = min(s_begin + seg, n);
    const uint32_t lt = lanemask_lt();
    for (int p = 0; p < passes; ++p) {
        const int shift = shift0 + 8 * p;
        const uint32_t* kin = (p & 1) ? keys1 : keys0;
        const uint32_t* vin = (p & 1) ? vals1 : vals0;
        uint32_t* kout = (p & 1) ? keys0 : keys1;
        uint32_t* vout = (p & 1) ? vals0 : vals1;
        const bool iota = (p == 0 && iota_first != 0);
        // ---- 1. count ----
        if (tid < 256) sm.part[0][tid] = 0u;
        __syncthreads();
        // (loads bypass L1: the previous pass's output was written by other CTAs of this launch)
        for (uint32_t e = s_begin + tid; e < s_end; e += CS_THREADS)
            atomicAdd(&sm.part[0][(__ldcg(kin + e) >> shift) & 255u], 1u);
        __syncthreads();
        if (tid < 256) cnt[(size_t)tid * G + c] = sm.part[0][tid];
        grid_barrier(bar, G, spin_limit, err);
        // ---- 3. offsets: thread (d = tid & 255, q = tid >> 8) sweeps a quarter of cnt[d][*] ----
        {
            const uint32_t d = tid & 255u, q = tid >> 8;
            const uint32_t per = (G + 3u) / 4u;
            const uint32_t cb = q * per, ce = min(cb + per, G);
            uint32_t pre = 0, tot = 0;
            const uint32_t* row = cnt + (size_t)d * G;
            for (uint32_t k = cb; k < ce; ++k) {
                const uint32_t v = __ldcg(row + k);
                tot += v;
                pre += k < c ? v : 0u;
            }
            sm.part[q][d] = tot;
            sm.wcnt[q][d] = pre;  // wcnt is free here; borrow 4 rows
        }
        __syncthreads();
        uint32_t dtotal = 0, dpre = 0;
        if (tid < 256) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                dtotal += sm.part[q][tid];
                dpre += sm.wcnt[q][tid];
            }
        }
        uint32_t all;
        const uint32_t gdig = scan256(tid < 256 ? dtotal : 0u, sm.scan, &all);
        if (tid < 256) {
            sm.base[tid] = gdig + dpre;
            sm.running[tid] = 0u;
        }
        __syncthreads();
        // ---- 4. scatter, sub-tile by sub-tile ----
        for (uint32_t tb = s_begin; tb < s_end; tb += CS_TILE) {
            const uint32_t tn = min((uint32_t)CS_TILE, s_end - tb);
#pragma unroll
            for (int k = 0; k < 8; ++k) sm.wcnt[w][lane + 32 * k] = 0u;
            __syncwarp();
            uint32_t key[CS_KPT], pos[CS_KPT];
            const uint32_t wb = tb + w * 256u + lane;
#pragma unroll
            for (int j = 0; j < CS_KPT; ++j) {
                const uint32_t e = wb + 32u * j;
                key[j] = e < tb + tn ? __ldcg(kin + e) : 0u;
            }
#pragma unroll
            for (int j = 0; j < CS_KPT; ++j) {
                const uint32_t e = wb + 32u * j;
                const bool valid = e < tb + tn;
                const uint32_t d = valid ? (key[j] >> shift) & 255u : 256u;
                const uint32_t peers = __match_any_sync(FULL_MASK, d);
                uint32_t cur = 0;
                if (valid) cur = sm.wcnt[w][d];
                __syncwarp();
                if (valid && lane == 31u - __clz(peers)) sm.wcnt[w][d] = cur + __popc(peers);
                __syncwarp();
                pos[j] = cur + __popc(peers & lt);
            }
            __syncthreads();
            // per digit: exclusive prefix over the 32 warps (thread (d, q) handles warps 8q..8q+7)
            {
                const uint32_t d = tid & 255u, q = tid >> 8;
                uint32_t s = 0;
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const uint32_t v = sm.wcnt[8 * q + k][d];
                    sm.wcnt[8 * q + k][d] = s;
                    s += v;
                }
                sm.part[q][d] = s;
            }
            __syncthreads();
            {
                const uint32_t d = tid & 255u, q = tid >> 8;
                uint32_t add = 0;
#pragma unroll
                for (uint32_t k = 0; k < 4; ++k) add += k < q ? sm.part[k][d] : 0u;
                if (add) {
#pragma unroll
                    for (int k = 0; k < 8; ++k) sm.wcnt[8 * q + k][d] += add;
                }
            }
            const uint32_t tc = tid < 256 ? ((sm.part[0][tid] + sm.part[1][tid]) + (sm.part[2][tid] + sm.part[3][tid])) : 0u;
            uint32_t tt;
            const uint32_t ds = scan256(tc, sm.scan, &tt);  // contains __syncthreads
            if (tid < 256) {
                sm.dstart[tid] = ds;
                sm.tcount[tid] = tc;
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < CS_KPT; ++j) {
                const uint32_t e = wb + 32u * j;
                if (e < tb + tn) {
                    const uint32_t d = (key[j] >> shift) & 255u;
                    pos[j] += sm.dstart[d] + sm.wcnt[w][d];
                    sm.buf[pos[j]] = key[j];
                }
            }
            __syncthreads();
            uint32_t dig[CS_KPT];
#pragma unroll
            for (int j = 0; j < CS_KPT; ++j) {
                const uint32_t i = tid + CS_THREADS * j;
                dig[j] = 0u;
                if (i < tn) {
                    const uint32_t k = sm.buf[i];
                    dig[j] = (k >> shift) & 255u;
                    const uint32_t g = sm.base[dig[j]] + sm.running[dig[j]] + (i - sm.dstart[dig[j]]);
                    if (g < n) kout[g] = k;
                }
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < CS_KPT; ++j) {
                const uint32_t e = wb + 32u * j;
                if (e < tb + tn) sm.buf[pos[j]] = iota ? e : __ldcg(vin + e);
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < CS_KPT; ++j) {
                const uint32_t i = tid + CS_THREADS * j;
                if (i < tn) {
                    const uint32_t g = sm.base[dig[j]] + sm.running[dig[j]] + (i - sm.dstart[dig[j]]);
                    if (g < n) vout[g] = sm.buf[i];
                }
            }
            __syncthreads();
            if (tid < 256) sm.running[tid] += sm.tcount[tid];
            __syncthreads();
        }
        // ---- 5. the next pass reads this pass's output ----
        grid_barrier(bar, G, spin_limit, err);
    }
}

static int g_cs_grid = 0;

int sort_coop_grid() {
    if (g_cs_grid == 0) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(k_sort_coop, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(CoopSmem));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sort_coop, CS_THREADS, sizeof(CoopSmem));
        g_cs_grid = sms * (per > 0 ? per : 1);
    }
    return g_cs_grid;
}

cudaError_t launch_sort_coop(uint32_t* keys0, uint32_t* keys1, uint32_t* vals0, uint32_t* vals1, bool iota_first,
                             const uint32_t* n_ptr, uint32_t n_cap, int passes, int shift0, uint32_t* cnt,
                             uint32_t* bar, uint32_t spin_limit, uint32_t* err, cudaStream_t st) {
    if (n_cap == 0 || passes == 0) return cudaSuccess;
    int grid = sort_coop_grid();
    const uint32_t want = (n_cap + 2047u) / 2048u;
    if ((uint32_t)grid > want) grid = (int)want;
    if (grid < 1) grid = 1;
    int iota = iota_first ? 1 : 0;
    void* args[] = {&keys0, &keys1, &vals0, &vals1, &iota, (void*)&n_ptr, &n_cap, &passes, &shift0, &cnt, &bar,
                    &spin_limit, &err};
    return cudaLaunchCooperativeKernel((const void*)k_sort_coop, dim3(grid), dim3(CS_THREADS), args,
                                       sizeof(CoopSmem), st);
}

}  // namespace spl
