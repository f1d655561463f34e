// Onesweep LSD radix sort pass (sm_103a), the GPU depth sort of splatter (radixSortB/radixSortC,
// Lichtso/splatter src/shaders.wgsl:338-498) rebuilt for CUDA:
//   * warp-level multisplit ranking (digit match by eight ballots; the reference ranks with shared
//     atomics because WebGPU has no subgroup ops, shaders.wgsl:428-429), which makes every pass STABLE;
//   * one CTA of 256 threads ranks a tile of 4096 keys (16 per thread, warp-striped, so global loads
//     are coalesced and the warp order is the input order);
//   * the global digit offsets come from the digit histogram computed upstream (the reference's
//     radixSortA/radixSortB); the CTA scans it itself, so there is no separate scan launch;
//   * decoupled look-back per digit with epoch-tagged status words (no clears between passes or
//     frames) and bounded waits that raise an error bit instead of hanging;
//   * dynamic tile ids and a persistent grid, so a wait only ever targets a tile held by a running CTA;
//   * keys, then values, are scattered through shared memory so global writes are runs per digit.
#include <atomic>

#include "spl_device.cuh"

namespace spl {

constexpr int OS_THREADS = 256;
constexpr int OS_KPT = 16;
static_assert(OS_THREADS * OS_KPT == SORT_TILE, "tile size");

template <bool IOTA>
__global__ void __launch_bounds__(OS_THREADS, 3)
    k_onesweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in, uint32_t* __restrict__ keys_out,
               uint32_t* __restrict__ vals_out, const uint32_t* __restrict__ n_ptr, uint32_t n_cap,
               const uint32_t* __restrict__ hist256, uint64_t* status, uint32_t* tile_counter,
               const uint32_t* __restrict__ epoch_word, int shift, uint32_t spin_limit, uint32_t* err) {
    __shared__ uint32_t s_buf[SORT_TILE];
    __shared__ uint32_t s_whist[8][256];
    __shared__ uint32_t s_gbase[256];
    __shared__ uint32_t s_dstart[256];
    __shared__ uint32_t s_gofs[256];
    __shared__ uint32_t s_scan[8];
    __shared__ uint32_t s_tile;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
    const uint32_t n = min(*n_ptr, n_cap);
    const uint32_t ntiles = (n + SORT_TILE - 1) / SORT_TILE;
    const uint32_t epoch = *epoch_word;
    {
        // exclusive scan of the global histogram of this digit place -> global digit bases
        uint32_t tot;
        s_gbase[tid] = block_exclusive_scan_256(__ldg(hist256 + tid), s_scan, &tot);
    }
    const uint32_t lt = lanemask_lt();
    for (;;) {
        if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
#pragma unroll
        for (int k = 0; k < 8; ++k) s_whist[k][tid] = 0u;
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= ntiles) break;
        const uint32_t tbase = tile * SORT_TILE;
        const uint32_t base = tbase + w * 512u + lane;
        uint32_t key[OS_KPT], pos[OS_KPT], val[OS_KPT];
#pragma unroll
        for (int j = 0; j < OS_KPT; ++j) {
            const uint32_t e = base + 32u * j;
            key[j] = e < n ? __ldg(keys_in + e) : 0u;
            val[j] = e < n ? (IOTA ? e : __ldg(vals_in + e)) : 0u;  // loaded with the keys
        }
        // warp-level multisplit: rank of each key among equal digits of its warp, in input order
#pragma unroll
        for (int j = 0; j < OS_KPT; ++j) {
            const uint32_t e = base + 32u * j;
            const bool valid = e < n;
            const uint32_t d = (key[j] >> shift) & 255u;
            const uint32_t peers = match_digit(d, valid);
            uint32_t cnt = 0;
            if (valid) cnt = s_whist[w][d];
            __syncwarp();
            const uint32_t leader = 31u - __clz(peers);
            if (valid && lane == leader) s_whist[w][d] = cnt + __popc(peers);
            __syncwarp();
            pos[j] = cnt + __popc(peers & lt);
        }
        __syncthreads();
        // per digit (thread tid == digit): exclusive prefix over warps, tile count
        uint32_t tcount = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t c = s_whist[k][tid];
            s_whist[k][tid] = tcount;
            tcount += c;
        }
        lb_store(status + (size_t)tile * 256u + tid, lb_pack(epoch, tile == 0 ? LB_INC : LB_AGG, tcount));
        uint32_t ttot;
        const uint32_t dstart = block_exclusive_scan_256(tcount, s_scan, &ttot);
        const uint32_t before = tile == 0 ? 0u : lookback_digit(status, tile, tid, epoch, spin_limit, err);
        if (tile != 0) lb_store(status + (size_t)tile * 256u + tid, lb_pack(epoch, LB_INC, before + tcount));
        s_dstart[tid] = dstart;
        s_gofs[tid] = s_gbase[tid] + before - dstart;
        __syncthreads();
        // scatter keys into shared memory in tile-sorted order
#pragma unroll
        for (int j = 0; j < OS_KPT; ++j) {
            const uint32_t e = base + 32u * j;
            if (e < n) {
                const uint32_t d = (key[j] >> shift) & 255u;
                pos[j] += s_dstart[d] + s_whist[w][d];
                s_buf[pos[j]] = key[j];
            }
        }
        __syncthreads();
        const uint32_t tn = min((uint32_t)SORT_TILE, n - tbase);
        uint32_t dig[OS_KPT];
#pragma unroll
        for (int j = 0; j < OS_KPT; ++j) {
            const uint32_t i = tid + 256u * j;
            dig[j] = 0u;
            if (i < tn) {
                const uint32_t k = s_buf[i];
                dig[j] = (k >> shift) & 255u;
                const uint32_t g = s_gofs[dig[j]] + i;
                if (g < n) keys_out[g] = k;  // always true unless a look-back wait timed out
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < OS_KPT; ++j) {
            const uint32_t e = base + 32u * j;
            if (e < n) s_buf[pos[j]] = val[j];
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < OS_KPT; ++j) {
            const uint32_t i = tid + 256u * j;
            const uint32_t g = s_gofs[dig[j]] + i;
            if (i < tn && g < n) vals_out[g] = s_buf[i];
        }
        __syncthreads();
    }
}

uint32_t device_sm_count() {
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1u;
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v == 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) v = 1;
        cache[dev].store(v, std::memory_order_relaxed);
    }
    return (uint32_t)v;
}

struct OnesweepShape {
    int num_sms = 1, blocks_per_sm = 1;
};

// Queried once per process (a function-local static: safe when several host threads launch).
static const OnesweepShape& onesweep_shape() {
    static const OnesweepShape shape = [] {
        OnesweepShape s;
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&s.num_sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&s.blocks_per_sm, k_onesweep<false>, OS_THREADS, 0);
        if (s.blocks_per_sm < 1) s.blocks_per_sm = 1;
        if (s.num_sms < 1) s.num_sms = 1;
        return s;
    }();
    return shape;
}

void onesweep_prepare() { (void)onesweep_shape(); }

void launch_onesweep(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                     const uint32_t* n_ptr, uint32_t n_cap, const uint32_t* hist256, uint64_t* status,
                     uint32_t* tile_counter, const uint32_t* epoch_word, int shift, uint32_t spin_limit,
                     uint32_t* err, cudaStream_t st) {
    if (n_cap == 0) return;
    const OnesweepShape& shape = onesweep_shape();
    const uint32_t tiles = (n_cap + SORT_TILE - 1) / SORT_TILE;
    uint32_t grid = (uint32_t)(shape.num_sms * shape.blocks_per_sm);
    if (grid > tiles) grid = tiles;
    if (vals_in == nullptr)
        k_onesweep<true><<<grid, OS_THREADS, 0, st>>>(keys_in, vals_in, keys_out, vals_out, n_ptr, n_cap, hist256,
                                                       status, tile_counter, epoch_word, shift, spin_limit, err);
    else
        k_onesweep<false><<<grid, OS_THREADS, 0, st>>>(keys_in, vals_in, keys_out, vals_out, n_ptr, n_cap, hist256,
                                                        status, tile_counter, epoch_word, shift, spin_limit, err);
}

// Digit histograms of all four 8-bit places of `n` keys (the upsweep the standalone sort needs;
// the frame's depth sort gets its histograms from the cull kernel).
__global__ void __launch_bounds__(256) k_histogram(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ n_ptr,
                                                   uint32_t n_cap, uint32_t* hist) {
    __shared__ uint32_t s_h[1024];
    for (uint32_t i = threadIdx.x; i < 1024u; i += 256u) s_h[i] = 0u;
    __syncthreads();
    const uint32_t n = min(*n_ptr, n_cap);
    for (uint32_t i = blockIdx.x * 256u + threadIdx.x; i < n; i += gridDim.x * 256u) {
        const uint32_t k = __ldg(keys + i);
        atomicAdd(&s_h[k & 255u], 1u);
        atomicAdd(&s_h[256u + ((k >> 8) & 255u)], 1u);
        atomicAdd(&s_h[512u + ((k >> 16) & 255u)], 1u);
        atomicAdd(&s_h[768u + (k >> 24)], 1u);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < 1024u; i += 256u)
        if (s_h[i]) atomicAdd(hist + i, s_h[i]);
}

void launch_histogram(const uint32_t* keys, const uint32_t* n_ptr, uint32_t n_cap, uint32_t* hist4x256,
                      cudaStream_t st) {
    if (n_cap == 0) return;
    uint32_t grid = (n_cap + 255) / 256;
    if (grid > device_sm_count() * 4u) grid = device_sm_count() * 4u;
    k_histogram<<<grid, 256, 0, st>>>(keys, n_ptr, n_cap, hist4x256);
}

__global__ void k_set_count(uint32_t* dst, uint32_t value) { *dst = value; }

void launch_set_count(uint32_t* dst, uint32_t value, cudaStream_t st) { k_set_count<<<1, 1, 0, st>>>(dst, value); }

}  // namespace spl
