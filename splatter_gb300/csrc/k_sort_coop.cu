// All passes of a stable LSD radix sort in ONE cooperative launch (sm_103a).
//
// The reference's GPU depth sort (radixSortA/B/C, Lichtso/splatter src/shaders.wgsl:298-498) is a
// onesweep sort whose tiles learn their global digit offsets through a decoupled look-back chain.
// At splat-pipeline sizes (a few million keys, L2-resident) that chain — one L2 round trip per
// tile — dominates.  Here every CTA is resident (cooperative launch, two 512-thread CTAs per SM) and
// owns one contiguous segment of the input; each 8-bit pass is:
//   1. count: the segment's digit histogram -> cnt[digit][cta]                       (global)
//   2. bounded grid barrier; the digit rows, dealt round robin over the CTAs, are scanned in place
//      (exclusive prefix over CTAs, by one warp or, for a few CTAs, one thread per row) and their
//      totals written; bounded grid barrier
//   3. offsets: each CTA reads its column of prefixes and the 256 totals (global digit bases)
//   4. scatter, sub-tile by sub-tile (4096 keys): warp-level multisplit ranking (digit match by eight
//      ballots),
//      per-digit warp prefixes, keys and values staged together through shared memory and written as runs
//   5. bounded grid barrier (the next pass reads this pass's output)
// The ranking keeps equal digits in input order, so every pass is stable, like the onesweep passes.
// Every barrier wait is bounded: on timeout the error bit is raised and the kernel runs to its end
// (writes stay in bounds), so a missing CTA can never hang the GPU.  The barrier word counts the
// launch's arrivals and must be zero when the launch starts (each sort of a frame has its own word in
// the frame counters, which the frame start zeroes).
#include "spl_device.cuh"

namespace spl {

constexpr int CS_THREADS = 512;               // two CTAs per SM
constexpr int CS_WARPS = CS_THREADS / 32;
constexpr int CS_NQ = CS_THREADS / 256;        // threads per digit in the per-digit phases
constexpr int CS_WPQ = CS_WARPS / CS_NQ;       // warps summed by one of those threads
constexpr int CS_KPT = 8;
constexpr int CS_TILE = CS_THREADS * CS_KPT;  // 4096 keys per sub-tile
constexpr int CS_SCAN_RUN = 16;               // count-table entries per lane in the row scan: grids <= 512
static_assert(CS_THREADS % 256 == 0, "the per-digit phases map 256 digits onto groups of threads");
static_assert(CS_THREADS == 512 && CS_WARPS == 16, "the sub-tile scan maps digit t / 2 and 8 warps to thread t");

struct CoopSmem {
    uint32_t buf[CS_TILE];             // keys of the sub-tile in digit order
    uint32_t vbuf[CS_TILE];            // their values
    uint32_t wcnt[CS_WARPS][256];      // per-warp digit counts -> exclusive prefixes
    uint32_t part[CS_NQ][256];         // partial sums over groups of warps / of the count table
    uint32_t base[256];                // global output base of each digit for this CTA
    uint32_t running[256];             // keys of each digit already written by this CTA
    uint32_t dstart[256];              // tile-local exclusive digit offsets
    uint32_t tcount[256];              // tile digit counts
    uint32_t scan[CS_WARPS];
};

// Grid barrier on a word that only counts arrivals (zero when the launch starts): the b-th barrier of
// the launch (b = 0, 1, ...) waits until *bar reaches (b + 1) * nblocks.  Releasing takes only the
// last arrival's atomic: no reset and no generation word on the critical path (those cost two more
// L2 round trips per barrier).
__device__ __forceinline__ void grid_barrier(uint32_t* bar, uint32_t target, uint32_t spin_limit, uint32_t* err) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(bar, 1u);
        const volatile uint32_t* v = bar;
        uint32_t spins = 0;
        while (*v < target) {
            if (++spins > spin_limit) {
                atomicOr(err, SPL_DEV_ERR_LOOKBACK);
                break;
            }
            // a barrier of this launch already timed out: the later ones would too, each after its own
            // spin limit; stop waiting (the frame reports the error)
            if ((spins & 1023u) == 0u && (*(volatile uint32_t*)err & SPL_DEV_ERR_LOOKBACK)) break;
            if (spins > 32) __nanosleep(32);
        }
        __threadfence();
    }
    __syncthreads();
}

// Block-wide exclusive scan over 256 values held by threads 0..255 (other threads pass 0 and ignore
// the result).  Uses sm->scan; every thread of the CTA must call it.
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

// Ranks one sub-tile's keys (key[j] is element wb + 32 j, valid below `end`) by the digit at `shift`
// (warp-level multisplit: equal digits keep their input order) and stages keys and values in digit
// order in sm.buf / sm.vbuf; sm.dstart / sm.tcount receive the sub-tile's digit offsets and counts.
// Every thread of the CTA calls it; it ends with a CTA barrier.
__device__ __forceinline__ void stage_subtile(CoopSmem& sm, const uint32_t (&key)[CS_KPT], const uint32_t (&val)[CS_KPT],
                                              uint32_t wb, uint32_t end, int shift, uint32_t lt) {
    const uint32_t tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
#pragma unroll
    for (int k = 0; k < 8; ++k) sm.wcnt[w][lane + 32 * k] = 0u;
    __syncwarp();
    uint32_t pos[CS_KPT];
#pragma unroll
    for (int j = 0; j < CS_KPT; ++j) {
        const uint32_t e = wb + 32u * j;
        const bool valid = e < end;
        const uint32_t d = (key[j] >> shift) & 255u;
        const uint32_t peers = match_digit(d, valid);
        uint32_t cur = 0;
        if (valid) cur = sm.wcnt[w][d];
        __syncwarp();
        if (valid && lane == 31u - __clz(peers)) sm.wcnt[w][d] = cur + __popc(peers);
        __syncwarp();
        pos[j] = cur + __popc(peers & lt);
    }
    __syncthreads();
    // One exclusive scan of the count table in (digit, warp) order gives every (warp, digit) its
    // first position in the sub-tile: thread t owns digit t / 2 and half of the warps; the thread
    // sums go through a warp scan and the warp totals.  dstart / tcount: each digit's start and count.
    {
        constexpr int HW = CS_WARPS / 2;
        const uint32_t d = tid >> 1, w0 = (tid & 1u) * HW;
        uint32_t c8[HW], sum = 0;
#pragma unroll
        for (int k = 0; k < HW; ++k) {
            c8[k] = sm.wcnt[w0 + k][d];
            sum += c8[k];
        }
        uint32_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL_MASK, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31u) sm.scan[w] = x;
        __syncthreads();
        uint32_t wpre = 0;
#pragma unroll
        for (uint32_t i = 0; i < (uint32_t)CS_WARPS; ++i) wpre += i < w ? sm.scan[i] : 0u;
        const uint32_t excl = wpre + x - sum;
        uint32_t run = excl;
#pragma unroll
        for (int k = 0; k < HW; ++k) {
            sm.wcnt[w0 + k][d] = run;
            run += c8[k];
        }
        const uint32_t first = __shfl_xor_sync(FULL_MASK, excl, 1);  // the digit's other half
        if (tid & 1u) {
            sm.dstart[d] = first;
            sm.tcount[d] = run - first;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < CS_KPT; ++j) {
        const uint32_t e = wb + 32u * j;
        if (e < end) {
            const uint32_t d = (key[j] >> shift) & 255u;
            const uint32_t p = pos[j] + sm.wcnt[w][d];
            sm.buf[p] = key[j];
            sm.vbuf[p] = val[j];
        }
    }
    __syncthreads();
}

// keys0 -> keys1 -> keys0 ... for `passes` passes starting at bit `shift0`; vals likewise (both value
// buffers are real; with iota_first the values read by pass 0 are the input positions instead of
// vals0).  The result of pass p is in keys1/vals1 for even p and keys0/vals0 for odd p (for at most
// one sub-tile of keys only the last pass's buffers are written).
__global__ void __launch_bounds__(CS_THREADS, 2)
    k_sort_coop(uint32_t* keys0, uint32_t* keys1, uint32_t* vals0, uint32_t* vals1, int iota_first,
                const uint32_t* n_ptr, uint32_t n_cap, int passes, int shift0, uint32_t* cnt /*[256][Gp] + tot[256]*/,
                uint32_t* bar, uint32_t spin_limit, uint32_t* err) {
    // cnt rows: [256][Gp], Gp = the working CTAs rounded up to a multiple of 4 (16-byte rows)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CoopSmem& sm = *reinterpret_cast<CoopSmem*>(smem_raw);
    const uint32_t tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
    const uint32_t c = blockIdx.x;
    const uint32_t n = min(*n_ptr, n_cap);
    // Contiguous segments, 256-aligned and at least one sub-tile long.  The live count is read on
    // the device (a captured graph replays with any count up to n_cap), so the grid is sized for
    // n_cap; CTAs past the last segment leave before the first barrier, which counts only the G
    // CTAs that work: a small sort pays for a few CTAs' barriers, not the whole grid's.
    uint32_t seg = (n + gridDim.x - 1) / gridDim.x;
    seg = max((seg + 255u) & ~255u, (uint32_t)CS_TILE);
    const uint32_t G = (n + seg - 1) / seg;
    if (c >= G) return;
    const uint32_t lt = lanemask_lt();
    if (G == 1u) {
        // n <= CS_TILE: one sub-tile.  Every pass ranks and stages it in shared memory (no count
        // table, no grid barriers); the keys are read once and written once, to the buffers the last
        // pass writes (keys1/vals1 after an odd number of passes, keys0/vals0 after an even one).
        uint32_t key[CS_KPT], val[CS_KPT];
        const uint32_t wb = w * (32u * CS_KPT) + lane;
#pragma unroll
        for (int j = 0; j < CS_KPT; ++j) {
            const uint32_t e = wb + 32u * j;
            const bool ok = e < n;
            key[j] = ok ? __ldcg(keys0 + e) : 0u;
            val[j] = ok ? (iota_first ? e : __ldcg(vals0 + e)) : 0u;
        }
        for (int p = 0; p < passes; ++p) {
            stage_subtile(sm, key, val, wb, n, shift0 + 8 * p, lt);
            if (p + 1 < passes) {
#pragma unroll
                for (int j = 0; j < CS_KPT; ++j) {
                    const uint32_t e = wb + 32u * j;
                    if (e < n) {
                        key[j] = sm.buf[e];
                        val[j] = sm.vbuf[e];
                    }
                }
                __syncthreads();
            }
        }
        uint32_t* kout = (passes & 1) ? keys1 : keys0;
        uint32_t* vout = (passes & 1) ? vals1 : vals0;
#pragma unroll
        for (int j = 0; j < CS_KPT; ++j) {
            const uint32_t i = tid + CS_THREADS * j;
            if (i < n) {
                kout[i] = sm.buf[i];
                vout[i] = sm.vbuf[i];
            }
        }
        return;
    }
    const uint32_t Gp = (G + 3u) & ~3u;  // padded row stride of cnt (16-byte rows)
    uint32_t bar_target = 0u;             // arrivals that release the next grid barrier
    uint32_t* tot = cnt + (size_t)256 * Gp;  // per-digit totals of a pass
    const uint32_t s_begin = c * seg, s_end = min(s_begin + seg, n);
    for (int p = 0; p < passes; ++p) {
        const int shift = shift0 + 8 * p;
        const uint32_t* kin = (p & 1) ? keys1 : keys0;
        const uint32_t* vin = (p & 1) ? vals1 : vals0;
        uint32_t* kout = (p & 1) ? keys0 : keys1;
        uint32_t* vout = (p & 1) ? vals0 : vals1;
        const bool iota = (p == 0 && iota_first != 0);
        // ---- 1. count: per-warp histograms (shared atomics) ----
#pragma unroll
        for (int k = 0; k < 8; ++k) sm.wcnt[w][lane + 32 * k] = 0u;
        __syncwarp();
        {
            // 16-byte loads (segments start 256-aligned), four in flight per thread; the loads bypass
            // L1 because the previous pass's output was written by other CTAs of this launch
            // s_begin is a multiple of 256 unless the segment is empty (s_begin == s_end == n)
            const uint32_t v_begin = s_begin >> 2, v_end = max(v_begin, s_end >> 2);
            const uint4* kin4 = reinterpret_cast<const uint4*>(kin);
            for (uint32_t v0 = v_begin; v0 < v_end; v0 += 4u * CS_THREADS) {
                uint4 q[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const uint32_t vi = v0 + (uint32_t)u * CS_THREADS + tid;
                    q[u] = vi < v_end ? __ldcg(kin4 + vi) : make_uint4(0u, 0u, 0u, 0u);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (v0 + (uint32_t)u * CS_THREADS + tid < v_end) {
                        atomicAdd(&sm.wcnt[w][(q[u].x >> shift) & 255u], 1u);
                        atomicAdd(&sm.wcnt[w][(q[u].y >> shift) & 255u], 1u);
                        atomicAdd(&sm.wcnt[w][(q[u].z >> shift) & 255u], 1u);
                        atomicAdd(&sm.wcnt[w][(q[u].w >> shift) & 255u], 1u);
                    }
                }
            }
            // tail (fewer than 4 keys past the last 16-byte group)
            for (uint32_t e = max(v_end << 2, s_begin) + tid; e < s_end; e += CS_THREADS)
                atomicAdd(&sm.wcnt[w][(__ldcg(kin + e) >> shift) & 255u], 1u);
        }
        __syncthreads();
        {
            const uint32_t d = tid & 255u, q = tid >> 8;
            uint32_t acc = 0;
#pragma unroll
            for (int k = 0; k < CS_WPQ; ++k) acc += sm.wcnt[CS_WPQ * q + k][d];
            sm.part[q][d] = acc;
        }
        __syncthreads();
        if (tid < 256) {
            uint32_t acc = 0;
#pragma unroll
            for (int q = 0; q < CS_NQ; ++q) acc += sm.part[q][tid];
            cnt[(size_t)tid * Gp + c] = acc;
        }
        __syncthreads();
        grid_barrier(bar, bar_target += G, spin_limit, err);
        // ---- 3a. distributed scan: digit row d of cnt[d][0..G) becomes its exclusive prefix over
        //          the CTAs and its total goes to tot[d].  The rows are dealt round robin over the
        //          CTAs, so every row's loads are in flight at once (one L2 round trip): with at most
        //          CS_SCAN_RUN CTAs one thread scans a row (d = tid * G + c), otherwise one warp
        //          (d = w * G + c), each lane a run of consecutive entries, a warp scan of the run
        //          sums giving the runs' offsets ----
        if (G <= (uint32_t)CS_SCAN_RUN) {
            const uint32_t d = tid * G + c;
            if (d < 256u) {
                uint32_t* row = cnt + (size_t)d * Gp;
                uint32_t v[CS_SCAN_RUN];
#pragma unroll
                for (int j = 0; j < CS_SCAN_RUN; ++j) v[j] = (uint32_t)j < G ? __ldcg(row + j) : 0u;
                uint32_t run = 0;
#pragma unroll
                for (int j = 0; j < CS_SCAN_RUN; ++j) {
                    if ((uint32_t)j < G) row[j] = run;
                    run += v[j];
                }
                tot[d] = run;
            }
        } else {
            const uint32_t d = w * G + c;  // warp-uniform
            if (d < 256u) {
                const uint32_t per = (G + 31u) / 32u;  // entries per lane, <= CS_SCAN_RUN
                uint32_t* row = cnt + (size_t)d * Gp;
                const uint32_t k0 = lane * per;
                uint32_t v[CS_SCAN_RUN];
                uint32_t sum = 0;
#pragma unroll
                for (int j = 0; j < CS_SCAN_RUN; ++j) {
                    const uint32_t k = k0 + (uint32_t)j;
                    v[j] = ((uint32_t)j < per && k < G) ? __ldcg(row + k) : 0u;
                    sum += v[j];
                }
                uint32_t x = sum;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(FULL_MASK, x, o);
                    if (lane >= (uint32_t)o) x += y;
                }
                uint32_t run = x - sum;
#pragma unroll
                for (int j = 0; j < CS_SCAN_RUN; ++j) {
                    const uint32_t k = k0 + (uint32_t)j;
                    if ((uint32_t)j < per && k < G) row[k] = run;
                    run += v[j];
                }
                if (lane == 31u) tot[d] = x;
            }
        }
        grid_barrier(bar, bar_target += G, spin_limit, err);
        // ---- 3b. offsets: this CTA's column of prefixes plus the global digit bases ----
        {
            uint32_t dtotal = 0, dpre = 0;
            if (tid < 256) {
                dpre = __ldcg(cnt + (size_t)tid * Gp + c);
                dtotal = __ldcg(tot + tid);
            }
            uint32_t all;
            const uint32_t gdig = scan256(tid < 256 ? dtotal : 0u, sm.scan, &all);
            if (tid < 256) {
                sm.base[tid] = gdig + dpre;
                sm.running[tid] = 0u;
            }
            __syncthreads();
        }
        // ---- 4. scatter, sub-tile by sub-tile ----
        for (uint32_t tb = s_begin; tb < s_end; tb += CS_TILE) {
            const uint32_t tn = min((uint32_t)CS_TILE, s_end - tb);
            uint32_t key[CS_KPT], val[CS_KPT];
            const uint32_t wb = tb + w * (32u * CS_KPT) + lane;  // warp w owns 32 x CS_KPT consecutive keys
#pragma unroll
            for (int j = 0; j < CS_KPT; ++j) {
                const uint32_t e = wb + 32u * j;
                const bool ok = e < tb + tn;
                key[j] = ok ? __ldcg(kin + e) : 0u;
                val[j] = ok ? (iota ? e : __ldcg(vin + e)) : 0u;
            }
            stage_subtile(sm, key, val, wb, tb + tn, shift, lt);
            // keys and values leave together: each digit's run is consecutive in the output
#pragma unroll
            for (int j = 0; j < CS_KPT; ++j) {
                const uint32_t i = tid + CS_THREADS * j;
                if (i < tn) {
                    const uint32_t k = sm.buf[i];
                    const uint32_t d = (k >> shift) & 255u;
                    const uint32_t g = sm.base[d] + sm.running[d] + (i - sm.dstart[d]);
                    if (g < n) {
                        kout[g] = k;
                        vout[g] = sm.vbuf[i];
                    }
                }
            }
            __syncthreads();
            // read by the next sub-tile's writes only, after its barriers
            if (tid < 256) sm.running[tid] += sm.tcount[tid];
        }
        // ---- 5. the next pass reads this pass's output ----
        grid_barrier(bar, bar_target += G, spin_limit, err);
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
        if (g_cs_grid > 32 * CS_SCAN_RUN) g_cs_grid = 32 * CS_SCAN_RUN;
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
