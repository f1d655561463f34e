// Compute rasteriser for the splat records (sm_103a).  The reference draws each splat as a rotated
// rectangle (triangle strip, renderer.rs:275-283) through the fixed-function rasteriser, runs the
// Gaussian fragment (shaders.wgsl:580-592) and blends front-to-back into a Bgra8Unorm target with
// destination alpha as transmittance (renderer.rs:260-271).  There is no fixed-function unit here,
// so the frame is tiled into 16x16-pixel tiles:
//   k_bin          - for each drawn entry in depth order, the tiles its pixel box touches; emitted as
//                    (tile id, record slot) pairs at offsets from a decoupled look-back scan, with
//                    load-balanced emission inside the CTA (a max-scan over the entries' first
//                    pairs) and, for the onesweep sort, the tile-id digit histograms
//   (a stable radix sort of the pairs by tile id, so each tile's list stays in depth order)
//   k_tile_ranges  - start/end of each tile's run in the sorted pair list
//   k_tile_order   - the raster's tile order: most pairs first
//   k_raster       - one CTA per tile, one thread per pixel; records staged through shared memory in
//                    batches of 256, per-pixel record lists from the boxes (bit-transposed ballots),
//                    exact coverage test, falloff, blend, and early exit once every pixel of the tile
//                    is opaque
#include "spl_device.cuh"

namespace spl {

// ------------------------------------------------------------------------------------------------
constexpr int BIN_PER = BIN_TILE / 256;  // consecutive draw entries per thread (thread order = depth order)
template <bool ORDERED, bool HIST>
__global__ void __launch_bounds__(256) k_bin(const uint32_t* __restrict__ order, const uint2* __restrict__ boxes,
                                             FrameCounters* fc, int mode, const uint32_t* __restrict__ epoch_word,
                                             uint64_t* status, uint32_t* __restrict__ pair_keys,
                                             uint32_t* __restrict__ pair_vals, uint32_t pair_cap, int tiles_x,
                                             uint32_t spin_limit) {
    __shared__ uint32_t s_off[BIN_TILE];  // exclusive pair offsets of the tile's entries
    __shared__ uint32_t s_slot[BIN_TILE];
    __shared__ uint32_t s_box[BIN_TILE];  // tx0 | ty0 << 16
    __shared__ uint16_t s_bw[BIN_TILE];
    __shared__ uint32_t s_map[1024];  // emission step: entry + 1 at each entry's first pair position
    __shared__ uint32_t s_hist[HIST ? 768 : 1];
    __shared__ uint32_t s_scan[8];
    __shared__ uint32_t s_tile, s_epoch, s_base, s_draw;
    const uint32_t tid = threadIdx.x;
    if (tid == 0) {
        s_tile = atomicAdd(&fc->tile_counter[8], 1u);
        s_epoch = *epoch_word;
        const uint32_t V = fc->visible;
        uint32_t draw = V;
        if (mode == DS_GPU) draw = V - fc->keys_all_ones;
        else if (mode == DS_GPU_INDIRECT) draw = V - fc->keys_top_ff;
        s_draw = draw;
    }
    if (HIST) {
        s_hist[tid] = 0u;
        s_hist[tid + 256] = 0u;
        s_hist[tid + 512] = 0u;
    }
    __syncthreads();
    const uint32_t tile = s_tile, epoch = s_epoch, draw = s_draw;
    const uint32_t ntiles = (draw + BIN_TILE - 1) / BIN_TILE;
    if (tile >= ntiles) {
        if (tile == 0 && tid == 0) {  // nothing to draw at all
            fc->draw = 0;
            fc->pairs = 0;
        }
        return;
    }
    if (tile == 0 && tid == 0) fc->draw = draw;
    // per-entry tile counts (4 consecutive entries per thread keep the thread order = depth order)
    uint32_t cnt[BIN_PER], tsum = 0;
#pragma unroll
    for (int e = 0; e < BIN_PER; ++e) {
        const uint32_t r = tile * BIN_TILE + tid * (uint32_t)BIN_PER + e;
        uint32_t c = 0, slot = 0, box = 0, bw = 0;
        if (r < draw) {
            slot = ORDERED ? __ldg(order + r) : r;
            const uint2 bb = __ldg(boxes + slot);
            const uint32_t lo = bb.x, hi = bb.y;
            const uint32_t x0 = lo & 0xFFFFu, y0 = lo >> 16, x1 = hi & 0xFFFFu, y1 = hi >> 16;
            if (x0 <= x1 && y0 <= y1) {
                const uint32_t tx0 = x0 / TILE_PIXELS, tx1 = x1 / TILE_PIXELS;
                const uint32_t ty0 = y0 / TILE_PIXELS, ty1 = y1 / TILE_PIXELS;
                bw = tx1 - tx0 + 1u;
                c = bw * (ty1 - ty0 + 1u);
                box = tx0 | (ty0 << 16);
            }
        }
        cnt[e] = c;
        s_slot[tid * BIN_PER + e] = slot;
        s_box[tid * BIN_PER + e] = box;
        s_bw[tid * BIN_PER + e] = (uint16_t)bw;
        tsum += c;
    }
    uint32_t btot;
    uint32_t off = block_exclusive_scan_256(tsum, s_scan, &btot);
#pragma unroll
    for (int e = 0; e < BIN_PER; ++e) {
        s_off[tid * BIN_PER + e] = off;
        off += cnt[e];
    }
    if (tid < 32) {
        if (tid == 0) lb_store(status + tile, lb_pack(epoch, tile == 0 ? LB_INC : LB_AGG, btot));
        const uint32_t excl = tile == 0 ? 0u : lookback_single(status, tile, epoch, spin_limit, &fc->err);
        if (tid == 0) {
            if (tile != 0) lb_store(status + tile, lb_pack(epoch, LB_INC, excl + btot));
            s_base = excl;
            if (tile == ntiles - 1) {
                fc->pairs = excl + btot;
                if (excl + btot > pair_cap) atomicOr(&fc->err, SPL_DEV_ERR_PAIR_OVERFLOW);
            }
        }
    }
    __syncthreads();
    const uint32_t gbase = s_base;
    // Load-balanced emission, 1024 pairs per step: pair q of this CTA belongs to the last entry whose
    // offset is <= q.  Each entry with pairs marks its first pair's position (entry + 1), and an
    // inclusive max-scan over the step's positions (carrying the previous step's last entry) hands
    // every position its entry; thread t emits positions 4t .. 4t + 3.
    uint32_t carry = 0u;
    for (uint32_t q0 = 0; q0 < btot; q0 += 1024u) {
#pragma unroll
        for (int k = 0; k < 4; ++k) s_map[tid * 4 + k] = 0u;
        __syncthreads();
#pragma unroll
        for (int e = 0; e < BIN_PER; ++e) {
            const uint32_t ei = tid * (uint32_t)BIN_PER + e;
            const uint32_t o = s_off[ei];
            if (cnt[e] != 0u && o >= q0 && o - q0 < 1024u) s_map[o - q0] = ei + 1u;
        }
        __syncthreads();
        uint32_t v[4], m = carry;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            m = max(m, s_map[tid * 4 + k]);
            v[k] = m;  // thread-local inclusive max (with the carry)
        }
        uint32_t x = m;  // inclusive max-scan of the thread maxima over the warp
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL_MASK, x, o);
            if ((tid & 31u) >= (uint32_t)o) x = max(x, y);
        }
        const uint32_t before_in_warp = __shfl_up_sync(FULL_MASK, x, 1);
        if ((tid & 31u) == 31u) s_scan[tid >> 5] = x;
        __syncthreads();
        uint32_t before = (tid & 31u) ? before_in_warp : 0u, all = 0u;
#pragma unroll
        for (uint32_t wi = 0; wi < 8; ++wi) {
            const uint32_t sw = s_scan[wi];
            before = wi < (tid >> 5) ? max(before, sw) : before;
            all = max(all, sw);
        }
        carry = all;  // the entry at the step's last position: the carry into the next step
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t q = q0 + tid * 4u + k;
            const uint32_t marked = max(before, v[k]);  // >= 1: position 0 of the first step is marked
            if (q >= btot || marked == 0u) break;
            const uint32_t e = marked - 1u;
            const uint32_t li = q - s_off[e];
            const uint32_t bw = s_bw[e], box = s_box[e];
            // li / bw and li % bw (li < 2^24): float estimate, corrected by one step
            uint32_t dy = __float2uint_rz(__fdividef((float)li, (float)bw));
            int32_t dx = (int32_t)(li - dy * bw);
            if (dx < 0) {
                --dy;
                dx += (int32_t)bw;
            } else if (dx >= (int32_t)bw) {
                ++dy;
                dx -= (int32_t)bw;
            }
            const uint32_t tid_tile = ((box >> 16) + dy) * (uint32_t)tiles_x + (box & 0xFFFFu) + (uint32_t)dx;
            const uint32_t g = gbase + q;
            if (g < pair_cap) {
                pair_keys[g] = tid_tile;
                pair_vals[g] = s_slot[e];
                if (HIST) {
                    atomicAdd(&s_hist[tid_tile & 255u], 1u);
                    atomicAdd(&s_hist[256u + ((tid_tile >> 8) & 255u)], 1u);
                    atomicAdd(&s_hist[512u + ((tid_tile >> 16) & 255u)], 1u);
                }
            }
        }
        __syncthreads();  // s_map and s_scan are rewritten by the next step
    }
    if (HIST) {
        __syncthreads();
        for (uint32_t i = tid; i < 768u; i += 256u) {
            const uint32_t v = s_hist[i];
            if (v) atomicAdd(&fc->hist_pairs[0][0] + i, v);
        }
    }
}

void launch_bin(int mode, bool hist, const uint32_t* order, const uint2* boxes, FrameCounters* fc,
                const uint32_t* epoch_word, uint64_t* status, uint32_t* pair_keys, uint32_t* pair_vals,
                uint32_t pair_cap, int tiles_x, uint32_t max_n, uint32_t spin_limit, cudaStream_t st) {
    const uint32_t grid = max_n == 0 ? 1u : (max_n + BIN_TILE - 1) / BIN_TILE;
    auto k = order ? (hist ? k_bin<true, true> : k_bin<true, false>) : (hist ? k_bin<false, true> : k_bin<false, false>);
    k<<<grid, 256, 0, st>>>(order, boxes, fc, mode, epoch_word, status, pair_keys, pair_vals, pair_cap, tiles_x,
                            spin_limit);
}

// ------------------------------------------------------------------------------------------------
__global__ void k_tile_ranges(const uint32_t* __restrict__ keys, const FrameCounters* __restrict__ fc,
                              uint32_t pair_cap, uint2* ranges) {
    const uint32_t P = min(fc->pairs, pair_cap);
    // four keys per thread (one 16-byte load; the neighbours across the group edges loaded singly)
    const uint32_t groups = (P + 3u) / 4u;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < groups; g += gridDim.x * blockDim.x) {
        const uint32_t i0 = g * 4u;
        uint32_t k[4];
        if (i0 + 4u <= P) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(keys + i0));
            k[0] = v.x;
            k[1] = v.y;
            k[2] = v.z;
            k[3] = v.w;
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) k[j] = i0 + j < P ? __ldg(keys + i0 + j) : 0u;
        }
        const bool has_prev = i0 > 0u, has_next = i0 + 4u < P;
        const uint32_t prev = has_prev ? __ldg(keys + i0 - 1u) : 0u;
        const uint32_t next = has_next ? __ldg(keys + i0 + 4u) : 0u;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t i = i0 + j;
            if (i >= P) break;
            const bool starts = j > 0 ? k[j - 1] != k[j] : (!has_prev || prev != k[j]);
            const bool ends = i + 1u == P || (j < 3 ? k[j + 1] != k[j] : next != k[j]);
            if (starts) ranges[k[j]].x = i;
            if (ends) ranges[k[j]].y = i + 1u;
        }
    }
}

void launch_tile_ranges(const uint32_t* pair_keys, const FrameCounters* fc, uint32_t pair_cap, uint2* ranges,
                        cudaStream_t st) {
    if (pair_cap == 0) return;
    uint32_t grid = (pair_cap + 255) / 256;
    if (grid > device_sm_count() * 8u) grid = device_sm_count() * 8u;
    k_tile_ranges<<<grid, 256, 0, st>>>(pair_keys, fc, pair_cap, ranges);
}

// ------------------------------------------------------------------------------------------------
// The raster's tile order: tiles with more (tile, splat) pairs first, in buckets of half an octave of
// the pair count (2 buckets per power of two), empty tiles last.  Tiles take very different times
// (dense clusters against open sky); started in row-major order, a few heavy tiles could begin in
// the last wave and set the kernel's end, while heavy-first is close to the longest-processing-time
// schedule.  Tiles are independent, so the order changes no pixel.  One CTA: a bucket histogram, its
// scan and a scatter of tile indices (the order within a bucket does not matter).
constexpr int ORDER_BUCKETS = 65;

__device__ __forceinline__ uint32_t order_bucket(uint2 r) {
    const uint32_t c = r.y - r.x;
    if (c == 0u) return ORDER_BUCKETS - 1;
    const uint32_t l = 31u - __clz(c);                     // floor(log2 c)
    const uint32_t half = l > 0u ? (c >> (l - 1u)) & 1u : 0u;  // the bit after the leading one
    return 63u - (2u * l + half);                          // more pairs -> smaller bucket
}

constexpr uint32_t ORDER_SMEM_TILES = 32768;  // tiles whose bucket is kept in shared memory (2160p: 32,400)

__global__ void __launch_bounds__(1024) k_tile_order(const uint2* __restrict__ ranges, uint32_t ntiles,
                                                     uint32_t* __restrict__ order) {
    __shared__ uint32_t cnt[ORDER_BUCKETS];
    __shared__ uint8_t bkt[ORDER_SMEM_TILES];
    const uint32_t lane = threadIdx.x & 31u;
    if (threadIdx.x < ORDER_BUCKETS) cnt[threadIdx.x] = 0u;
    __syncthreads();
    // histogram; lanes of a warp with the same bucket add once (most tiles share a few buckets)
#pragma unroll 4
    for (uint32_t t = threadIdx.x; t < ntiles; t += blockDim.x) {
        const uint32_t b = order_bucket(__ldg(ranges + t));
        if (t < ORDER_SMEM_TILES) bkt[t] = (uint8_t)b;
        const uint32_t peers = __match_any_sync(__activemask(), b);
        if (lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&cnt[b], __popc(peers));
    }
    __syncthreads();
    if (threadIdx.x < 32) {  // exclusive scan of the 65 bucket counts by one warp
        uint32_t carry = 0;
        for (int b0 = 0; b0 < ORDER_BUCKETS; b0 += 32) {
            const int b = b0 + (int)threadIdx.x;
            const uint32_t v = b < ORDER_BUCKETS ? cnt[b] : 0u;
            uint32_t x = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL_MASK, x, o);
                if ((int)threadIdx.x >= o) x += y;
            }
            if (b < ORDER_BUCKETS) cnt[b] = carry + x - v;
            carry += __shfl_sync(FULL_MASK, x, 31);
        }
    }
    __syncthreads();
    // scatter: one atomic per (warp, bucket), lanes take consecutive places in lane order
    for (uint32_t t = threadIdx.x; t < ntiles; t += blockDim.x) {
        const uint32_t b = t < ORDER_SMEM_TILES ? bkt[t] : order_bucket(__ldg(ranges + t));
        const uint32_t peers = __match_any_sync(__activemask(), b);
        const uint32_t leader = (uint32_t)(__ffs(peers) - 1);
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&cnt[b], __popc(peers));
        base = __shfl_sync(peers, base, (int)leader);
        order[base + __popc(peers & lanemask_lt())] = t;
    }
}

// ------------------------------------------------------------------------------------------------
constexpr int RASTER_BATCH = 256;

// One CTA per 16x16 tile, one thread per pixel.  Warp w owns the strip of rows 2w, 2w+1; lane l holds
// column 2 (l / 4) + (l & 1) and row 2w + ((l >> 1) & 1), so the strip's 2x2 blocks are groups of four
// lanes.  The tile's records (depth order) are staged through shared memory in batches of 256; the
// thread staging a record also forms its mask of the lanes (pixels) it may draw in each of the eight
// strips.  Warp-wide bit transposes, four 32-record words at a time, turn its strip's masks into each
// pixel's list of the batch's records.  The warp then walks the 32 lists of the whole batch at once: in
// every iteration each pixel takes its next record, so one pass of the per-pixel code serves as many
// splats as there are lanes with work (most splats here cover a few pixels).  Per pixel: coverage
// test, falloff, 1/255 discard, blend — the operations of the oracle's raster_tile in the same order,
// so the image is bit-identical.  Lists are walked in depth order per pixel, a warp whose pixels are
// all finished skips the rest, and the CTA stops once every pixel is finished (T == 0 in unorm8 mode,
// T < 1e-4 in fp32 mode).
// Block indices g (of the eight along a warp's strip) with |c + s g| <= T, widened conservatively:
// the quotients are clamped to [-1, 9] before rounding outwards, so their float error (a few ulp of
// at most 9) stays far below the 1e-3 widening.  Empty when lo > hi.
__device__ __forceinline__ void g_interval(float c, float s, float rs, float T, int& lo, int& hi) {
    if (fabsf(s) < 1e-30f) {
        const bool all = fabsf(c) <= T;
        lo = all ? -1 : 1;
        hi = all ? 9 : 0;
        return;
    }
    const float q1 = (-T - c) * rs, q2 = (T - c) * rs;  // rs = 1 / s (IEEE: finite, within half an ulp)
    const float a = fminf(fmaxf(fminf(q1, q2), -1.0f), 9.0f), b = fminf(fmaxf(fmaxf(q1, q2), -1.0f), 9.0f);
    lo = (int)ceilf(a - 1e-3f);
    hi = (int)floorf(b + 1e-3f);
}

// Lanes of a warp's 2x16-pixel strip whose column is >= c (0 <= c <= 16); lane l holds column
// 2 (l / 4) + (l & 1) and row (l >> 1) & 1.
__device__ __forceinline__ uint32_t strip_columns_from(int c) {
    const int k = c >> 1;
    if (c & 1) return (uint32_t)(0xFFFFFFFFull << (4 * k + 4)) | (uint32_t)(0xAull << (4 * k));
    return (uint32_t)(0xFFFFFFFFull << (4 * k));
}

// N 32x32 bit-matrix transposes across the warp: afterwards bit i of x[c] in lane l is bit l of the
// old x[c] in lane i.  Each step d exchanges lane-index bit d with bit-index bit d; the N words go
// through each step together, so their independent shuffle chains overlap their latency (one word
// at a time, the list building took a quarter of the raster's warp time at 6M splats, 1080p).
template <int N>
__device__ __forceinline__ void transpose_lane_bits_n(uint32_t* x, uint32_t lane) {
    const uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const uint32_t d = 16u >> k, m = masks[k];
#pragma unroll
        for (int c = 0; c < N; ++c) {
            const uint32_t p = __shfl_xor_sync(FULL_MASK, x[c], (int)d);
            x[c] = (lane & d) ? ((x[c] & ~m) | ((p >> d) & m)) : ((x[c] & m) | ((p & m) << d));
        }
    }
}

template <bool RECT, int BLEND>
__global__ void __launch_bounds__(256, 6) k_raster(const uint2* __restrict__ ranges, const uint32_t* __restrict__ tile_order,
                                                const uint32_t* __restrict__ pair_vals,
                                                const float4* __restrict__ rec, int W, int H, int tiles_x, float margin,
                                                float psx, float psy, void* __restrict__ out) {
    __shared__ float4 s_q0[RASTER_BATCH], s_q1[RASTER_BATCH], s_q2[RASTER_BATCH];
    __shared__ float4 s_q3[RECT ? 1 : RASTER_BATCH];
    __shared__ float s_lut[256];
    __shared__ uint32_t s_pm[8][RASTER_BATCH];             // [strip][record]: lane masks of the batch's records
    __shared__ uint32_t s_plist[RASTER_BATCH / 32][256];  // [word][pixel]: the pixels' record lists of the batch
    const uint32_t tid = threadIdx.x, lane = tid & 31u, w = tid >> 5;
    const uint32_t grp = lane >> 2, li = lane & 3u;
    const int tile = tile_order ? (int)__ldg(tile_order + blockIdx.x) : (int)blockIdx.x;
    const int tx = tile % tiles_x, ty = tile / tiles_x;
    const int bx0 = tx * TILE_PIXELS + 2 * (int)grp;  // this lane's 2x2 block
    const int by0 = ty * TILE_PIXELS + 2 * (int)w;
    const int px = bx0 + (int)(li & 1u), py = by0 + (int)(li >> 1);
    const float X = (float)px + 0.5f, Y = (float)py + 0.5f;
    s_lut[tid] = (float)tid / 255.0f;
    const uint2 rg = ranges[tile];
    const bool inside = px < W && py < H;
    bool done = !inside;
    bool warp_done = __all_sync(FULL_MASK, done);
    int cr = 0, cg = 0, cb = 0, ta = 255;
    float fr = 0.0f, fg = 0.0f, fb = 0.0f, ft = 1.0f;
    const float alpha_min = 1.0f / 255.0f;
    const int wx0 = tx * TILE_PIXELS;  // the eight blocks of this warp: columns wx0 + 2g, + 1, rows by0, by0+1
    for (uint32_t b = rg.x; b < rg.y; b += RASTER_BATCH) {
        __syncthreads();
        const uint32_t i = b + tid;
        if (i < rg.y) {
            const uint32_t slot = __ldg(pair_vals + i);
            const float4* r = rec + (size_t)slot * 4;
            const float4 r0 = __ldg(r + 0), r1 = __ldg(r + 1), r2 = __ldg(r + 2);
            s_q0[tid] = r0;
            s_q1[tid] = r1;
            s_q2[tid] = r2;
            if (!RECT) s_q3[tid] = __ldg(r + 3);
            // The record's lane mask for each of the tile's eight strips (rows 2w, 2w + 1): the pixels
            // inside its pixel box and, for rectangles, only in the 2x2 blocks where some pixel
            // centre may lie in the rectangle: over a block's four centres tc lies within tc(block
            // centre) +- ext (half the block's extent mapped by |A|, widened by a rounding bound far
            // above the per-pixel FMA chains' error), and along the strip the block centre's tc is
            // c + 2g A, so |c + 2g A| <= margin + ext is an interval of block indices g.  Skipped
            // pixels are not drawn by the record: the image is unchanged.
#pragma unroll
            for (int sw = 0; sw < 8; ++sw) s_pm[sw][tid] = 0u;
            const uint32_t lo = __float_as_uint(r1.w), hi = __float_as_uint(r2.w);
            const int x0 = (int)(lo & 0xFFFFu), y0 = (int)(lo >> 16);
            const int x1 = (int)(hi & 0xFFFFu), y1 = (int)(hi >> 16);
            if (x0 <= x1 && y0 <= y1) {
                const int ty0 = ty * TILE_PIXELS;
                const int sw0 = max((y0 - ty0) >> 1, 0), sw1 = min((y1 - ty0) >> 1, 7);  // floor halves
                float rsx = 0.0f, rsy = 0.0f;
                if (RECT) {
                    rsx = 1.0f / (2.0f * r0.x);
                    rsy = 1.0f / (2.0f * r0.w);
                }
                for (int sw = sw0; sw <= sw1; ++sw) {
                    const int sy0 = ty0 + 2 * sw;  // the strip's first row
                    int ca = x0 - wx0, cb = x1 - wx0;  // strip columns of the box
                    if (RECT) {
                        const float Xc = (float)(wx0 + 1), Yc = (float)(sy0 + 1);  // block 0's centre
                        const float Xm = (float)(wx0 + 16), Ym = (float)(sy0 + 2);
                        const float cx = fmaf(r0.y, Yc, fmaf(r0.x, Xc, r0.z));
                        const float cy = fmaf(r1.x, Yc, fmaf(r0.w, Xc, r1.y));
                        const float Tx = margin + 0.5f * (fabsf(r0.x) + fabsf(r0.y)) +
                                         1e-6f * (fabsf(r0.x) * Xm + fabsf(r0.y) * Ym + fabsf(r0.z));
                        const float Ty = margin + 0.5f * (fabsf(r0.w) + fabsf(r1.x)) +
                                         1e-6f * (fabsf(r0.w) * Xm + fabsf(r1.x) * Ym + fabsf(r1.y));
                        int lx, hx, ly, hy;
                        g_interval(cx, 2.0f * r0.x, rsx, Tx, lx, hx);
                        g_interval(cy, 2.0f * r0.w, rsy, Ty, ly, hy);
                        ca = max(ca, 2 * max(lx, ly));
                        cb = min(cb, 2 * min(hx, hy) + 1);
                    }
                    ca = max(ca, 0);
                    cb = min(cb, 15);
                    if (ca <= cb) {
                        uint32_t pm = strip_columns_from(ca) & ~strip_columns_from(cb + 1);
                        if (y0 > sy0) pm &= 0xCCCCCCCCu;      // lanes of the strip's second row
                        if (y1 < sy0 + 1) pm &= 0x33333333u;  // lanes of its first row
                        s_pm[sw][tid] = pm;
                    }
                }
            }
        }
        __syncthreads();
        const uint32_t cnt = min((uint32_t)RASTER_BATCH, rg.y - b);
        if (!warp_done) {
            // Per-pixel lists of the batch, 32 records per step: the strip's lane masks of records
            // 32c + l, transposed so that lane p holds word c of pixel p's list (bit i: record 32c + i),
            // kept in s_plist; bit c of `nz` marks a non-empty word.
            uint32_t nz = 0u;
            uint32_t t[RASTER_BATCH / 32];
#pragma unroll
            for (int c = 0; c < RASTER_BATCH / 32; ++c) {
                const uint32_t jl = (uint32_t)c * 32u + lane;
                t[c] = jl < cnt ? s_pm[w][jl] : 0u;
            }
            // four words at a time; a group whose 128 records miss the strip stays zero
            if (__any_sync(FULL_MASK, ((t[0] | t[1]) | (t[2] | t[3])) != 0u)) transpose_lane_bits_n<4>(t, lane);
            if (cnt > 128u && __any_sync(FULL_MASK, ((t[4] | t[5]) | (t[6] | t[7])) != 0u))
                transpose_lane_bits_n<4>(t + 4, lane);
#pragma unroll
            for (int c = 0; c < RASTER_BATCH / 32; ++c) {
                s_plist[c][tid] = t[c];
                nz |= (t[c] != 0u ? 1u : 0u) << c;
            }
            // Walk the 32 lists at once across the whole batch: in every iteration each pixel takes its
            // next record.  The warp leaves once every pixel is finished or has walked its list.
            uint32_t cur = 0u, cbase = 0u;
            while (true) {
                if (cur == 0u && nz != 0u) {
                    const uint32_t c = (uint32_t)(__ffs(nz) - 1);
                    nz &= nz - 1u;
                    cur = s_plist[c][tid];
                    cbase = c * 32u;
                }
                if (!__any_sync(FULL_MASK, cur != 0u && !done)) break;
                if (cur == 0u || done) continue;
                const uint32_t j = cbase + (uint32_t)(__ffs(cur) - 1);
                cur &= cur - 1u;
                const float4 q1 = s_q1[j], q2 = s_q2[j];
                const float4 q0 = s_q0[j];
                const float tcx = fmaf(q0.y, Y, fmaf(q0.x, X, q0.z));
                const float tcy = fmaf(q1.x, Y, fmaf(q0.w, X, q1.y));
                if (RECT) {
                    if (!(fabsf(tcx) <= margin && fabsf(tcy) <= margin)) continue;
                } else {
                    const float4 q3 = s_q3[j];
                    const float dx = fmaf(psx, X, q3.x), dy = fmaf(psy, Y, q3.y);
                    if (!(fabsf(dx) <= q3.z && fabsf(dy) <= q3.z)) continue;
                }
                const float power = fmaf(tcx, tcx, tcy * tcy);
                const float alpha = q1.z * spl_expf_nonpos(-0.5f * power);
                if (alpha < alpha_min) continue;
                // __saturatef == clamp to [0, 1] (NaN -> 0); __float2int_rn == (int)rintf
                const float sr = __saturatef(q2.x * alpha), sg = __saturatef(q2.y * alpha);
                const float sb = __saturatef(q2.z * alpha), sa = __saturatef(alpha);
                if (BLEND == 0) {
                    const float dA = s_lut[ta];
                    cr = __float2int_rn(__saturatef(sr * dA + s_lut[cr]) * 255.0f);
                    cg = __float2int_rn(__saturatef(sg * dA + s_lut[cg]) * 255.0f);
                    cb = __float2int_rn(__saturatef(sb * dA + s_lut[cb]) * 255.0f);
                    ta = __float2int_rn(__saturatef(dA * (1.0f - sa)) * 255.0f);
                    done = ta == 0;
                } else {
                    fr = sr * ft + fr;
                    fg = sg * ft + fg;
                    fb = sb * ft + fb;
                    ft = ft * (1.0f - sa);
                    done = ft < FP32_T_MIN;
                }
            }
            warp_done = __all_sync(FULL_MASK, done);
        }
        if (__syncthreads_and(done)) break;
    }
    if (inside) {
        const size_t pix = (size_t)py * (size_t)W + (size_t)px;
        if (BLEND == 0) {
            reinterpret_cast<uchar4*>(out)[pix] = make_uchar4((unsigned char)cr, (unsigned char)cg, (unsigned char)cb,
                                                              (unsigned char)ta);
        } else {
            reinterpret_cast<float4*>(out)[pix] = make_float4(fr, fg, fb, ft);
        }
    }
}

const void* raster_kernel(bool rect, int blend) {
    if (rect) return blend == 0 ? reinterpret_cast<const void*>(&k_raster<true, 0>)
                                : reinterpret_cast<const void*>(&k_raster<true, 1>);
    return blend == 0 ? reinterpret_cast<const void*>(&k_raster<false, 0>)
                      : reinterpret_cast<const void*>(&k_raster<false, 1>);
}

void launch_raster(bool rect, int blend, const uint2* ranges, uint32_t* tile_order, const uint32_t* pair_vals,
                   const float4* rec, const Uniforms& u, void* out, cudaStream_t st) {
    const int W = (int)u.image_size[0], H = (int)u.image_size[1];
    const int tiles_x = (W + TILE_PIXELS - 1) / TILE_PIXELS, tiles_y = (H + TILE_PIXELS - 1) / TILE_PIXELS;
    const int grid = tiles_x * tiles_y;
    if (grid == 0) return;
    const float psx = (2.0f * u.view_size[0]) / (float)W;
    const float psy = -((2.0f * u.view_size[1]) / (float)H);
    if (tile_order) k_tile_order<<<1, 1024, 0, st>>>(ranges, (uint32_t)grid, tile_order);
    const uint32_t* o = tile_order;
    if (rect) {
        if (blend == 0)
            k_raster<true, 0><<<grid, 256, 0, st>>>(ranges, o, pair_vals, rec, W, H, tiles_x, u.margin, psx, psy, out);
        else
            k_raster<true, 1><<<grid, 256, 0, st>>>(ranges, o, pair_vals, rec, W, H, tiles_x, u.margin, psx, psy, out);
    } else {
        if (blend == 0)
            k_raster<false, 0><<<grid, 256, 0, st>>>(ranges, o, pair_vals, rec, W, H, tiles_x, u.margin, psx, psy, out);
        else
            k_raster<false, 1><<<grid, 256, 0, st>>>(ranges, o, pair_vals, rec, W, H, tiles_x, u.margin, psx, psy, out);
    }
}

}  // namespace spl
