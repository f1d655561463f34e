// spl_sort_pairs_no_alloc: the stable onesweep pair sort with its scratch in a file-scope device
// array instead of memory from cudaMalloc.
//
// Why: some callers of this library cannot allocate device memory when they sort — a host that
// hands every byte of device memory to its own pool up front (so cudaMalloc would fail or bypass its
// accounting), a plug-in that may only touch the buffers it is given, or a loop that must not take
// the device-wide synchronisation a cudaMalloc may imply.  They pass the input and output arrays;
// this entry point finds everything else in g_noalloc_scratch, which the library reserves once per
// device when the module loads and keeps until the process exits.
//
// Limits and sharing:
//   * at most SPL_NO_ALLOC_MAX_PAIRS (262,144) pairs per call; larger counts are rejected;
//   * the scratch is 2.6 MB per device (temporary keys/values, look-back status words, counters);
//   * every call on a device uses the same scratch, and the scratch keeps what the last call left
//     there.  The counters that must start at zero (error word included) are zeroed by the call
//     itself; the look-back status words carry an epoch that each call advances, so stale words are
//     never read as valid;
//   * calls whose GPU work overlaps (two streams, or two host threads without ordering) race on the
//     scratch and give wrong results: order them on one stream or synchronise between them;
//   * the first call on a device looks up the array's device address with cudaGetSymbolAddress
//     (with that device current); make that first call before any stream capture begins.  The
//     address is cached per device ordinal, so only the primary context is supported;
//   * a look-back wait that runs out sets the scratch's error word instead of hanging;
//     spl_sort_pairs_no_alloc_status reads it back after the call's work (allocating nothing).
#include <mutex>

#include "../../include/splatter.h"
#include "spl_types.h"

namespace spl {

constexpr uint32_t NA_MAX = SPL_NO_ALLOC_MAX_PAIRS;
constexpr uint32_t NA_TILES = (NA_MAX + SORT_TILE - 1) / SORT_TILE;

struct NoAllocScratch {
    FrameCounters fc;
    uint32_t epoch;
    uint32_t pad[63];
    uint32_t tmp_keys[NA_MAX];
    uint32_t tmp_vals[NA_MAX];
    uint64_t status[4][NA_TILES * 256];
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

namespace {
std::mutex g_na_mu;
void* g_na_addr[64] = {};  // device address of g_noalloc_scratch, per device ordinal
}  // namespace

}  // namespace spl

using namespace spl;

int spl_internal_fail(int code, const char* fmt, ...);

// Device address of g_noalloc_scratch on the current device, looked up once per device (with that
// device current) and cached.
static int scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return spl_internal_fail(SPL_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return spl_internal_fail(SPL_ERR_INVALID, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return spl_internal_fail(SPL_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch): %s",
                                     cudaGetErrorString(e));
        g_na_addr[dev] = p;
    }
    *out = g_na_addr[dev];
    return SPL_OK;
}

extern "C" int spl_sort_pairs_no_alloc(const uint32_t* keys_in, const uint32_t* values_in, uint32_t* keys_out,
                                       uint32_t* values_out, uint64_t count, uint32_t key_bits, void* stream) {
    if (!keys_in || !values_in || !keys_out || !values_out)
        return spl_internal_fail(SPL_ERR_INVALID, "NULL argument");
    if (count > NA_MAX)
        return spl_internal_fail(SPL_ERR_INVALID, "spl_sort_pairs_no_alloc sorts at most %u pairs, got %llu",
                                 (unsigned)NA_MAX, (unsigned long long)count);
    if (key_bits == 0 || key_bits > 32 || key_bits % 8 != 0)
        return spl_internal_fail(SPL_ERR_INVALID, "key_bits %u (must be 8, 16, 24 or 32)", key_bits);
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    if (count == 0) return SPL_OK;
    NoAllocScratch* s = static_cast<NoAllocScratch*>(base);
    cudaStream_t st = (cudaStream_t)stream;
    const int passes = (int)(key_bits / 8);
    launch_frame_begin(&s->fc, &s->epoch, st);  // zeroes counters, histograms and tile counters
    launch_set_count(&s->fc.visible, (uint32_t)count, st);
    launch_histogram(keys_in, &s->fc.visible, (uint32_t)count, s->fc.hist_depth[0], st);
    const uint32_t* kin = keys_in;
    const uint32_t* vin = values_in;
    for (int p = 0; p < passes; ++p) {
        const bool to_out = ((passes - 1 - p) % 2) == 0;
        uint32_t* kout = to_out ? keys_out : s->tmp_keys;
        uint32_t* vout = to_out ? values_out : s->tmp_vals;
        launch_onesweep(kin, vin, kout, vout, &s->fc.visible, (uint32_t)count, s->fc.hist_depth[p], s->status[p],
                        &s->fc.tile_counter[1 + p], &s->epoch, 8 * p, 1u << 20, &s->fc.err, st);
        kin = kout;
        vin = vout;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return spl_internal_fail(SPL_ERR_CUDA, "launch: %s", cudaGetErrorString(e));
    return SPL_OK;
}

extern "C" int spl_sort_pairs_no_alloc_status(void* stream, uint32_t* device_error) {
    if (device_error) *device_error = 0;
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    NoAllocScratch* s = static_cast<NoAllocScratch*>(base);
    cudaStream_t st = (cudaStream_t)stream;
    // a stack word: the copy to pageable memory completes before cudaMemcpyAsync returns
    uint32_t err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, &s->fc.err, sizeof(err), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return spl_internal_fail(SPL_ERR_CUDA, "reading the sort status: %s", cudaGetErrorString(e));
    if (device_error) *device_error = err;
    if (err & SPL_DEV_ERR_LOOKBACK)
        return spl_internal_fail(SPL_ERR_LOOKBACK_TIMEOUT, "a look-back wait of the last no-allocation sort timed out");
    return SPL_OK;
}
