// mb_static.cu — mb_sort_and_hash_static: the sort + cell-range stage without
// any device allocation.
//
// Who needs it: code that records GPU work where it may not allocate - a frame
// loop of a game engine or render graph that forbids allocations after start-up
// (allocator stalls cause frame-time spikes and break fixed memory budgets), or
// a caller that records into a CUDA stream capture, where cudaMalloc is not a
// stream operation and cannot be recorded.  mb_sort_and_hash needs a plan
// created with cudaMalloc first; this entry point instead uses one fixed block
// of scratch memory that lives in the library image itself.
//
// The scratch is the file-scope array below.  Its address is only valid in
// device code; host code obtains the device address with cudaGetSymbolAddress,
// once per device, with that device current.  The first call on a device does
// that set-up (and zeroes the array with cudaMemsetAsync on the caller's
// stream), so that first call should come before any stream capture.
//
// Every call on a device shares the one array, and the array keeps what the
// last call left in it.  Calls whose work overlaps on the GPU (different
// streams, or host threads racing) corrupt each other's results; callers must
// order them, e.g. by issuing them all on one stream.  Each call clears, on its
// stream, the part of the array whose stale contents could be misread (the sort's
// look-back words), so recorded calls replayed in any order stay correct.
// mb_sort_static_status reads (and clears) the array's error word: a bounded
// device-side wait that gave up.

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "mb_internal.h"

namespace {

constexpr uint32_t kStaticMaxKeys = MB_STATIC_MAX_KEYS;
constexpr uint32_t kStaticMaxCells = MB_STATIC_MAX_CELLS;
constexpr uint32_t kStaticDigitBits = 8;  // R = 256: small look-back table
constexpr uint32_t kStaticTiles = (kStaticMaxKeys + mb::kSortTile - 1u) / mb::kSortTile;
constexpr size_t kLookbackPerPass = (size_t)kStaticTiles * (1u << kStaticDigitBits);

constexpr size_t align4(size_t w) { return (w + 3u) & ~(size_t)3u; }  // 16-byte steps of u32 words
constexpr size_t kOffAltKeys = 0;
constexpr size_t kOffAltVals = kOffAltKeys + align4(kStaticMaxKeys);
constexpr size_t kOffCounts = kOffAltVals + align4(kStaticMaxKeys);
constexpr size_t kOffBases = kOffCounts + align4((size_t)mb::kMaxPasses * mb::kMaxRadix);
constexpr size_t kOffLookback = kOffBases + align4((size_t)mb::kMaxPasses * (mb::kMaxRadix + 1u));
constexpr size_t kOffCtl = kOffLookback + align4((size_t)mb::kMaxPasses * kLookbackPerPass);
constexpr size_t kOffOffs = kOffCtl + align4(mb::kCtlWords);
constexpr size_t kOffGaps = kOffOffs + align4((size_t)kStaticMaxCells + 1u);
constexpr size_t kScratchWords = kOffGaps + align4((size_t)3u * ((size_t)kStaticMaxCells / mb::kGapCells + 2u));

// The shared scratch: about 3.5 MB, resident on every GPU that loads the library.
static __device__ __align__(256) uint32_t g_static_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct DeviceSlot {
    bool ready = false;
    mb::SortScratch view;  // pointers into g_static_scratch on that device
};
DeviceSlot g_dev[kMaxDevices];
mb_status fail(mb_status st, const std::string& m) {
    mb::set_process_error(m);  // readable with mb_last_error(NULL)
    return st;
}

}  // namespace

extern "C" mb_status mb_sort_and_hash_static(const uint32_t* keys, const uint32_t* vals, uint32_t n,
                                             uint32_t number_of_cells, uint32_t* sorted_keys,
                                             uint32_t* sorted_vals, uint32_t* start, uint32_t* close,
                                             void* cuda_stream) {
    if (n > kStaticMaxKeys)
        return fail(MB_ERR_INVALID_ARG, "mb_sort_and_hash_static: n exceeds MB_STATIC_MAX_KEYS (262144)");
    if (number_of_cells == 0 || number_of_cells > kStaticMaxCells)
        return fail(MB_ERR_INVALID_ARG,
                    "mb_sort_and_hash_static: number_of_cells must be in [1, MB_STATIC_MAX_CELLS (262144)]");
    if (n && (!keys || !sorted_keys || !sorted_vals))
        return fail(MB_ERR_INVALID_ARG, "mb_sort_and_hash_static: NULL key/value buffer");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return fail(MB_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(MB_ERR_INVALID_ARG, "mb_sort_and_hash_static: device id too large");
    cudaStream_t st = (cudaStream_t)cuda_stream;

    std::lock_guard<std::mutex> lock(g_mu);
    DeviceSlot& slot = g_dev[dev];
    if (!slot.ready) {  // once per device, with that device current
        uint32_t* base = nullptr;
        e = cudaGetSymbolAddress((void**)&base, g_static_scratch);
        if (e) return fail(MB_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        e = cudaMemsetAsync(base, 0, sizeof(uint32_t) * kScratchWords, st);
        if (e) return fail(MB_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
        mb::SortScratch& v = slot.view;
        v.max_keys = kStaticMaxKeys;
        v.max_cells = kStaticMaxCells;
        v.alt_keys = base + kOffAltKeys;
        v.alt_vals = base + kOffAltVals;
        v.counts = base + kOffCounts;
        v.bases = base + kOffBases;
        v.lookback = base + kOffLookback;
        v.ctl = base + kOffCtl;
        v.offs = base + kOffOffs;
        v.gaps = base + kOffGaps;
        v.lookback_words_per_pass = kLookbackPerPass;
        v.last_tiles = 0;
        v.last_passes = 0;
        slot.ready = true;
    }
    mb::SortSchedule sch = mb::make_schedule(n, number_of_cells, kStaticDigitBits);
    e = mb::sort_pairs(slot.view, sch, keys, vals, sorted_keys, sorted_vals, st, /*clear_always=*/true);
    if (!e && (start || close)) e = mb::hash_ranges(slot.view, sorted_keys, n, number_of_cells, start, close, st);
    if (e) return fail(e == cudaErrorMemoryAllocation ? MB_ERR_OOM : MB_ERR_CUDA,
                       std::string("mb_sort_and_hash_static: ") + cudaGetErrorString(e));
    return MB_OK;
}

extern "C" mb_status mb_sort_static_status(void* cuda_stream) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return fail(MB_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(MB_ERR_INVALID_ARG, "mb_sort_static_status: device id too large");
    std::lock_guard<std::mutex> lock(g_mu);
    DeviceSlot& slot = g_dev[dev];
    if (!slot.ready) return MB_OK;  // nothing ran on this device
    uint32_t flags = 0;
    e = mb::sort_take_error(slot.view, (cudaStream_t)cuda_stream, &flags);
    if (e) return fail(MB_ERR_CUDA, std::string("mb_sort_static_status: ") + cudaGetErrorString(e));
    if (flags)
        return fail(MB_ERR_TIMEOUT,
                    "mb_sort_static_status: a bounded look-back wait gave up; results of the calls since the "
                    "last status check are invalid");
    return MB_OK;
}
