// mb_sort.cu — onesweep LSD radix sort of cell keys + cell-offset build.
//
// Replaces the external bevy_radix_sort crate (called at src/physics/mod.rs:880-890
// with pass range 0..3, vals = iota) and the spatial-hashing passes
// (src/physics/spatial_hashing.wgsl:29-70).
//
// Sort: one histogram kernel computes the digit counts of every pass in a single
// read of the keys and the exclusive digit bases (last-block-done scan).  Each
// pass is one onesweep kernel: a block takes the next tile (atomic ticket), ranks
// its keys per warp with one ballot per digit bit (stable: warp-striped order,
// warps in order),
// publishes per-digit tile counts into a look-back table, resolves its global
// digit offsets by decoupled look-back over predecessor tiles, stages the tile in
// shared memory in digit order and writes it out in contiguous runs.
//
// Cell offsets: offs[c] = number of keys < c, c in [0, cells].  Sorted slot i
// (and one extra thread for the end) writes offs[c] = i for the cells c in
// (key[i-1], key[i]]: every cell is written once, coalesced where keys are
// dense; a run longer than kGapCells cells is listed and filled by a second
// kernel across many threads.  start[c] / close[c] of the reference are offs[c]
// / offs[c+1]-1 for non-empty cells.

#include <cuda_runtime.h>

#include <algorithm>

#include "mb_internal.h"

namespace mb {
namespace {

constexpr uint32_t kFlagAggregate = 1u;
constexpr uint32_t kFlagPrefix = 2u;
constexpr uint32_t kValueMask = (1u << 28) - 1u;
constexpr uint32_t kSpinLimit = 1u << 21;  // look-back polls before a wait gives up (~0.2 s)
constexpr int kWindow = 8;  // look-back words loaded per step

__device__ __forceinline__ uint32_t lb_pack(uint32_t flag, uint32_t epoch, uint32_t value) {
    return (flag << 30) | ((epoch & 3u) << 28) | (value & kValueMask);
}

__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

struct HistParams {
    int passes;
    uint32_t shift[kMaxPasses];
    uint32_t bits[kMaxPasses];
    uint32_t hist_off[kMaxPasses];   // offset of each pass inside the shared histogram
    uint32_t total_bins;
};

// ---------------------------------------------------------------- histogram
// Digit counts of every pass in one read of the keys (shared-memory atomics; a
// warp whose lanes share a digit adds once, while that keeps happening); the block that finishes last turns
// the counts into exclusive bases and zeroes them for the next sort.
// Returns whether any digit of the key was warp-uniform (full_warp only).
__device__ __forceinline__ bool hist_key(uint32_t* s_hist, const HistParams& hp, uint32_t key, bool full_warp) {
    bool hit = false;
#pragma unroll
    for (int p = 0; p < kMaxPasses; ++p) {  // static indices: the parameters stay in registers
        if (p >= hp.passes) break;
        const uint32_t d = (key >> hp.shift[p]) & ((1u << hp.bits[p]) - 1u);
        if (full_warp) {
            const uint32_t d0 = __shfl_sync(0xFFFFFFFFu, d, 0);
            if (__all_sync(0xFFFFFFFFu, d == d0)) {
                if ((threadIdx.x & 31u) == 0u) atomicAdd(&s_hist[hp.hist_off[p] + d], 32u);
                hit = true;
                continue;
            }
        }
        atomicAdd(&s_hist[hp.hist_off[p] + d], 1u);
    }
    return hit;
}

__global__ void __launch_bounds__(512) k_sort_hist(const uint32_t* __restrict__ keys, uint32_t n,
                                                   HistParams hp, uint32_t* counts,
                                                   uint32_t* bases, uint32_t* ctl) {
    extern __shared__ uint32_t s_hist[];
    __shared__ uint32_t s_last;
    __shared__ uint32_t s_warp[16];
    const uint32_t tid = threadIdx.x, lane = tid & 31u;
    for (uint32_t b = tid; b < hp.total_bins; b += blockDim.x) s_hist[b] = 0;
    if (blockIdx.x == 0 && tid < (uint32_t)kMaxPasses) ctl[kCtlTile0 + tid] = 0;
    if (blockIdx.x == 0 && tid == 0) ctl[kCtlGaps] = 0;  // the cell-offset build of this sort lists anew
    __syncthreads();

    const uint32_t stride = gridDim.x * blockDim.x;
    const bool vec = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0u;
    const uint32_t n4 = vec ? n / 4u : 0u;  // whole uint4 groups, read four keys at a time
    // a warp stops looking for uniform digits once a group of its keys had none
    // (random keys); nearly sorted keys keep hitting and keep the check
    bool check = true;
    for (uint32_t g0 = blockIdx.x * blockDim.x; g0 < n4; g0 += stride) {
        const uint32_t g = g0 + tid;
        const bool full = g0 + blockDim.x <= n4;  // every lane of the block has a group
        if (g < n4) {
            const uint4 k4 = __ldg(reinterpret_cast<const uint4*>(keys) + g);
            const bool c = full && check;
            bool hit = hist_key(s_hist, hp, k4.x, c);
            hit = hist_key(s_hist, hp, k4.y, c) || hit;
            hit = hist_key(s_hist, hp, k4.z, c) || hit;
            hit = hist_key(s_hist, hp, k4.w, c) || hit;
            if (c) check = hit;
        }
    }
    for (uint32_t i = 4u * n4 + blockIdx.x * blockDim.x + tid; i < n; i += stride)
        hist_key(s_hist, hp, __ldg(keys + i), false);
    __syncthreads();
    for (int p = 0; p < hp.passes; ++p) {
        uint32_t R = 1u << hp.bits[p];
        for (uint32_t d = tid; d < R; d += blockDim.x) {
            uint32_t c = s_hist[hp.hist_off[p] + d];
            if (c) atomicAdd(&counts[p * kMaxRadix + d], c);
        }
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = (atomicAdd(&ctl[kCtlDone], 1u) == gridDim.x - 1u) ? 1u : 0u;
    __syncthreads();
    if (!s_last) return;
    __threadfence();

    // exclusive scan of each pass's counts (blockDim.x threads, consecutive bins)
    const uint32_t nt = blockDim.x, warp = tid >> 5, nwarps = nt >> 5;
    for (int p = 0; p < hp.passes; ++p) {
        uint32_t R = 1u << hp.bits[p];
        uint32_t per = (R + nt - 1u) / nt;
        uint32_t beg = min(R, tid * per), end = min(R, beg + per);
        uint32_t sum = 0;
        for (uint32_t d = beg; d < end; ++d) sum += __ldcg(&counts[p * kMaxRadix + d]);
        uint32_t incl = sum;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        if (lane == 31u) s_warp[warp] = incl;
        __syncthreads();
        uint32_t wbase = 0;
        for (uint32_t w = 0; w < warp; ++w) wbase += s_warp[w];
        uint32_t run = wbase + incl - sum;
        for (uint32_t d = beg; d < end; ++d) {
            uint32_t c = __ldcg(&counts[p * kMaxRadix + d]);
            bases[p * (kMaxRadix + 1) + d] = run;
            run += c;
            counts[p * kMaxRadix + d] = 0;
        }
        if (tid == 0) bases[p * (kMaxRadix + 1) + R] = n;
        __syncthreads();
        (void)nwarps;
    }
    if (tid == 0) {
        ctl[kCtlDone] = 0;
        ctl[kCtlEpoch] = ctl[kCtlEpoch] % 3u + 1u;  // new look-back epoch for this sort
    }
}

// ---------------------------------------------------------------- onesweep pass
template <int THREADS, int ITEMS>
__global__ void __launch_bounds__(THREADS, 3)
    k_onesweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
               uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint32_t n,
               uint32_t shift, uint32_t bits, const uint32_t* __restrict__ bases,
               uint32_t* lookback, uint32_t* tile_ticket, uint32_t* err, const uint32_t* epoch_word,
               uint32_t spin_limit) {
    constexpr int WARPS = THREADS / 32;
    constexpr uint32_t TILE = THREADS * ITEMS;
    const uint32_t R = 1u << bits, mask = R - 1u;
    extern __shared__ uint4 smem_raw[];
    uint32_t* s_keys = reinterpret_cast<uint32_t*>(smem_raw);  // [TILE]
    uint32_t* s_vals = s_keys + TILE;                            // [TILE]
    uint32_t* s_cnt = s_vals + TILE;                             // [R] tile count -> local excl
    uint32_t* s_goff = s_cnt + R;                                // [R] global base of the tile
    uint16_t* s_whist = reinterpret_cast<uint16_t*>(s_goff + R); // [WARPS][R]
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_wsum[WARPS];

    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    __shared__ uint32_t s_epoch;
    if (tid == 0) {
        s_tile = atomicAdd(tile_ticket, 1u);
        s_epoch = __ldcg(epoch_word);
    }
    {
        uint32_t* wz = reinterpret_cast<uint32_t*>(s_whist);
        for (uint32_t i = tid; i < (uint32_t)WARPS * R / 2u; i += THREADS) wz[i] = 0u;
        for (uint32_t d = tid; d < R; d += THREADS) s_cnt[d] = 0u;
    }
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t epoch = s_epoch;
    const uint32_t wbase = tile * TILE + warp * 32u * ITEMS;

    uint32_t k[ITEMS], rank[ITEMS];  // values are fetched when the tile is staged
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        uint32_t idx = wbase + (uint32_t)j * 32u + lane;
        bool valid = idx < n;
        k[j] = valid ? __ldg(keys_in + idx) : 0u;
        // the value moves with the key at staging time; start pulling it into L2 now
        if (valid && vals_in) asm volatile("prefetch.global.L2 [%0];" ::"l"(vals_in + idx));
    }
    // the tile's digit counts first, published at once, so that later tiles'
    // look-back finds them while this tile is still ranking its keys
#pragma unroll
    for (int j = 0; j < ITEMS; ++j)
        if (wbase + (uint32_t)j * 32u + lane < n) atomicAdd(&s_cnt[(k[j] >> shift) & mask], 1u);
    __syncthreads();
    uint32_t* lb_tile = lookback + (size_t)tile * R;
    for (uint32_t d = tid; d < R; d += THREADS)
        st_relaxed(lb_tile + d, lb_pack(tile == 0 ? kFlagPrefix : kFlagAggregate, epoch, s_cnt[d]));

    // per-warp stable ranking; the lanes holding the same digit are found with one
    // ballot per digit bit (warp-level multi-split)
    uint16_t* wh = s_whist + warp * R;
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        uint32_t idx = wbase + (uint32_t)j * 32u + lane;
        bool valid = idx < n;
        uint32_t d = valid ? ((k[j] >> shift) & mask) : 0xFFFFFFFFu;
        uint32_t peers = __ballot_sync(0xFFFFFFFFu, valid);
        for (uint32_t bit = 0; bit < bits; ++bit) {
            const bool on = (d >> bit) & 1u;
            const uint32_t bal = __ballot_sync(0xFFFFFFFFu, on);
            peers &= on ? bal : ~bal;
        }
        if (!valid) peers = 1u << lane;
        uint32_t b = valid ? (uint32_t)wh[d] : 0u;
        rank[j] = b + (uint32_t)__popc(peers & lt);
        __syncwarp();
        if (valid && lane == (uint32_t)(__ffs(peers) - 1)) wh[d] = (uint16_t)(b + __popc(peers));
        __syncwarp();
    }
    __syncthreads();

    // per digit: exclusive scan across warps (the tile count is s_cnt already)
    for (uint32_t d = tid; d < R; d += THREADS) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < WARPS; ++w) {
            uint32_t c = s_whist[w * R + d];
            s_whist[w * R + d] = (uint16_t)run;
            run += c;
        }
    }
    __syncthreads();

    // decoupled look-back: exclusive prefix of this digit over all earlier tiles,
    // reading a window of kWindow predecessor words at once (independent loads)
    bool gave_up = false;
    for (uint32_t d = tid; d < R; d += THREADS) {
        uint32_t cnt = s_cnt[d];
        uint32_t excl = 0;
        if (tile > 0) {
            int32_t top = (int32_t)tile - 1;
            uint32_t spins = 0;
            while (top >= 0 && !gave_up) {
                uint32_t e[kWindow];
#pragma unroll
                for (int q = 0; q < kWindow; ++q)
                    e[q] = (top - q >= 0) ? ld_relaxed(lookback + (size_t)(top - q) * R + d)
                                          : lb_pack(kFlagPrefix, epoch, 0u);
                uint32_t sum = 0;
                bool ready = true, found = false;
#pragma unroll
                for (int q = 0; q < kWindow; ++q) {
                    if (!ready || found) continue;
                    uint32_t f = e[q] >> 30;
                    if (f == 0u || ((e[q] >> 28) & 3u) != (epoch & 3u)) {
                        ready = false;
                        continue;
                    }
                    sum += e[q] & kValueMask;
                    if (f == kFlagPrefix) found = true;
                }
                if (!ready) {  // a predecessor has not published yet: retry this window
                    if (++spins > spin_limit) {
                        atomicOr(err, 1u);
                        gave_up = true;
                    } else if (spins > 16u) {
                        __nanosleep(64);
                    }
                    continue;
                }
                excl += sum;
                if (found) break;
                top -= kWindow;
            }
            st_relaxed(lb_tile + d, lb_pack(kFlagPrefix, epoch, excl + cnt));
        }
        s_goff[d] = __ldg(bases + d) + excl;
    }
    __syncthreads();

    // block-wide exclusive scan of the tile counts (consecutive digits per thread)
    {
        uint32_t per = (R + THREADS - 1u) / THREADS;
        uint32_t beg = min(R, tid * per), end = min(R, beg + per);
        uint32_t sum = 0;
        for (uint32_t d = beg; d < end; ++d) sum += s_cnt[d];
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        if (lane == 31u) s_wsum[warp] = incl;
        __syncthreads();
        uint32_t run = incl - sum;
        for (uint32_t w = 0; w < warp; ++w) run += s_wsum[w];
        for (uint32_t d = beg; d < end; ++d) {
            uint32_t c = s_cnt[d];
            s_cnt[d] = run;
            run += c;
        }
    }
    __syncthreads();

    // stage in digit order
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
        uint32_t idx = wbase + (uint32_t)j * 32u + lane;
        if (idx < n) {
            uint32_t d = (k[j] >> shift) & mask;
            uint32_t lpos = s_cnt[d] + (uint32_t)s_whist[warp * R + d] + rank[j];
            s_keys[lpos] = k[j];
            s_vals[lpos] = vals_in ? __ldg(vals_in + idx) : idx;
        }
    }
    __syncthreads();

    // contiguous runs out
    const uint32_t tile_begin = tile * TILE;
    const uint32_t tile_n = (tile_begin < n) ? min(TILE, n - tile_begin) : 0u;
    for (uint32_t i = tid; i < tile_n; i += THREADS) {
        uint32_t key = s_keys[i];
        uint32_t d = (key >> shift) & mask;
        uint32_t pos = s_goff[d] + (i - s_cnt[d]);
        if (pos < n) {  // always true unless a look-back wait gave up (error flagged)
            keys_out[pos] = key;
            vals_out[pos] = s_vals[i];
        }
    }
}

// ---------------------------------------------------------------- cell offsets
// Thread i in [0, n] writes offs[c] = i for c in (key[i-1], key[i]] (key[-1] =
// -1, key[n] = cells; keys clamped to cells).
__global__ void __launch_bounds__(256)
    k_cell_offsets(const uint32_t* __restrict__ sorted_keys, uint32_t n, uint32_t cells, uint32_t* offs,
                   uint32_t* gaps, uint32_t gap_cap, uint32_t* gap_count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    const uint32_t k = i < n ? min(__ldg(sorted_keys + i), cells) : cells;
    const uint32_t from = i > 0u ? min(__ldg(sorted_keys + i - 1u), cells) + 1u : 0u;
    if (from > k) return;  // same cell as the previous key (or a caller's unsorted input)
    if (k - from < kGapCells) {
        for (uint32_t c = from; c <= k; ++c) offs[c] = i;
        return;
    }
    const uint32_t g = atomicAdd(gap_count, 1u);
    if (g < gap_cap) {
        gaps[3u * g] = from;
        gaps[3u * g + 1u] = k;
        gaps[3u * g + 2u] = i;
    }
}

// Each block fills listed runs (run e = blockIdx.x, + gridDim.x, ...).
__global__ void __launch_bounds__(256)
    k_fill_gaps(const uint32_t* __restrict__ gaps, uint32_t gap_cap, const uint32_t* __restrict__ gap_count,
                uint32_t* offs) {
    const uint32_t m = min(*gap_count, gap_cap);
    for (uint32_t e = blockIdx.x; e < m; e += gridDim.x) {
        const uint32_t from = gaps[3u * e], to = gaps[3u * e + 1u], v = gaps[3u * e + 2u];
        for (uint32_t c = from + threadIdx.x; c <= to; c += blockDim.x) offs[c] = v;
    }
}

__global__ void k_offs_to_start_close(const uint32_t* __restrict__ offs, uint32_t cells,
                                      uint32_t* start, uint32_t* close) {
    uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    uint32_t a = offs[c], b = offs[c + 1u];
    bool full = b > a;
    if (start) start[c] = full ? a : kInvalid;
    if (close) close[c] = full ? b - 1u : kInvalid;
}

// HASHING (spatial_hashing.wgsl:46-70) straight from the sorted keys, every cell
// written once: thread i (i in [0, n], i = n a sentinel with key = cells) that
// starts a run of key k writes start[k] = i, closes the previous run
// (close[key[i-1]] = i - 1) and marks the empty cells between the two keys
// (0xFFFFFFFF in both tables; runs of more than kGapCells empty cells are
// listed for k_fill_empty).  Keys >= cells belong to no cell.
__global__ void __launch_bounds__(256)
    k_hash_ranges(const uint32_t* __restrict__ sorted_keys, uint32_t n, uint32_t cells, uint32_t* start,
                  uint32_t* close, uint32_t* gaps, uint32_t gap_cap, uint32_t* gap_count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    const uint32_t k = i < n ? min(__ldg(sorted_keys + i), cells) : cells;
    const uint32_t p = i > 0u ? min(__ldg(sorted_keys + i - 1u), cells) : 0xFFFFFFFFu;
    const uint32_t from = p + 1u;  // first cell after the previous key (0 for i = 0)
    if (i > 0u && p == k) return;  // inside a run
    if (i > 0u && p < cells && close) close[p] = i - 1u;
    if (k < cells && start) start[k] = i;
    if (from >= k) return;  // no empty cells in between
    if (k - from <= kGapCells) {
        for (uint32_t c = from; c < k; ++c) {
            if (start) start[c] = kInvalid;
            if (close) close[c] = kInvalid;
        }
        return;
    }
    const uint32_t g = atomicAdd(gap_count, 1u);
    if (g < gap_cap) {
        gaps[3u * g] = from;
        gaps[3u * g + 1u] = k - 1u;
        gaps[3u * g + 2u] = kInvalid;
    }
}

// The listed runs of empty cells (run e = blockIdx.x, + gridDim.x, ...).
__global__ void __launch_bounds__(256)
    k_fill_empty(const uint32_t* __restrict__ gaps, uint32_t gap_cap, const uint32_t* __restrict__ gap_count,
                 uint32_t* start, uint32_t* close) {
    const uint32_t m = min(*gap_count, gap_cap);
    for (uint32_t e = blockIdx.x; e < m; e += gridDim.x) {
        const uint32_t from = gaps[3u * e], to = gaps[3u * e + 1u];
        for (uint32_t c = from + threadIdx.x; c <= to; c += blockDim.x) {
            if (start) start[c] = kInvalid;
            if (close) close[c] = kInvalid;
        }
    }
}

__global__ void __launch_bounds__(256)
    k_gather_state(const uint32_t* __restrict__ perm, uint32_t n, const float4* __restrict__ pos_in,
                   const uint4* __restrict__ vfme_in, float4* __restrict__ spos, uint4* __restrict__ svfme,
                   const uint32_t* __restrict__ sorted_keys, const uint32_t* __restrict__ offs,
                   uint4* __restrict__ bands, uint32_t N) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (spos) {  // the sorted state copy (none when the physics pass reads through perm)
        const uint32_t o = min(__ldg(perm + i), n - 1u);
        spos[i] = __ldg(pos_in + o);
        svfme[i] = __ldg(vfme_in + o);
    }
    if (bands) write_band_bounds(bands, offs, N, n, i, __ldg(sorted_keys + i));
}

size_t onesweep_smem(uint32_t R) {
    return sizeof(uint32_t) * (2u * kSortTile + 2u * R) + sizeof(uint16_t) * (kSortThreads / 32) * R;
}

}  // namespace

int device_sm_count() {
    constexpr int kDevices = 64;
    static int sms[kDevices] = {};  // 0: not looked up yet (benign race: every thread stores the same value)
    int dev = 0;
    cudaGetDevice(&dev);
    int got = (dev >= 0 && dev < kDevices) ? __atomic_load_n(&sms[dev], __ATOMIC_RELAXED) : 0;
    if (got > 0) return got;
    if (cudaDeviceGetAttribute(&got, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || got <= 0) got = 1;
    if (dev >= 0 && dev < kDevices) __atomic_store_n(&sms[dev], got, __ATOMIC_RELAXED);
    return got;
}

SortSchedule make_schedule(uint32_t n, uint32_t cells, uint32_t digit_bits_max) {
    SortSchedule s;
    s.n = n;
    s.cells = cells;
    uint32_t dmax = std::min<uint32_t>(std::max<uint32_t>(digit_bits_max, 4u), kMaxDigitBits);
    uint32_t bits = 1;
    while (bits < 32u && (1ull << bits) < (uint64_t)cells) ++bits;
    s.total_bits = bits;
    uint32_t last = std::min(bits, dmax);
    uint32_t rest = bits - last;
    int prest = (int)((rest + dmax - 1u) / dmax);
    s.passes = prest + 1;
    uint32_t shift = 0;
    for (int p = 0; p < prest; ++p) {
        uint32_t b = rest / (uint32_t)prest + ((uint32_t)p < rest % (uint32_t)prest ? 1u : 0u);
        s.shift[p] = shift;
        s.bits[p] = b;
        shift += b;
    }
    s.shift[prest] = shift;
    s.bits[prest] = last;
    s.tiles = (n + kSortTile - 1u) / kSortTile;
    return s;
}

cudaError_t scratch_alloc(SortScratch& s, uint32_t max_keys, uint32_t max_cells) {
    s.max_keys = max_keys;
    s.max_cells = max_cells;
    size_t tiles = (max_keys + kSortTile - 1u) / kSortTile;
    if (tiles == 0) tiles = 1;
    s.lookback_words_per_pass = tiles * kMaxRadix;
    cudaError_t e;
    if ((e = cudaMalloc(&s.alt_keys, sizeof(uint32_t) * std::max<uint32_t>(max_keys, 1u)))) return e;
    if ((e = cudaMalloc(&s.alt_vals, sizeof(uint32_t) * std::max<uint32_t>(max_keys, 1u)))) return e;
    if ((e = cudaMalloc(&s.counts, sizeof(uint32_t) * kMaxPasses * kMaxRadix))) return e;
    if ((e = cudaMalloc(&s.bases, sizeof(uint32_t) * kMaxPasses * (kMaxRadix + 1)))) return e;
    if ((e = cudaMalloc(&s.lookback, sizeof(uint32_t) * kMaxPasses * s.lookback_words_per_pass))) return e;
    if ((e = cudaMalloc(&s.ctl, sizeof(uint32_t) * kCtlWords))) return e;
    if ((e = cudaMalloc(&s.offs, sizeof(uint32_t) * ((size_t)max_cells + 1u)))) return e;
    if ((e = cudaMalloc(&s.gaps, sizeof(uint32_t) * 3u * gap_capacity(max_cells)))) return e;
    if ((e = cudaMemset(s.counts, 0, sizeof(uint32_t) * kMaxPasses * kMaxRadix))) return e;
    if ((e = cudaMemset(s.lookback, 0, sizeof(uint32_t) * kMaxPasses * s.lookback_words_per_pass))) return e;
    if ((e = cudaMemset(s.ctl, 0, sizeof(uint32_t) * kCtlWords))) return e;
    if ((e = cudaFuncSetAttribute(k_onesweep<kSortThreads, kSortItems>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)onesweep_smem(kMaxRadix))))
        return e;
    s.last_tiles = 0;
    s.last_passes = 0;
    return cudaSuccess;
}

namespace {
// Look-back words are tagged with the epoch of the sort that wrote them (1..3,
// advanced by every sort's histogram kernel) and reused without clearing when
// the previous sort had the same layout (tiles, passes and digit widths): it
// then overwrote every word this sort reads with the previous epoch, so a word
// not yet published by this sort never carries the current epoch.  Any other
// layout could leave a word of the sort three epochs back in place, so the
// table is cleared (and the epoch restarted) instead.
bool same_layout(const SortScratch& s, const SortSchedule& sch) {
    if (sch.tiles != s.last_tiles || sch.passes != s.last_passes) return false;
    for (int p = 0; p < sch.passes; ++p)
        if (sch.bits[p] != s.last_bits[p]) return false;
    return true;
}
void remember_layout(SortScratch& s, const SortSchedule& sch) {
    s.last_tiles = sch.tiles;
    s.last_passes = sch.passes;
    for (int p = 0; p < kMaxPasses; ++p) s.last_bits[p] = p < sch.passes ? sch.bits[p] : 0u;
}
void forget_layout(SortScratch& s) {
    s.last_tiles = 0;
    s.last_passes = 0;
}
}  // namespace

void scratch_free(SortScratch& s) {
    cudaFree(s.alt_keys);
    cudaFree(s.alt_vals);
    cudaFree(s.counts);
    cudaFree(s.bases);
    cudaFree(s.lookback);
    cudaFree(s.ctl);
    cudaFree(s.offs);
    cudaFree(s.gaps);
    s = SortScratch();
}

cudaError_t sort_pairs(SortScratch& s, const SortSchedule& sch, const uint32_t* keys,
                       const uint32_t* vals, uint32_t* sorted_keys, uint32_t* sorted_vals,
                       cudaStream_t st, bool clear_always) {
    const uint32_t n = sch.n;
    if (n == 0) return cudaSuccess;
    if (clear_always) {
        // every word this sort reads starts unpublished, whatever ran before
        for (int p = 0; p < sch.passes; ++p) {
            cudaError_t e = cudaMemsetAsync(s.lookback + (size_t)p * s.lookback_words_per_pass, 0,
                                            sizeof(uint32_t) * (size_t)sch.tiles * (1u << sch.bits[p]), st);
            if (e) return e;
        }
        forget_layout(s);
    } else if (!same_layout(s, sch)) {
        cudaError_t e = cudaMemsetAsync(s.lookback, 0,
                                        sizeof(uint32_t) * kMaxPasses * s.lookback_words_per_pass, st);
        if (e) return e;
        if ((e = cudaMemsetAsync(s.ctl + kCtlEpoch, 0, sizeof(uint32_t), st))) return e;
        remember_layout(s, sch);
    }

    HistParams hp;
    hp.passes = sch.passes;
    hp.total_bins = 0;
    for (int p = 0; p < kMaxPasses; ++p) {
        hp.shift[p] = sch.shift[p];
        hp.bits[p] = sch.bits[p];
        hp.hist_off[p] = hp.total_bins;
        if (p < sch.passes) hp.total_bins += 1u << sch.bits[p];
    }
    int sms = device_sm_count();
    uint32_t hist_blocks = std::max<uint32_t>(1u, std::min<uint32_t>((n + 2047u) / 2048u, (uint32_t)sms * 4u));
    k_sort_hist<<<hist_blocks, 512, sizeof(uint32_t) * hp.total_bins, st>>>(keys, n, hp, s.counts,
                                                                             s.bases, s.ctl);
    cudaError_t e = cudaGetLastError();
    if (e) return e;

    // ping-pong so that the last pass lands in the outputs
    const uint32_t* kin = keys;
    const uint32_t* vin = vals;
    for (int p = 0; p < sch.passes; ++p) {
        bool to_out = ((sch.passes - 1 - p) % 2) == 0;
        uint32_t* kout = to_out ? sorted_keys : s.alt_keys;
        uint32_t* vout = to_out ? sorted_vals : s.alt_vals;
        uint32_t R = 1u << sch.bits[p];
        k_onesweep<kSortThreads, kSortItems><<<sch.tiles, kSortThreads, onesweep_smem(R), st>>>(
            kin, vin, kout, vout, n, sch.shift[p], sch.bits[p], s.bases + p * (kMaxRadix + 1),
            s.lookback + (size_t)p * s.lookback_words_per_pass, s.ctl + kCtlTile0 + p,
            s.ctl + kCtlError, s.ctl + kCtlEpoch, kSpinLimit);
        if ((e = cudaGetLastError())) return e;
        kin = kout;
        vin = vout;
    }
    return cudaSuccess;
}

cudaError_t sort_take_error(SortScratch& s, cudaStream_t st, uint32_t* flags) {
    uint32_t f = 0;
    cudaError_t e = cudaStreamSynchronize(st);
    if (!e) e = cudaMemcpy(&f, s.ctl + kCtlError, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (!e && f) {
        e = cudaMemset(s.ctl + kCtlError, 0, sizeof(uint32_t));
        forget_layout(s);  // the look-back words of the failed sort may be half written
    }
    if (flags) *flags = e ? 0u : f;
    return e;
}

cudaError_t sort_stall_for_test(SortScratch& s, uint32_t spin_limit, cudaStream_t st) {
    // pass 0's words unpublished (tile 0 never runs), ticket 1 for the one block:
    // it is tile 1 of a one-key sort, so it reads and writes no keys, and its
    // look-back on tile 0 polls until spin_limit runs out
    constexpr uint32_t kBits = 8, R = 1u << kBits;
    if (2u * R > s.lookback_words_per_pass) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(s.lookback, 0, sizeof(uint32_t) * 2u * R, st);
    if (e) return e;
    const uint32_t one = 1u;
    if ((e = cudaMemcpyAsync(s.ctl + kCtlTile0, &one, sizeof(uint32_t), cudaMemcpyHostToDevice, st))) return e;
    k_onesweep<kSortThreads, kSortItems><<<1, kSortThreads, onesweep_smem(R), st>>>(
        s.alt_keys, nullptr, s.alt_vals, s.alt_vals, 1u, 0u, kBits, s.bases, s.lookback, s.ctl + kCtlTile0,
        s.ctl + kCtlError, s.ctl + kCtlEpoch, spin_limit);
    if ((e = cudaGetLastError())) return e;
    forget_layout(s);
    return cudaStreamSynchronize(st);  // `one` lives on this stack frame
}

cudaError_t cell_offsets(SortScratch& s, const SortSchedule& sch, const uint32_t* sorted_keys,
                         cudaStream_t st) {
    if (sch.n == 0)  // every cell offset is 0
        return cudaMemsetAsync(s.offs, 0, sizeof(uint32_t) * ((size_t)sch.cells + 1u), st);
    const uint32_t cap = gap_capacity(s.max_cells);
    k_cell_offsets<<<(sch.n + 256u) / 256u, 256, 0, st>>>(sorted_keys, sch.n, sch.cells, s.offs, s.gaps, cap,
                                                          s.ctl + kCtlGaps);
    cudaError_t e = cudaGetLastError();
    if (e) return e;
    k_fill_gaps<<<(uint32_t)device_sm_count() * 4u, 256, 0, st>>>(s.gaps, cap, s.ctl + kCtlGaps, s.offs);
    return cudaGetLastError();
}

cudaError_t gather_state(const uint32_t* perm, uint32_t n, const float4* pos_in, const uint4* vfme_in,
                         float4* spos, uint4* svfme, const uint32_t* sorted_keys, const uint32_t* offs,
                         uint4* bands, uint32_t N, cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_gather_state<<<(n + 255u) / 256u, 256, 0, st>>>(perm, n, pos_in, vfme_in, spos, svfme, sorted_keys, offs,
                                                      bands, N);
    return cudaGetLastError();
}

cudaError_t hash_ranges(SortScratch& s, const uint32_t* sorted_keys, uint32_t n, uint32_t cells, uint32_t* start,
                        uint32_t* close, cudaStream_t st) {
    if (!start && !close) return cudaSuccess;
    cudaError_t e;
    // the gap counter is cleared by the sort's histogram kernel; an empty sort has none
    if (n == 0 && (e = cudaMemsetAsync(s.ctl + kCtlGaps, 0, sizeof(uint32_t), st))) return e;
    const uint32_t cap = gap_capacity(s.max_cells);
    k_hash_ranges<<<(n + 256u) / 256u, 256, 0, st>>>(sorted_keys, n, cells, start, close, s.gaps, cap,
                                                     s.ctl + kCtlGaps);
    if ((e = cudaGetLastError())) return e;
    k_fill_empty<<<(uint32_t)device_sm_count() * 4u, 256, 0, st>>>(s.gaps, cap, s.ctl + kCtlGaps, start, close);
    return cudaGetLastError();
}

cudaError_t offsets_to_start_close(const uint32_t* offs, uint32_t cells, uint32_t* start,
                                   uint32_t* close, cudaStream_t st) {
    if (cells == 0) return cudaSuccess;
    k_offs_to_start_close<<<(cells + 255u) / 256u, 256, 0, st>>>(offs, cells, start, close);
    return cudaGetLastError();
}

}  // namespace mb
