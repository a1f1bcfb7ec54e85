// mb_count.cu — counting sort of cell keys (the default frame sort).
//
// The reference sorts the cell keys with a generic 3 x 8-bit radix sort
// (bevy_radix_sort, called at src/physics/mod.rs:880-890) and then derives each
// cell's slot range from the sorted keys (spatial_hashing.wgsl:29-70).  Here the
// key space *is* the cell table, so the same stable permutation comes from:
//
//   1. per-cell counts, accumulated by the physics pass of the previous frame as
//      it emits the keys (one red.add per sphere);
//   2. k_cell_scan: one exclusive scan turns the counts into the cell offsets
//      offs[c] (= start of cell c; offs[C] = n); each
//      chunk of cells takes its base from per-4096-cell-tile counts emitted with
//      the per-cell ones (plus the counts of its tile's earlier chunks), so
//      chunks never wait on each other;
//   3. k_cell_scatter: each sphere claims a slot of its cell with one atomic per
//      run of equal keys in its warp (match.any) - it subtracts the run's length
//      from the cell's count, and the count left before it says where the run
//      starts (offs[c+1] - left), so the counts are back to zero when the
//      scatter ends - spheres of one warp keep their order, and its 32-byte
//      state is copied to that slot; the run that
//      fills a cell last marks the cell (a bit per input slot) if earlier runs
//      of other warps got there first (only such cells can be out of order);
//   4. k_fix_collect: the marked cells are listed by size;
//   5. k_cell_fix: the listed cells' slots are put back in ascending input order
//      (what a stable sort yields), re-gathering their state copy.
//
// The result is bit-identical to a stable sort; offs[] replaces start/close.

#include <cuda_runtime.h>

#include <algorithm>

#include "mb_internal.h"

namespace mb {
namespace {

// ---------------------------------------------------------------- scan
// Block b of the scan covers the chunk of cells [kScanChunk b, kScanChunk (b + 1))
// inside tile t = b kScanChunk / 4096 (cells [4096 t, 4096 t + 4096)).  coarse[t] holds the number of
// spheres in tile t (emitted with the per-cell counts), so a chunk finds its base
// by summing coarse[0..t) and the counts of the tile's cells before it - no
// look-back, no waiting on other blocks.  The counts are left in place (other
// chunks read them); the fixup kernel clears them.
//
// kScenes (a batch): every scene's cell range is padded to whole tiles, so a tile
// belongs to one scene; its base is that scene's first slot plus the coarse
// counts of the scene's earlier tiles, and tiles of HOLD scenes are left alone.
template <bool kScenes>
__global__ void __launch_bounds__(kScanThreads)
    k_cell_scan(const uint32_t* __restrict__ hist, const uint32_t* __restrict__ coarse, uint32_t cells,
                uint32_t* __restrict__ offs, uint32_t* fix_ctl,
                const SceneDev* __restrict__ scenes, const uint32_t* __restrict__ cell_tile_scene) {
    constexpr int W = kScanThreads / 32;
    __shared__ uint32_t s_warp[W], s_base[W];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t chunk = blockIdx.x, c0 = chunk * kScanChunk, tile = c0 / kScanTile;
    griddep_wait();  // after the previous frame's physics pass, when chained to it
    griddep_launch();
    if (chunk == 0 && tid < (uint32_t)kFixLists) fix_ctl[tid] = 0u;  // fixup lists of this frame start empty
    const uint32_t base = c0 + tid * kScanItems;

    uint32_t first_tile = 0, base_slot = 0;
    if (kScenes) {
        const uint32_t sc = __ldg(cell_tile_scene + tile);
        if (__ldg(&scenes[sc].mode) == kModeHold) return;
        first_tile = __ldg(&scenes[sc].cell_base) / kScanTile;
        base_slot = __ldg(&scenes[sc].agent_base);
    }
    // exclusive base of this chunk: the coarse counts of the earlier tiles, plus
    // the counts of the tile's cells before the chunk
    uint32_t bsum = 0;
    for (uint32_t t = first_tile + tid; t < tile; t += kScanThreads) bsum += __ldg(coarse + t);
    for (uint32_t c = tile * kScanTile + tid * 4u; c < c0; c += kScanThreads * 4u) {
        const uint4 x = __ldcg(reinterpret_cast<const uint4*>(hist + c));
        bsum += (x.x + x.y) + (x.z + x.w);
    }

    uint32_t v[kScanItems];
    if (base + kScanItems <= cells) {
        const uint4* h4 = reinterpret_cast<const uint4*>(hist + base);
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            uint4 x = __ldcg(h4 + q);
            v[4 * q] = x.x;
            v[4 * q + 1] = x.y;
            v[4 * q + 2] = x.z;
            v[4 * q + 3] = x.w;
        }
    } else {
#pragma unroll
        for (int q = 0; q < kScanItems; ++q) v[q] = (base + q < cells) ? __ldcg(hist + base + q) : 0u;
    }
    uint32_t sum = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) sum += v[q];
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) bsum += __shfl_xor_sync(0xFFFFFFFFu, bsum, o);
    if (lane == 31u) s_warp[warp] = incl;
    if (lane == 0u) s_base[warp] = bsum;
    __syncthreads();
    uint32_t run = base_slot + incl - sum;
#pragma unroll
    for (int w = 0; w < W; ++w) {
        if ((uint32_t)w < warp) run += s_warp[w];
        run += s_base[w];
    }
    if (base + kScanItems <= cells) {
        uint4* o4 = reinterpret_cast<uint4*>(offs + base);
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            uint4 x;
            x.x = run; run += v[4 * q];
            x.y = run; run += v[4 * q + 1];
            x.z = run; run += v[4 * q + 2];
            x.w = run; run += v[4 * q + 3];
            o4[q] = x;
        }
        // end of the tile: the next tile's first offset, or the scene's / table's end
        if (base + kScanItems == cells || (kScenes && tid == kScanThreads - 1)) offs[base + kScanItems] = run;
    } else {
        for (int q = 0; q < kScanItems; ++q) {
            uint32_t c = base + q;
            if (c < cells) {
                offs[c] = run;
                run += v[q];
                if (c + 1u == cells) offs[cells] = run;
            }
        }
    }
}

// ---------------------------------------------------------------- scatter
// Fixup lists, filled with one global atomic per list per block iteration.
struct FixLists {
    uint32_t* ctl;
    uint32_t* list[kFixLists];
    uint32_t cap[kFixLists];
};

// The run [b, b + g) of a cell with slots [lo, hi) ends the cell and did not
// start it: other warps' runs came first, so the cell may be out of input order.
// The run's leader marks its input slot in the fixup bitmap (once per cell: one
// run ends it); k_fix_collect lists the marked cells.
__device__ __forceinline__ bool listed(uint32_t lo, uint32_t hi, uint32_t b, uint32_t g) {
    return b + g == hi && b != lo;
}
// One word of the bitmap per 32 input slots, written whole by the warp that
// scatters them (every word below ceil(n / 32) is rewritten each frame, so
// nothing is cleared and the scatter needs no atomics or barriers for it).
__device__ __forceinline__ void mark_fix(uint32_t* __restrict__ fix_bits, uint32_t i, uint32_t n, bool mark) {
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, mark);
    if ((threadIdx.x & 31u) == 0u && i < n) fix_bits[i >> 5] = m;
}
// Also (spos != NULL) moves each sphere's state to its slot (a sorted copy for
// the physics pass; without it the physics pass reads the state through perm)
// and, where a slot begins or ends a physics tile, writes that side of the
// tile's band table entry (the cell of a slot is final here; the fixup only
// reorders slots inside a cell).
__global__ void __launch_bounds__(256)
    k_cell_scatter(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ hist,
                   uint32_t* __restrict__ perm, const float4* __restrict__ pos_in,
                   const uint4* __restrict__ vfme_in, float4* __restrict__ spos,
                   uint4* __restrict__ svfme, const uint32_t* __restrict__ offs, uint4* __restrict__ bands,
                   uint32_t N, uint32_t* __restrict__ fix_bits) {
    griddep_wait();
    griddep_launch();
    const uint32_t lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        uint32_t i = i0 + threadIdx.x;
        bool valid = i < n;
        uint32_t k = valid ? __ldg(keys + i) : 0xFFFFFFFFu;
        float4 p;
        uint4 q;
        if (valid && spos) {
            p = __ldg(pos_in + i);
            q = __ldg(vfme_in + i);
        }
        // a key flagged kInitKeyBit belongs to a scene in its INIT frame: all its
        // keys are equal, so its stable order is the identity and the slot is i
        const bool ident = valid && (k & kInitKeyBit);
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, ident ? 0xFFFFFFFEu : k);
        uint32_t leader = (uint32_t)(__ffs(peers) - 1);
        uint32_t b = 0;
        bool mark = false;
        if (valid && !ident && lane == leader) {
            const uint32_t g = (uint32_t)__popc(peers);
            const uint32_t lo = __ldg(offs + k), hi = __ldg(offs + k + 1u);
            b = hi - atomicSub(hist + k, g);  // the run's first slot
            mark = listed(lo, hi, b, g);
        }
        b = __shfl_sync(0xFFFFFFFFu, b, (int)leader);
        mark_fix(fix_bits, i, n, mark);
        if (valid) {
            const uint32_t dst = ident ? i : b + (uint32_t)__popc(peers & lt);
            if (dst >= n) continue;  // only counts that disagree with the keys get here
            perm[dst] = i;
            if (spos) {
                spos[dst] = p;
                svfme[dst] = q;
            }
            if (bands && !ident) write_band_bounds(bands, offs, N, n, dst, k);
        }
    }
}

// The same for a batch: slot i's scene (from the tile table) gives the buffer
// holding its state; spheres of HOLD scenes are left alone.
__global__ void __launch_bounds__(256)
    k_cell_scatter_scenes(const SceneDev* __restrict__ scenes, const uint32_t* __restrict__ tile_scene,
                          const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ hist,
                          uint32_t* __restrict__ perm, const float4* __restrict__ pos0,
                          const float4* __restrict__ pos1, const uint4* __restrict__ vfme0,
                          const uint4* __restrict__ vfme1, float4* __restrict__ spos, uint4* __restrict__ svfme,
                          const uint32_t* __restrict__ offs, uint32_t* __restrict__ fix_bits,
                          uint4* __restrict__ bands) {
    const uint32_t lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        uint32_t i = i0 + threadIdx.x;
        bool valid = i < n;
        uint32_t mode = kModeHold, parity = 0, sc = 0;
        if (valid) {
            uint32_t s = __ldg(tile_scene + i / kPhysicsTile);
            while (i >= __ldg(&scenes[s].agent_end)) ++s;
            mode = __ldg(&scenes[s].mode);
            parity = __ldg(&scenes[s].parity);
            sc = s;
        }
        valid = valid && mode != kModeHold;
        uint32_t k = valid ? __ldg(keys + i) : 0xFFFFFFFFu;
        float4 p;
        uint4 q;
        if (valid) {
            p = __ldg((parity ? pos1 : pos0) + i);
            q = __ldg((parity ? vfme1 : vfme0) + i);
        }
        const bool ident = valid && (k & kInitKeyBit);
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, ident ? 0xFFFFFFFEu : k);
        uint32_t leader = (uint32_t)(__ffs(peers) - 1);
        uint32_t b = 0;
        bool mark = false;
        if (valid && !ident && lane == leader) {
            const uint32_t g = (uint32_t)__popc(peers);
            const uint32_t lo = __ldg(offs + k), hi = __ldg(offs + k + 1u);
            b = hi - atomicSub(hist + k, g);  // the run's first slot
            mark = listed(lo, hi, b, g);
        }
        b = __shfl_sync(0xFFFFFFFFu, b, (int)leader);
        mark_fix(fix_bits, i, n, mark);
        if (valid) {
            const uint32_t dst = ident ? i : b + (uint32_t)__popc(peers & lt);
            if (dst >= n) continue;  // only counts that disagree with the keys get here
            perm[dst] = i;
            spos[dst] = p;
            svfme[dst] = q;
            if (bands && !ident) {  // the scene's band table entries, in its own cell coordinates
                const uint32_t cb = __ldg(&scenes[sc].cell_base);
                write_band_bounds(bands, offs + cb, __ldg(&scenes[sc].P.N), n, dst, k - cb);
            }
        }
    }
}

// ---------------------------------------------------------------- collect
// Lists the cells marked in the fixup bitmap by size class (a marked input
// slot's key is its cell).  A block reads kCollectWords words, a byte per
// thread, stages the cells in shared memory and appends them to the global
// lists with one atomic per list.
constexpr uint32_t kCollectThreads = 256, kCollectWords = kCollectThreads / 4u;

__global__ void __launch_bounds__(kCollectThreads)
    k_fix_collect(const uint32_t* __restrict__ fix_bits, const uint32_t* __restrict__ keys, uint32_t n,
                  const uint32_t* __restrict__ offs, FixLists lists) {
    __shared__ uint32_t s_cell[kFixLists][kCollectWords * 32u];
    __shared__ uint32_t s_n[kFixLists], s_base[kFixLists];
    griddep_wait();  // the scatter's bitmap is complete
    griddep_launch();
    const uint32_t tid = threadIdx.x;
    if (tid < (uint32_t)kFixLists) s_n[tid] = 0u;
    __syncthreads();
    const uint32_t words = (n + 31u) / 32u;
    const uint32_t w = blockIdx.x * kCollectWords + tid / 4u, sh = 8u * (tid & 3u);
    uint32_t bits = w < words ? (__ldcg(fix_bits + w) >> sh) & 0xFFu : 0u;
    while (bits) {
        const uint32_t c = __ldg(keys + 32u * w + sh + (uint32_t)(__ffs(bits) - 1));
        bits &= bits - 1u;
        const uint32_t m = __ldg(offs + c + 1u) - __ldg(offs + c);
        const int cls = m <= kFixSmall ? kFixListSmall : (m <= kFixWarp ? kFixListWarp : kFixListHuge);
        s_cell[cls][atomicAdd(&s_n[cls], 1u)] = c;  // at most 32 * kCollectWords marks per block
    }
    __syncthreads();
    if (tid < (uint32_t)kFixLists && s_n[tid]) s_base[tid] = atomicAdd(lists.ctl + tid, s_n[tid]);
    __syncthreads();
#pragma unroll
    for (int c = 0; c < kFixLists; ++c) {
        for (uint32_t j = tid; j < s_n[c]; j += kCollectThreads) {
            const uint32_t at = s_base[c] + j;  // lists hold every cell that can qualify; the bound guards bad counts
            if (at < lists.cap[c]) lists.list[c][at] = s_cell[c][j];
        }
    }
}

// ---------------------------------------------------------------- fixup
// The listed cells (see k_fix_collect) get their slots back in ascending input order
// and (spos != NULL) re-gather their sorted state copy from the state source: one
// buffer (a world), or each scene's current buffer (a batch, where cells and
// coarse tiles of HOLD scenes are left alone).  Cells of up to kFixSmall slots: a thread
// each (sorting network in registers); up to kFixWarp: a warp each (bitonic sort
// in registers and shuffles); larger: a block each (bitmap of the input indices,
// chunk by chunk of their range, read back in order).
constexpr uint32_t kFixThreads = 256;
constexpr uint32_t kBitmapWords = 8192;                 // 32 KB of shared memory
constexpr uint32_t kBitmapValues = kBitmapWords * 32u;  // input indices per bitmap chunk

// Block-wide min (is_min) or max of v; every thread gets the result.
__device__ __forceinline__ uint32_t block_reduce(uint32_t v, uint32_t* s_red, bool is_min) {
    for (int o = 16; o > 0; o >>= 1) {
        const uint32_t u = __shfl_xor_sync(0xFFFFFFFFu, v, o);
        v = is_min ? min(v, u) : max(v, u);
    }
    __syncthreads();
    if ((threadIdx.x & 31u) == 0u) s_red[threadIdx.x >> 5] = v;
    __syncthreads();
    v = s_red[0];
    for (uint32_t w = 1; w < blockDim.x / 32u; ++w) v = is_min ? min(v, s_red[w]) : max(v, s_red[w]);
    __syncthreads();
    return v;
}

// Block-wide exclusive prefix sum of v; `total` receives the sum over the block.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_red, uint32_t& total) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31u) s_red[warp] = incl;
    __syncthreads();
    uint32_t base = 0, sum = 0;
    for (uint32_t w = 0; w < blockDim.x / 32u; ++w) {
        if (w < warp) base += s_red[w];
        sum += s_red[w];
    }
    __syncthreads();
    total = sum;
    return base + incl - v;
}

struct OneBuffer {
    const float4* p;
    const uint4* q;
    __device__ __forceinline__ bool tile_active(uint32_t) const { return true; }
    __device__ __forceinline__ bool any_init() const { return false; }
    __device__ __forceinline__ bool tile_init(uint32_t) const { return false; }
    __device__ __forceinline__ float4 pos(uint32_t o) const { return __ldg(p + o); }
    __device__ __forceinline__ uint4 vfme(uint32_t o) const { return __ldg(q + o); }
};

struct SceneBuffers {
    const SceneDev* scenes;
    const uint32_t* slot_tile_scene;  // scene of slot t * kPhysicsTile
    const uint32_t* cell_tile_scene;  // scene of scan tile t
    const float4* p0;
    const float4* p1;
    const uint4* q0;
    const uint4* q1;
    __device__ __forceinline__ bool tile_active(uint32_t t) const {
        return __ldg(&scenes[__ldg(cell_tile_scene + t)].mode) != kModeHold;
    }
    __device__ __forceinline__ bool any_init() const { return true; }
    __device__ __forceinline__ bool tile_init(uint32_t t) const {
        return __ldg(&scenes[__ldg(cell_tile_scene + t)].mode) == kModeInit;
    }
    __device__ __forceinline__ uint32_t parity(uint32_t o) const {
        uint32_t s = __ldg(slot_tile_scene + o / kPhysicsTile);
        while (o >= __ldg(&scenes[s].agent_end)) ++s;
        return __ldg(&scenes[s].parity);
    }
    __device__ __forceinline__ float4 pos(uint32_t o) const { return __ldg((parity(o) ? p1 : p0) + o); }
    __device__ __forceinline__ uint4 vfme(uint32_t o) const { return __ldg((parity(o) ? q1 : q0) + o); }
};

// Ascending bitonic sort of the warp's 32 S keys, key e = 32 s + lane in v[s]
// (S a power of two, at most kFixWarp / 32): partners e ^ j in other lanes are
// exchanged with shuffles, partners in other registers of the same lane in place.
template <uint32_t S>
__device__ __forceinline__ void warp_bitonic(uint32_t (&v)[kFixWarp / 32], uint32_t lane) {
#pragma unroll
    for (uint32_t k = 2u; k <= 32u * S; k <<= 1) {
#pragma unroll
        for (uint32_t j = k >> 1; j > 0u; j >>= 1) {
            if (j < 32u) {
#pragma unroll
                for (uint32_t s = 0; s < S; ++s) {
                    const uint32_t e = 32u * s + lane;
                    const uint32_t o = __shfl_xor_sync(0xFFFFFFFFu, v[s], (int)j);
                    const bool up = (e & k) == 0u, low = (e & j) == 0u;
                    v[s] = (low == up) ? min(v[s], o) : max(v[s], o);
                }
            } else {
                const uint32_t js = j / 32u;
#pragma unroll
                for (uint32_t s = 0; s < S; ++s) {
                    if (s & js) continue;
                    const uint32_t e = 32u * s + lane;
                    const uint32_t a = v[s], b = v[s | js];
                    const bool up = (e & k) == 0u;
                    v[s] = up ? min(a, b) : max(a, b);
                    v[s | js] = up ? max(a, b) : min(a, b);
                }
            }
        }
    }
}

template <class Src>
__global__ void __launch_bounds__(kFixThreads)
    k_cell_fix(const uint32_t* __restrict__ offs, uint32_t* perm, uint32_t* __restrict__ hist, uint32_t cells,
               uint32_t* __restrict__ coarse, uint32_t tiles,
               FixLists lists, uint32_t* __restrict__ tmp, Src src,
               float4* __restrict__ spos, uint4* __restrict__ svfme) {
    __shared__ uint32_t s_v[kBitmapWords];
    __shared__ uint32_t s_red[kFixThreads / 32 + 1];
    griddep_wait();
    griddep_launch();
    const uint32_t tid = threadIdx.x, lane = tid & 31u;
    // the scan of this frame is over: clear the tile counts for the next one; the
    // cell counts went back to zero in the scatter, except those of scenes in
    // their INIT frame (placed in identity order, nothing subtracted)
    if (blockIdx.x == 0)
        for (uint32_t t = tid; t < tiles; t += blockDim.x)
            if (src.tile_active(t)) coarse[t] = 0u;
    if (src.any_init())
        for (uint32_t c = (blockIdx.x * blockDim.x + tid) * 4u; c < cells; c += gridDim.x * blockDim.x * 4u)
            if (src.tile_init(c / kScanTile)) *reinterpret_cast<uint4*>(hist + c) = make_uint4(0u, 0u, 0u, 0u);

    const uint32_t* __restrict__ small = lists.list[0];
    const uint32_t* __restrict__ mid = lists.list[1];
    const uint32_t* __restrict__ huge = lists.list[2];

    // small cells: one thread each, the cell held in registers (a sorting
    // network over kFixSmall slots; empty slots hold 0xFFFFFFFF and stay last)
    const uint32_t n_small = min(lists.ctl[kFixListSmall], lists.cap[0]);
    for (uint32_t x = blockIdx.x * blockDim.x + tid; x < n_small; x += gridDim.x * blockDim.x) {
        const uint32_t c = small[x];
        const uint32_t lo = offs[c], m = offs[c + 1u] - lo;
        uint32_t v[kFixSmall];
        bool sorted = true;
#pragma unroll
        for (uint32_t k = 0; k < kFixSmall; ++k) v[k] = k < m ? perm[lo + k] : 0xFFFFFFFFu;
#pragma unroll
        for (uint32_t k = 1; k < kFixSmall; ++k) sorted = sorted && v[k - 1u] <= v[k];
        if (sorted) continue;
        // Batcher's odd-even merge sort of 8 keys (19 compare-exchanges)
        constexpr uint8_t kNet[19][2] = {{0, 1}, {2, 3}, {4, 5}, {6, 7}, {0, 2}, {1, 3}, {4, 6}, {5, 7}, {1, 2},
                                         {5, 6}, {0, 4}, {1, 5}, {2, 6}, {3, 7}, {2, 4}, {3, 5}, {1, 2}, {3, 4},
                                         {5, 6}};
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const uint32_t a = v[kNet[q][0]], b = v[kNet[q][1]];
            v[kNet[q][0]] = min(a, b);
            v[kNet[q][1]] = max(a, b);
        }
#pragma unroll
        for (uint32_t k = 0; k < kFixSmall; ++k) {
            if (k < m) {
                perm[lo + k] = v[k];
                if (spos) {
                    spos[lo + k] = src.pos(v[k]);
                    svfme[lo + k] = src.vfme(v[k]);
                }
            }
        }
    }

    // mid cells: one warp each, a bitonic sort of the cell's input indices held
    // in registers (slot e = 32 s + lane is v[s]; padded with 0xFFFFFFFF to 32 S
    // slots, S a power of two)
    const uint32_t n_mid = min(lists.ctl[kFixListWarp], lists.cap[1]);
    const uint32_t warps = gridDim.x * (blockDim.x / 32u);
    for (uint32_t x = blockIdx.x * (blockDim.x / 32u) + tid / 32u; x < n_mid; x += warps) {
        const uint32_t c = mid[x];
        const uint32_t lo = offs[c], m = offs[c + 1u] - lo;  // 9 <= m <= kFixWarp
        uint32_t v[kFixWarp / 32];
#pragma unroll
        for (uint32_t s = 0; s < kFixWarp / 32; ++s) {
            const uint32_t e = 32u * s + lane;
            v[s] = e < m ? perm[lo + e] : 0xFFFFFFFFu;
        }
        {  // the runs may have claimed their slots in input order already
            bool ok = true;
#pragma unroll
            for (uint32_t s = 0; s < kFixWarp / 32; ++s) {
                const uint32_t down = __shfl_down_sync(0xFFFFFFFFu, v[s], 1);
                const uint32_t wrap = s + 1u < kFixWarp / 32 ? __shfl_sync(0xFFFFFFFFu, v[s + 1u < kFixWarp / 32 ? s + 1u : s], 0)
                                                              : 0xFFFFFFFFu;
                ok = ok && v[s] <= (lane == 31u ? wrap : down);
            }
            if (__all_sync(0xFFFFFFFFu, ok)) continue;
        }
        if (m <= 32u) warp_bitonic<1>(v, lane);
        else if (m <= 64u) warp_bitonic<2>(v, lane);
        else if (m <= 128u) warp_bitonic<4>(v, lane);
        else warp_bitonic<8>(v, lane);
        __syncwarp();  // every lane has read the cell before any slot is rewritten
#pragma unroll
        for (uint32_t s = 0; s < kFixWarp / 32; ++s) {
            const uint32_t e = 32u * s + lane;
            if (e < m) {
                perm[lo + e] = v[s];
                if (spos) {
                    spos[lo + e] = src.pos(v[s]);
                    svfme[lo + e] = src.vfme(v[s]);
                }
            }
        }
    }

    // huge cells: one block each.  The cell's input indices are copied aside,
    // then each chunk of their value range becomes a bitmap in shared memory: the
    // set bits, read in order, are the chunk's indices in ascending order, and a
    // block scan of per-thread bit counts gives every thread its output position.
    const uint32_t n_huge = min(lists.ctl[kFixListHuge], lists.cap[2]);
    for (uint32_t x = blockIdx.x; x < n_huge; x += gridDim.x) {
        const uint32_t c = huge[x];
        const uint32_t lo = offs[c], m = offs[c + 1u] - lo;
        uint32_t vmin = 0xFFFFFFFFu, vmax = 0u;
        for (uint32_t j = tid; j < m; j += blockDim.x) {
            const uint32_t v = perm[lo + j];
            tmp[lo + j] = v;
            vmin = min(vmin, v);
            vmax = max(vmax, v);
        }
        vmin = block_reduce(vmin, s_red, true);
        vmax = block_reduce(vmax, s_red, false);  // ends with a barrier: tmp is complete
        uint32_t done = 0;
        for (uint32_t c0 = vmin;; c0 += kBitmapValues) {
            for (uint32_t w = tid; w < kBitmapWords; w += blockDim.x) s_v[w] = 0u;
            __syncthreads();
            for (uint32_t j = tid; j < m; j += blockDim.x) {
                const uint32_t d = tmp[lo + j] - c0;
                if (d < kBitmapValues) atomicOr(&s_v[d >> 5], 1u << (d & 31u));
            }
            __syncthreads();
            constexpr uint32_t kWordsPer = kBitmapWords / kFixThreads;
            uint32_t mine = 0;
#pragma unroll 8
            for (uint32_t w = 0; w < kWordsPer; ++w) mine += (uint32_t)__popc(s_v[tid * kWordsPer + w]);
            uint32_t total;
            const uint32_t before = block_exclusive_scan(mine, s_red, total);
            uint32_t at = lo + done + before;
            for (uint32_t w = 0; w < kWordsPer; ++w) {
                uint32_t bits = s_v[tid * kWordsPer + w];
                const uint32_t vb = c0 + (tid * kWordsPer + w) * 32u;
                while (bits) {  // four at a time, so the state loads overlap
                    uint32_t vv[4];
                    uint32_t got = 0;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        vv[q] = bits ? vb + (uint32_t)(__ffs(bits) - 1) : 0u;
                        got += bits ? 1u : 0u;
                        bits &= bits - 1u;
                    }
#pragma unroll
                    for (uint32_t q = 0; q < 4; ++q) {
                        if (q < got) {
                            perm[at + q] = vv[q];
                            if (spos) {
                                spos[at + q] = src.pos(vv[q]);
                                svfme[at + q] = src.vfme(vv[q]);
                            }
                        }
                    }
                    at += got;
                }
            }
            done += total;
            __syncthreads();  // bitmap free for the next chunk
            if (vmax - c0 < kBitmapValues) break;
        }
    }
}

// INIT frame after an upload: every key is 0, so the stable order is the
// identity and cell 0 holds everyone.  Also clears the counts (only hist[0] is set).
__global__ void k_init_order(uint32_t n, uint32_t cells, uint32_t* perm, uint32_t* offs,
                             uint32_t* hist, uint32_t* coarse, uint32_t tiles) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= max(n, cells); i += stride) {
        if (i < n) perm[i] = i;
        if (i <= cells) offs[i] = i == 0u ? 0u : n;
        if (i < cells) hist[i] = 0u;
        if (i < tiles) coarse[i] = 0u;
    }
}

// ---------------------------------------------------------------- tile counts
// coarse[t] := sum of hist over tile t's 4096 cells, one block per tile; for a
// batch only the tiles of scenes in their INIT frame (the others' tile counts
// are emitted by their LOOP pass or kept while they are held).
template <bool kScenes>
__global__ void __launch_bounds__(256)
    k_tile_counts(const uint32_t* __restrict__ hist, uint32_t cells, uint32_t* __restrict__ coarse,
                  const SceneDev* __restrict__ scenes, const uint32_t* __restrict__ cell_tile_scene) {
    __shared__ uint32_t s_red[8];
    const uint32_t t = blockIdx.x, tid = threadIdx.x;
    if (kScenes && __ldg(&scenes[__ldg(cell_tile_scene + t)].mode) != kModeInit) return;
    uint32_t sum = 0;
    for (uint32_t c = t * kScanTile + tid * 4u; c < min((t + 1u) * kScanTile, cells); c += 1024u) {
        if (c + 4u <= cells) {
            const uint4 x = __ldcg(reinterpret_cast<const uint4*>(hist + c));
            sum += (x.x + x.y) + (x.z + x.w);
        } else {
            for (uint32_t q = c; q < cells; ++q) sum += __ldcg(hist + q);
        }
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xFFFFFFFFu, sum, o);
    if ((tid & 31u) == 0u) s_red[tid >> 5] = sum;
    __syncthreads();
    if (tid == 0) {
        uint32_t total = 0;
        for (int w = 0; w < 8; ++w) total += s_red[w];
        coarse[t] = total;
    }
}

// ---------------------------------------------------------------- counting
// hist[keys[i]] += 1 for every sphere, one atomic per run of equal keys in a warp.
__global__ void __launch_bounds__(256)
    k_count_keys(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ hist,
                 uint32_t* __restrict__ coarse) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        uint32_t i = i0 + threadIdx.x;
        bool valid = i < n;
        uint32_t k = valid ? (__ldg(keys + i) & ~kInitKeyBit) : 0xFFFFFFFFu;
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, k);
        if (valid && lane == (uint32_t)(__ffs(peers) - 1)) atomicAdd(hist + k, (uint32_t)__popc(peers));
        uint32_t t = valid ? k / kScanTile : 0xFFFFFFFFu;
        uint32_t tp = __match_any_sync(0xFFFFFFFFu, t);
        if (valid && lane == (uint32_t)(__ffs(tp) - 1)) atomicAdd(coarse + t, (uint32_t)__popc(tp));
    }
}

__global__ void k_set_word(uint32_t* p, uint32_t v, uint32_t* q) {
    *p = v;
    *q = v;
}

}  // namespace

namespace {
FixLists fix_lists(const CountScratch& s) {
    return FixLists{s.fix_ctl, {s.fix[0], s.fix[1], s.fix[2]}, {s.fix_cap[0], s.fix_cap[1], s.fix_cap[2]}};
}
uint32_t fix_blocks() { return (uint32_t)device_sm_count() * 4u; }
uint32_t fix_words(uint32_t max_keys) { return max_keys / 32u + 1u; }
uint32_t collect_grid(uint32_t n) { return ((n + 31u) / 32u + kCollectWords - 1u) / kCollectWords; }
uint32_t scan_tiles(uint32_t cells) { return (cells + kScanTile - 1u) / kScanTile; }
uint32_t fix_capacity(int cls, uint32_t max_cells, uint32_t max_keys) {
    const uint32_t per = cls == kFixListSmall ? 2u : (cls == kFixListWarp ? kFixSmall + 1u : kFixWarp + 1u);
    return std::min(max_cells, max_keys / per) + 1u;
}
}  // namespace

uint64_t count_scratch_bytes(uint32_t max_cells, uint32_t max_keys) {
    const uint64_t padded = ((uint64_t)max_cells + kScanTile) & ~(uint64_t)15;
    uint64_t b = 4u * (padded + (max_cells + kScanTile - 1u) / kScanTile + 1u + kFixLists);
    for (int c = 0; c < kFixLists; ++c) b += 4u * fix_capacity(c, max_cells, max_keys);
    return b + 4u * ((uint64_t)max_keys + 1u) + 4u * (uint64_t)fix_words(max_keys);
}

cudaError_t count_scratch_alloc(CountScratch& s, uint32_t max_cells, uint32_t max_keys) {
    s.max_cells = max_cells;
    size_t padded = ((size_t)max_cells + kScanTile) & ~(size_t)15;  // uint4-aligned, room for offs[C]
    s.tiles = (max_cells + kScanTile - 1u) / kScanTile;
    cudaError_t e;
    if ((e = cudaMalloc(&s.hist, sizeof(uint32_t) * padded))) return e;
    if ((e = cudaMalloc(&s.coarse, sizeof(uint32_t) * (s.tiles + 1u)))) return e;
    if ((e = cudaMalloc(&s.fix_ctl, sizeof(uint32_t) * kFixLists))) return e;
    if ((e = cudaMalloc(&s.fix_tmp, sizeof(uint32_t) * ((size_t)max_keys + 1u)))) return e;
    if ((e = cudaMalloc(&s.fix_bits, sizeof(uint32_t) * fix_words(max_keys)))) return e;
    for (int c = 0; c < kFixLists; ++c) {
        s.fix_cap[c] = fix_capacity(c, max_cells, max_keys);
        if ((e = cudaMalloc(&s.fix[c], sizeof(uint32_t) * s.fix_cap[c]))) return e;
    }
    if ((e = cudaMemset(s.hist, 0, sizeof(uint32_t) * padded))) return e;
    if ((e = cudaMemset(s.coarse, 0, sizeof(uint32_t) * (s.tiles + 1u)))) return e;
    if ((e = cudaMemset(s.fix_ctl, 0, sizeof(uint32_t) * kFixLists))) return e;
    return cudaSuccess;
}

void count_scratch_free(CountScratch& s) {
    cudaFree(s.hist);
    cudaFree(s.coarse);
    cudaFree(s.fix_ctl);
    cudaFree(s.fix_tmp);
    cudaFree(s.fix_bits);
    for (auto* l : s.fix) cudaFree(l);
    s = CountScratch();
}

cudaError_t count_clear(CountScratch& s, uint32_t cells, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(s.hist, 0, sizeof(uint32_t) * cells, st);
    if (e) return e;
    return cudaMemsetAsync(s.coarse, 0, sizeof(uint32_t) * ((cells + kScanTile - 1u) / kScanTile), st);
}

cudaError_t count_keys(CountScratch& s, const uint32_t* keys, uint32_t n, uint32_t cells,
                       cudaStream_t st) {
    cudaError_t e = count_clear(s, cells, st);
    if (e || !n) return e;
    uint32_t blocks = std::min<uint32_t>((n + 255u) / 256u, (uint32_t)device_sm_count() * 8u);
    k_count_keys<<<blocks, 256, 0, st>>>(keys, n, s.hist, s.coarse);
    return cudaGetLastError();
}

cudaError_t count_reset_zero_keys(CountScratch& s, uint32_t n, uint32_t cells, cudaStream_t st) {
    cudaError_t e = count_clear(s, cells, st);
    if (e) return e;
    k_set_word<<<1, 1, 0, st>>>(s.hist, n, s.coarse);
    return cudaGetLastError();
}

cudaError_t count_scan(CountScratch& s, uint32_t* ctl, uint32_t cells, uint32_t* offs, cudaStream_t st, bool pdl) {
    (void)ctl;
    const uint32_t chunks = (cells + kScanChunk - 1u) / kScanChunk;
    return launch_pdl(pdl, k_cell_scan<false>, dim3(chunks), dim3(kScanThreads), 0, st, (const uint32_t*)s.hist,
                      (const uint32_t*)s.coarse, cells, offs, s.fix_ctl, (const SceneDev*)nullptr,
                      (const uint32_t*)nullptr);
}

cudaError_t count_scatter(CountScratch& s, const uint32_t* keys, uint32_t n, uint32_t cells,
                          const uint32_t* offs, uint32_t* perm, const float4* pos_in, const uint4* vfme_in,
                          float4* spos, uint4* svfme, uint4* bands, uint32_t N, cudaStream_t st, bool pdl) {
    cudaError_t e;
    if (n) {
        uint32_t blocks = std::min<uint32_t>((n + 255u) / 256u, (uint32_t)device_sm_count() * 8u);
        if ((e = launch_pdl(pdl, k_cell_scatter, dim3(blocks), dim3(256), 0, st, keys, n, s.hist, perm, pos_in,
                            vfme_in, spos, svfme, offs, bands, N, s.fix_bits)))
            return e;
        if ((e = launch_pdl(pdl, k_fix_collect, dim3(collect_grid(n)), dim3(kCollectThreads), 0, st,
                            (const uint32_t*)s.fix_bits, keys, n, offs, fix_lists(s))))
            return e;
    }
    OneBuffer src{pos_in, vfme_in};
    return launch_pdl(pdl && n, k_cell_fix<OneBuffer>, dim3(fix_blocks()), dim3(kFixThreads), 0, st, offs, perm,
                      s.hist, cells, s.coarse, scan_tiles(cells), fix_lists(s), s.fix_tmp, src, spos, svfme);
}

cudaError_t count_scan_scenes(CountScratch& s, const SceneDev* scenes, const uint32_t* cell_tile_scene,
                              uint32_t cells, uint32_t* offs, cudaStream_t st) {
    const uint32_t chunks = (cells + kScanChunk - 1u) / kScanChunk;
    k_cell_scan<true><<<chunks, kScanThreads, 0, st>>>(s.hist, s.coarse, cells, offs, s.fix_ctl, scenes,
                                                      cell_tile_scene);
    return cudaGetLastError();
}

cudaError_t count_scatter_scenes(CountScratch& s, const SceneDev* scenes, const uint32_t* tile_scene,
                                 const uint32_t* cell_tile_scene, const uint32_t* keys, uint32_t n, uint32_t cells,
                                 const uint32_t* offs, uint32_t* perm, const float4* pos_buf0,
                                 const float4* pos_buf1, const uint4* vfme_buf0, const uint4* vfme_buf1,
                                 float4* spos, uint4* svfme, uint4* bands, cudaStream_t st) {
    cudaError_t e;
    if (n) {
        uint32_t blocks = std::min<uint32_t>((n + 255u) / 256u, (uint32_t)device_sm_count() * 8u);
        k_cell_scatter_scenes<<<blocks, 256, 0, st>>>(scenes, tile_scene, keys, n, s.hist, perm, pos_buf0,
                                                      pos_buf1, vfme_buf0, vfme_buf1, spos, svfme, offs,
                                                      s.fix_bits, bands);
        if ((e = cudaGetLastError())) return e;
        k_fix_collect<<<collect_grid(n), kCollectThreads, 0, st>>>(s.fix_bits, keys, n, offs, fix_lists(s));
        if ((e = cudaGetLastError())) return e;
    }
    SceneBuffers src{scenes, tile_scene, cell_tile_scene, pos_buf0, pos_buf1, vfme_buf0, vfme_buf1};
    k_cell_fix<SceneBuffers><<<fix_blocks(), kFixThreads, 0, st>>>(offs, perm, s.hist, cells, s.coarse,
                                                                   scan_tiles(cells),
                                                                   fix_lists(s), s.fix_tmp, src, spos, svfme);
    return cudaGetLastError();
}

cudaError_t count_tile_counts(CountScratch& s, uint32_t cells, cudaStream_t st) {
    if (!cells) return cudaSuccess;
    k_tile_counts<false><<<scan_tiles(cells), 256, 0, st>>>(s.hist, cells, s.coarse, nullptr, nullptr);
    return cudaGetLastError();
}

cudaError_t count_tile_counts_scenes(CountScratch& s, const SceneDev* scenes, const uint32_t* cell_tile_scene,
                                     uint32_t cells, cudaStream_t st) {
    if (!cells) return cudaSuccess;
    k_tile_counts<true><<<scan_tiles(cells), 256, 0, st>>>(s.hist, cells, s.coarse, scenes, cell_tile_scene);
    return cudaGetLastError();
}

cudaError_t count_init_order(CountScratch& s, uint32_t n, uint32_t cells, uint32_t* offs, uint32_t* perm,
                             cudaStream_t st) {
    uint32_t m = std::max(n, cells) + 1u;
    uint32_t blocks = std::min<uint32_t>((m + 255u) / 256u, (uint32_t)device_sm_count() * 8u);
    k_init_order<<<blocks, 256, 0, st>>>(n, cells, perm, offs, s.hist, s.coarse,
                                         (cells + kScanTile - 1u) / kScanTile);
    return cudaGetLastError();
}

}  // namespace mb
