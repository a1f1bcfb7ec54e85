// mb_count_dev.cuh - device code of the counting sort (see mb_count.cu), as
// functions of an explicit block index so that both the per-stage kernels
// (mb_count.cu) and the fused frame kernel (mb_physics.cu) run the same code.
#pragma once

#include <cuda_runtime.h>

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
// One chunk (kScanThreads threads); s_warp, s_base: kScanThreads / 32 words each.
// A block that runs several chunks must synchronise between them.
template <bool kScenes, bool kCg = false>
__device__ __forceinline__ void scan_chunk(uint32_t chunk, const uint32_t* __restrict__ hist,
                                           const uint32_t* __restrict__ coarse, uint32_t cells,
                                           uint32_t* __restrict__ offs, uint32_t* fix_ctl,
                                           const SceneDev* __restrict__ scenes,
                                           const uint32_t* __restrict__ cell_tile_scene, uint32_t* s_warp,
                                           uint32_t* s_base) {
    constexpr int W = kScanThreads / 32;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t c0 = chunk * kScanChunk, tile = c0 / kScanTile;
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
    for (uint32_t t = first_tile + tid; t < tile; t += kScanThreads) bsum += ld_in<kCg>(coarse + t);
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
// run ends it); k_fix_marked puts the marked cells back in order.
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
// Input slots [vb * 256 kPer, ...) with a stride of nvb * 256 kPer (256-thread
// blocks): each thread takes kPer inputs 256 apart per step, their loads issued
// together (the agents-per-thread knob; warps still see 32 consecutive inputs).
template <bool kCg = false, uint32_t kPer = 1>
__device__ __forceinline__ void scatter_range(uint32_t vb, uint32_t nvb, const uint32_t* __restrict__ keys,
                                              uint32_t n, uint32_t* __restrict__ hist,
                                              uint32_t* __restrict__ perm, const float4* __restrict__ pos_in,
                                              const uint4* __restrict__ vfme_in, float4* __restrict__ spos,
                                              uint4* __restrict__ svfme, const uint32_t* __restrict__ offs,
                                              uint4* __restrict__ bands, uint32_t N,
                                              uint32_t* __restrict__ fix_bits) {
    const uint32_t lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
    const uint32_t stride = nvb * blockDim.x * kPer;
    for (uint32_t i0 = vb * blockDim.x * kPer; i0 < n; i0 += stride) {
        uint32_t k[kPer];
        float4 p[kPer];
        uint4 q[kPer];
#pragma unroll
        for (uint32_t r = 0; r < kPer; ++r) {
            const uint32_t i = i0 + r * blockDim.x + threadIdx.x;
            const bool valid = i < n;
            k[r] = valid ? ld_in<kCg>(keys + i) : 0xFFFFFFFFu;
            if (valid && spos) {
                p[r] = ld_in<kCg>(pos_in + i);
                q[r] = ld_in<kCg>(vfme_in + i);
            }
        }
#pragma unroll
        for (uint32_t r = 0; r < kPer; ++r) {
            const uint32_t i = i0 + r * blockDim.x + threadIdx.x;
            const bool valid = i < n;
            // a key flagged kInitKeyBit belongs to a scene in its INIT frame: all its
            // keys are equal, so its stable order is the identity and the slot is i
            const bool ident = valid && (k[r] & kInitKeyBit);
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, ident ? 0xFFFFFFFEu : k[r]);
            const uint32_t leader = (uint32_t)(__ffs(peers) - 1);
            uint32_t b = 0;
            bool mark = false;
            if (valid && !ident && lane == leader) {
                const uint32_t g = (uint32_t)__popc(peers);
                const uint32_t lo = ld_in<kCg>(offs + k[r]), hi = ld_in<kCg>(offs + k[r] + 1u);
                b = hi - atomicSub(hist + k[r], g);  // the run's first slot
                mark = listed(lo, hi, b, g);
            }
            b = __shfl_sync(0xFFFFFFFFu, b, (int)leader);
            mark_fix(fix_bits, i, n, mark);
            const uint32_t dst = ident ? i : b + (uint32_t)__popc(peers & lt);
            if (valid && dst < n) {  // only counts that disagree with the keys fail dst < n
                perm[dst] = i;
                if (spos) {
                    spos[dst] = p[r];
                    svfme[dst] = q[r];
                }
                if (bands && !ident) write_band_bounds<kCg>(bands, offs, N, n, dst, k[r]);
            }
        }
    }
}

// The marked cells are read kCollectWords bitmap words per block of
// kCollectThreads threads, a byte (8 input slots) per thread.
constexpr uint32_t kCollectThreads = 256, kCollectWords = kCollectThreads / 4u;
constexpr uint32_t kMarkedBitmapWords = 2u * kCollectThreads * 8u;  // the last block's bitmap: 16 KB

// ---------------------------------------------------------------- fixup
// The listed cells get their slots back in ascending input order
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

template <bool kCg>
struct OneBufferT {
    const float4* p;
    const uint4* q;
    __device__ __forceinline__ bool tile_active(uint32_t) const { return true; }
    __device__ __forceinline__ bool any_init() const { return false; }
    __device__ __forceinline__ bool tile_init(uint32_t) const { return false; }
    __device__ __forceinline__ float4 pos(uint32_t o) const { return ld_in<kCg>(p + o); }
    __device__ __forceinline__ uint4 vfme(uint32_t o) const { return ld_in<kCg>(q + o); }
};
using OneBuffer = OneBufferT<false>;

struct SceneBuffers {
    const SceneDev* scenes;
    const uint32_t* slot_tile_scene;  // scene of slot t * kPhysicsTile
    const uint32_t* cell_tile_scene;  // scene of scan tile t
    const float4* p0;
    const float4* p1;
    const uint4* q0;
    const uint4* q1;
    bool init;  // a scene may be in its INIT frame (false for chained and ranked frames)
    __device__ __forceinline__ bool tile_active(uint32_t t) const {
        return __ldg(&scenes[__ldg(cell_tile_scene + t)].mode) != kModeHold;
    }
    __device__ __forceinline__ bool any_init() const { return init; }
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

// A cell of m <= kFixSmall slots from lo back in input order, by one thread (a
// sorting network over kFixSmall slots held in registers; empty slots hold
// 0xFFFFFFFF and stay last), with its sorted state copy re-gathered (spos != NULL).
template <class Src, bool kCg>
__device__ __forceinline__ void fix_small_cell(uint32_t lo, uint32_t m, uint32_t* perm, const Src& src,
                                               float4* __restrict__ spos, uint4* __restrict__ svfme) {
    uint32_t v[kFixSmall];
    bool sorted = true;
#pragma unroll
    for (uint32_t k = 0; k < kFixSmall; ++k) v[k] = k < m ? ld_cur<kCg>(perm + lo + k) : 0xFFFFFFFFu;
#pragma unroll
    for (uint32_t k = 1; k < kFixSmall; ++k) sorted = sorted && v[k - 1u] <= v[k];
    if (sorted) return;
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

// A cell of kFixSmall < m <= kFixWarp slots from lo back in input order, by one
// whole warp (a bitonic sort of the cell's input indices in registers: slot
// e = 32 s + lane is v[s], padded with 0xFFFFFFFF to 32 S slots, S a power of two).
template <class Src, bool kCg>
__device__ __forceinline__ void fix_warp_cell(uint32_t lo, uint32_t m, uint32_t lane, uint32_t* perm, const Src& src,
                                              float4* __restrict__ spos, uint4* __restrict__ svfme) {
    uint32_t v[kFixWarp / 32];
#pragma unroll
    for (uint32_t s = 0; s < kFixWarp / 32; ++s) {
        const uint32_t e = 32u * s + lane;
        v[s] = e < m ? ld_cur<kCg>(perm + lo + e) : 0xFFFFFFFFu;
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
        if (__all_sync(0xFFFFFFFFu, ok)) return;
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

// ---------------------------------------------------------------- marked cells
// The sort of this frame is past its scan: clear the tile counts for the next
// frame's physics pass and the cell counts of scenes in their INIT frame, which
// the scatter does not count down (they keep identity order); both spread over
// the blocks (a batch has thousands of tiles, each checked against its scene).
template <class Src>
__device__ __forceinline__ void clear_counts(uint32_t vb, uint32_t nvb, const Src& src, uint32_t* __restrict__ hist,
                                             uint32_t cells, uint32_t* __restrict__ coarse, uint32_t tiles) {
    const uint32_t tid = threadIdx.x;
    for (uint32_t t = vb * blockDim.x + tid; t < tiles; t += nvb * blockDim.x)
        if (src.tile_active(t)) coarse[t] = 0u;
    if (src.any_init())
        for (uint32_t c = (vb * blockDim.x + tid) * 4u; c < cells; c += nvb * blockDim.x * 4u)
            if (src.tile_init(c / kScanTile)) *reinterpret_cast<uint4*>(hist + c) = make_uint4(0u, 0u, 0u, 0u);
}

// Cells of more than kFixWarp slots listed in lists.list[kFixListHuge], one block
// each (block vb of nvb; kFixThreads threads, kWords a multiple of them).  The
// cell's input indices are copied aside, then each chunk of their value range
// becomes a bitmap in shared memory: the set bits, read in order, are the chunk's
// indices in ascending order, and a block scan of per-thread bit counts gives
// every thread its output position.  The list was written by other blocks of
// the same launch or an earlier one: read from L2.  s_v: kWords words, s_red:
// kFixThreads / 32 + 1 words.
template <class Src, bool kCg, uint32_t kWords>
__device__ __forceinline__ void fix_huge(uint32_t vb, uint32_t nvb, const FixLists& lists,
                                         const uint32_t* __restrict__ offs, uint32_t* perm,
                                         uint32_t* __restrict__ tmp, const Src& src, float4* __restrict__ spos,
                                         uint4* __restrict__ svfme, uint32_t* s_v, uint32_t* s_red) {
    constexpr uint32_t kValues = kWords * 32u, kWordsPer = kWords / kFixThreads;
    static_assert(kWords % kFixThreads == 0, "bitmap words per thread");
    const uint32_t tid = threadIdx.x;
    const uint32_t n_huge = min(__ldcg(lists.ctl + kFixListHuge), lists.cap[kFixListHuge]);
    for (uint32_t x = vb; x < n_huge; x += nvb) {
        const uint32_t c = __ldcg(lists.list[kFixListHuge] + x);
        const uint32_t lo = ld_cur<kCg>(offs + c), m = ld_cur<kCg>(offs + c + 1u) - lo;
        uint32_t vmin = 0xFFFFFFFFu, vmax = 0u;
        for (uint32_t j = tid; j < m; j += blockDim.x) {
            const uint32_t v = __ldcg(perm + lo + j);
            tmp[lo + j] = v;
            vmin = min(vmin, v);
            vmax = max(vmax, v);
        }
        vmin = block_reduce(vmin, s_red, true);
        vmax = block_reduce(vmax, s_red, false);  // ends with a barrier: tmp is complete
        uint32_t done = 0;
        for (uint32_t c0 = vmin;; c0 += kValues) {
            for (uint32_t w = tid; w < kWords; w += blockDim.x) s_v[w] = 0u;
            __syncthreads();
            for (uint32_t j = tid; j < m; j += blockDim.x) {
                const uint32_t d = tmp[lo + j] - c0;
                if (d < kValues) atomicOr(&s_v[d >> 5], 1u << (d & 31u));
            }
            __syncthreads();
            uint32_t mine = 0;
#pragma unroll 8
            for (uint32_t w = 0; w < kWordsPer; ++w) mine += (uint32_t)__popc(s_v[tid * kWordsPer + w]);
            uint32_t total;
            const uint32_t before = block_exclusive_scan(mine, s_red, total);
            uint32_t at = lo + done + before;
            for (uint32_t w = 0; w < kWordsPer; ++w) {
                uint32_t bits = s_v[tid * kWordsPer + w];
                const uint32_t vb0 = c0 + (tid * kWordsPer + w) * 32u;
                while (bits) {  // four at a time, so the state loads overlap
                    uint32_t vv[4];
                    uint32_t got = 0;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        vv[q] = bits ? vb0 + (uint32_t)(__ffs(bits) - 1) : 0u;
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
            if (vmax - c0 < kValues) break;
        }
    }
}

// One block (kCollectThreads threads) of the fixup of the marked cells: it reads
// kCollectWords words of the bitmap, a byte (8 input slots) per thread.  A
// marked input slot names a cell (its key) that runs of several warps filled.
// Each warp gathers the marked slots of its 256 input slots in shared memory and
// deals them out to its lanes, so a lane usually has one cell at most: cells of
// up to kFixSmall slots are put back in input order by that lane; cells of up to
// kFixWarp slots are collected for the block, whose eight warps then take one
// each in turn (crowded scenes mark many close together, so the block shares
// them out rather than the warp that found them); larger cells are listed
// (fix_huge).  kLast: the last block to finish fixes the listed cells (the
// per-stage kernel); otherwise the caller does after a grid barrier.
struct MarkedSmem {
    union {
        struct {
            uint32_t slot[kCollectThreads * 8u];  // each warp's marked input slots
            uint32_t mid[kCollectThreads * 8u];   // the block's cells of kFixSmall+1 .. kFixWarp slots
        } a;
        uint32_t v[kMarkedBitmapWords];           // the last block's bitmap (fix_huge)
    } u;
    uint32_t red[kCollectThreads / 32 + 1];
    uint32_t cnt[4];  // [0] mid cells, [1] huge cells, [2] list base, [3] last block
};
template <class Src, bool kCg = false, bool kLast = false>
__device__ __forceinline__ void fix_marked_block(uint32_t vb, uint32_t nvb, const uint32_t* __restrict__ fix_bits,
                                                 const uint32_t* __restrict__ keys, uint32_t n,
                                                 const uint32_t* __restrict__ offs, uint32_t* perm,
                                                 const FixLists& lists, uint32_t* __restrict__ tmp, const Src& src,
                                                 float4* __restrict__ spos, uint4* __restrict__ svfme,
                                                 MarkedSmem& S) {
    constexpr uint32_t kPerWarp = 32u * 8u;  // input slots a warp reads the marks of
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t words = (n + 31u) / 32u;
    const uint32_t w = vb * kCollectWords + tid / 4u, sh = 8u * (tid & 3u);
    uint32_t byte = w < words ? (__ldcg(fix_bits + w) >> sh) & 0xFFu : 0u;
    if (tid < 2u) S.cnt[tid] = 0u;
    // compact the warp's marked slots
    const uint32_t cnt = (uint32_t)__popc(byte);
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    uint32_t* const my = S.u.a.slot + warp * kPerWarp;
    for (uint32_t at = incl - cnt; byte; byte &= byte - 1u, ++at) my[at] = 32u * w + sh + (uint32_t)(__ffs(byte) - 1);
    __syncthreads();  // slots written; counters cleared
    for (uint32_t k = lane; k < total; k += 32u) {
        const uint32_t c = ld_in<kCg>(keys + my[k]);
        const uint32_t lo = ld_cur<kCg>(offs + c), m = ld_cur<kCg>(offs + c + 1u) - lo;
        if (m <= kFixSmall) {
            fix_small_cell<Src, kCg>(lo, m, perm, src, spos, svfme);
        } else if (m <= kFixWarp) {
            S.u.a.mid[atomicAdd(&S.cnt[0], 1u)] = c;
        } else {
            const uint32_t at = atomicAdd(lists.ctl + kFixListHuge, 1u);
            if (at < lists.cap[kFixListHuge]) lists.list[kFixListHuge][at] = c;  // holds every cell that can qualify
        }
    }
    __syncthreads();  // the block's mid cells are collected
    const uint32_t n_mid = S.cnt[0];
    for (uint32_t x = warp; x < n_mid; x += kCollectThreads / 32u) {
        const uint32_t c = S.u.a.mid[x];
        const uint32_t lo = ld_cur<kCg>(offs + c), m = ld_cur<kCg>(offs + c + 1u) - lo;
        fix_warp_cell<Src, kCg>(lo, m, lane, perm, src, spos, svfme);
    }
    if (kLast) {
        __syncthreads();  // every warp is done with the shared lists
        if (tid == 0) {
            __threadfence();  // this block's list entries before it counts itself finished
            S.cnt[3] = atomicAdd(lists.ctl + kFixListDone, 1u) == nvb - 1u ? 1u : 0u;
        }
        __syncthreads();
        if (S.cnt[3]) {
            __threadfence();  // every other block's list entries
            if (tid == 0) lists.ctl[kFixListDone] = 0u;
            fix_huge<Src, kCg, kMarkedBitmapWords>(0u, 1u, lists, offs, perm, tmp, src, spos, svfme, S.u.v, S.red);
        }
    }
}

}  // namespace
}  // namespace mb
