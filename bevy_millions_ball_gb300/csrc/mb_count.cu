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
//   4. k_fix_marked: the marked cells' slots are put back in ascending input
//      order (what a stable sort yields), re-gathering their state copy - cells
//      of up to 8 slots by the thread that reads the mark, up to 256 by a warp
//      of the block that found them, larger ones by the last block to finish;
//      it also clears the tile counts for the next frame.
//
// The result is bit-identical to a stable sort; offs[] replaces start/close.

#include <cuda_runtime.h>

#include <algorithm>

#include "mb_count_dev.cuh"
#include "mb_internal.h"

namespace mb {
namespace {

// far_reset (nullable): a far-move list emptied for this frame's physics pass
// (rank placement).
template <bool kScenes>
__global__ void __launch_bounds__(kScanThreads)
    k_cell_scan(const uint32_t* __restrict__ hist, const uint32_t* __restrict__ coarse, uint32_t cells,
                uint32_t* __restrict__ offs, uint32_t* fix_ctl,
                const SceneDev* __restrict__ scenes, const uint32_t* __restrict__ cell_tile_scene,
                uint32_t* __restrict__ far_reset) {
    __shared__ uint32_t s_warp[kScanThreads / 32], s_base[kScanThreads / 32];
    griddep_wait();  // after the previous frame's physics pass, when chained to it
    griddep_launch();
    if (far_reset && blockIdx.x == 0 && threadIdx.x == 0) *far_reset = 0u;
    scan_chunk<kScenes>(blockIdx.x, hist, coarse, cells, offs, fix_ctl, scenes, cell_tile_scene, s_warp, s_base);
}

// Rank placement of one world's spheres (MB_SORT_RANK), kPer spheres per
// thread (kRankThreads kPer per block, their loads issued together).  The input is the
// previous frame's sorted order, described by offs_old; a sphere of new cell
// k = (kx, kz) that moved at most one cell sits in the old ranges of cells
// (kx-1..kx+1, kz-1..kz+1), three slot ranges, one per row.  Its stable slot is
// offs[k] plus the spheres with key k before it in those ranges, plus the
// listed far moves with key k before it (a per-block bit filter of their cells
// spares the others the list).  No atomics, no marks: the order is final, so
// the band table is written here too.  The first sphere of each cell clears
// its count for the next frame.  A far list that overflowed (more than kFarCap
// moves, or forced after an upload, a grid or a tuning change) sends every
// block down the claim-and-fixup path instead (the fixup kernel after this one
// then runs too).
__device__ __forceinline__ uint32_t bloom_bit(uint32_t k) { return (k * 2654435761u) >> 20; }  // 12 bits

constexpr uint32_t kRankThreads = 128;  // (256-thread blocks: P-1M frame +1.8 us)

template <uint32_t kPer>
__global__ void __launch_bounds__(kRankThreads)
    k_cell_rank(const uint32_t* __restrict__ keys, uint32_t n, uint32_t cells, uint32_t* __restrict__ hist,
                uint32_t* __restrict__ perm, const float4* __restrict__ pos_in, const uint4* __restrict__ vfme_in,
                float4* __restrict__ spos, uint4* __restrict__ svfme, const uint32_t* __restrict__ offs,
                const uint32_t* __restrict__ offs_old, const uint32_t* __restrict__ far, uint4* __restrict__ bands,
                uint32_t N, uint32_t* __restrict__ fix_bits) {
    __shared__ uint32_t s_key[kFarCap], s_slot[kFarCap], s_bloom[kBloomWords];
    griddep_wait();  // the scan's offsets, the previous physics pass's keys and far moves
    griddep_launch();
    const uint32_t F = __ldcg(far);
    if (F > kFarCap) {
        scatter_range<false, 1>(blockIdx.x, gridDim.x, keys, n, hist, perm, pos_in, vfme_in, spos, svfme, offs,
                                bands, N, fix_bits);
        return;
    }
    const uint32_t tid = threadIdx.x;
    if (F) {
        for (uint32_t t = tid; t < kBloomWords; t += blockDim.x) s_bloom[t] = 0u;
        __syncthreads();
        for (uint32_t t = tid; t < F; t += blockDim.x) {
            const uint32_t sl = min(__ldcg(far + 1u + t), n - 1u), k = __ldg(keys + sl);
            s_slot[t] = sl;
            s_key[t] = k;
            const uint32_t b = bloom_bit(k);
            atomicOr(&s_bloom[b >> 5], 1u << (b & 31u));
        }
        __syncthreads();
    }
    const uint32_t i0 = blockIdx.x * blockDim.x * kPer + tid;
    uint32_t k[kPer], lo[kPer][3], hi[kPer][3], base[kPer];
    float4 p[kPer];
    uint4 q[kPer];
#pragma unroll
    for (uint32_t r = 0; r < kPer; ++r) {
        const uint32_t i = i0 + r * blockDim.x;
        k[r] = i < n ? __ldg(keys + i) : cells;
        if (spos && i < n) {
            p[r] = __ldg(pos_in + i);
            q[r] = __ldg(vfme_in + i);
        }
    }
#pragma unroll
    for (uint32_t r = 0; r < kPer; ++r) {
        const uint32_t i = i0 + r * blockDim.x;
        const bool ok = k[r] < cells;  // keys the physics pass cannot emit are skipped
        const uint32_t kz = ok ? k[r] / N : 0u, kx = ok ? k[r] - kz * N : 0u;
        const uint32_t c0 = kx > 0u ? kx - 1u : 0u, c1 = (kx + 1u < N ? kx + 1u : kx) + 1u;
        base[r] = ok ? __ldg(offs + k[r]) : 0u;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const bool row = ok && (d == 0 ? kz > 0u : (d == 2 ? kz + 1u < N : true));
            const uint32_t rw = kz + (uint32_t)d - 1u;
            lo[r][d] = row ? __ldg(offs_old + rw * N + c0) : 0u;
            hi[r][d] = row ? min(__ldg(offs_old + rw * N + c1), i) : 0u;
        }
    }
#pragma unroll
    for (uint32_t r = 0; r < kPer; ++r) {
        const uint32_t i = i0 + r * blockDim.x;
        if (k[r] >= cells) continue;
        uint32_t cnt = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            for (uint32_t j = lo[r][d]; j < hi[r][d]; j += 4u) {
                uint32_t kk[4];
#pragma unroll
                for (uint32_t u = 0; u < 4u; ++u) kk[u] = __ldg(keys + min(j + u, hi[r][d] - 1u));
#pragma unroll
                for (uint32_t u = 0; u < 4u; ++u) cnt += (j + u < hi[r][d] && kk[u] == k[r]) ? 1u : 0u;
            }
        }
        if (F) {
            const uint32_t b = bloom_bit(k[r]);
            if (s_bloom[b >> 5] & (1u << (b & 31u)))
                for (uint32_t t = 0; t < F; ++t) cnt += (s_key[t] == k[r] && s_slot[t] < i) ? 1u : 0u;
        }
        if (cnt == 0u) hist[k[r]] = 0u;  // the cell's first sphere
        const uint32_t dst = base[r] + cnt;
        if (dst < n) {
            perm[dst] = i;
            if (spos) {
                spos[dst] = p[r];
                svfme[dst] = q[r];
            }
            if (bands) write_band_bounds(bands, offs, N, n, dst, k[r]);
        }
    }
}

template <uint32_t kPer>
__global__ void __launch_bounds__(256)
    k_cell_scatter(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ hist,
                   uint32_t* __restrict__ perm, const float4* __restrict__ pos_in,
                   const uint4* __restrict__ vfme_in, float4* __restrict__ spos,
                   uint4* __restrict__ svfme, const uint32_t* __restrict__ offs, uint4* __restrict__ bands,
                   uint32_t N, uint32_t* __restrict__ fix_bits) {
    griddep_wait();
    griddep_launch();
    scatter_range<false, kPer>(blockIdx.x, gridDim.x, keys, n, hist, perm, pos_in, vfme_in, spos, svfme, offs, bands,
                               N, fix_bits);
}

// The same for a batch: slot i's scene (from the tile table) gives the buffer
// holding its state; spheres of HOLD scenes are left alone.  kPer inputs per
// thread per step, as in scatter_range; blocks vb of nvb, grid-strided.
template <uint32_t kPer>
__device__ __forceinline__ void scatter_scenes_range(
    uint32_t vb, uint32_t nvb, const SceneDev* __restrict__ scenes, const uint32_t* __restrict__ tile_scene,
    const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ hist, uint32_t* __restrict__ perm,
    const float4* __restrict__ pos0, const float4* __restrict__ pos1, const uint4* __restrict__ vfme0,
    const uint4* __restrict__ vfme1, float4* __restrict__ spos, uint4* __restrict__ svfme,
    const uint32_t* __restrict__ offs, uint32_t* __restrict__ fix_bits, uint4* __restrict__ bands) {
    const uint32_t lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
    const uint32_t stride = nvb * blockDim.x * kPer;
    for (uint32_t i0 = vb * blockDim.x * kPer; i0 < n; i0 += stride) {
        uint32_t k[kPer], sc[kPer];
        bool act[kPer];
        float4 p[kPer];
        uint4 q[kPer];
#pragma unroll
        for (uint32_t r = 0; r < kPer; ++r) {
            const uint32_t i = i0 + r * blockDim.x + threadIdx.x;
            uint32_t mode = kModeHold, parity = 0, s = 0;
            if (i < n) {
                s = __ldg(tile_scene + i / kPhysicsTile);
                while (i >= __ldg(&scenes[s].agent_end)) ++s;
                mode = __ldg(&scenes[s].mode);
                parity = __ldg(&scenes[s].parity);
            }
            sc[r] = s;
            act[r] = i < n && mode != kModeHold;
            k[r] = act[r] ? __ldg(keys + i) : 0xFFFFFFFFu;
            if (act[r]) {
                p[r] = __ldg((parity ? pos1 : pos0) + i);
                q[r] = __ldg((parity ? vfme1 : vfme0) + i);
            }
        }
#pragma unroll
        for (uint32_t r = 0; r < kPer; ++r) {
            const uint32_t i = i0 + r * blockDim.x + threadIdx.x;
            const bool valid = act[r];
            const bool ident = valid && (k[r] & kInitKeyBit);
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, ident ? 0xFFFFFFFEu : k[r]);
            const uint32_t leader = (uint32_t)(__ffs(peers) - 1);
            uint32_t b = 0;
            bool mark = false;
            if (valid && !ident && lane == leader) {
                const uint32_t g = (uint32_t)__popc(peers);
                const uint32_t lo = __ldg(offs + k[r]), hi = __ldg(offs + k[r] + 1u);
                b = hi - atomicSub(hist + k[r], g);  // the run's first slot
                mark = listed(lo, hi, b, g);
            }
            b = __shfl_sync(0xFFFFFFFFu, b, (int)leader);
            mark_fix(fix_bits, i, n, mark);
            const uint32_t dst = ident ? i : b + (uint32_t)__popc(peers & lt);
            if (valid && dst < n) {  // only counts that disagree with the keys fail dst < n
                perm[dst] = i;
                spos[dst] = p[r];
                svfme[dst] = q[r];
                if (bands && !ident) {  // the scene's band table entries, in its own cell coordinates
                    const uint32_t cb = __ldg(&scenes[sc[r]].cell_base);
                    write_band_bounds(bands, offs + cb, __ldg(&scenes[sc[r]].P.N), n, dst, k[r] - cb);
                }
            }
        }
    }
}

template <uint32_t kPer>
__global__ void __launch_bounds__(256)
    k_cell_scatter_scenes(const SceneDev* __restrict__ scenes, const uint32_t* __restrict__ tile_scene,
                          const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ hist,
                          uint32_t* __restrict__ perm, const float4* __restrict__ pos0,
                          const float4* __restrict__ pos1, const uint4* __restrict__ vfme0,
                          const uint4* __restrict__ vfme1, float4* __restrict__ spos, uint4* __restrict__ svfme,
                          const uint32_t* __restrict__ offs, uint32_t* __restrict__ fix_bits,
                          uint4* __restrict__ bands) {
    scatter_scenes_range<kPer>(blockIdx.x, gridDim.x, scenes, tile_scene, keys, n, hist, perm, pos0, pos1, vfme0,
                               vfme1, spos, svfme, offs, fix_bits, bands);
}

// Rank placement of a batch whose scenes are all in LOOP (k_cell_rank per scene:
// the neighbourhood in the scene's own cell coordinates, its state from its
// current buffer); one sphere per thread.  The far list holds pool-wide slots,
// its keys pool-wide cells.  An overflowed list: the batched scatter instead.
__global__ void __launch_bounds__(kRankThreads)
    k_cell_rank_scenes(const SceneDev* __restrict__ scenes, const uint32_t* __restrict__ tile_scene,
                       const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ hist,
                       uint32_t* __restrict__ perm, const float4* __restrict__ pos0, const float4* __restrict__ pos1,
                       const uint4* __restrict__ vfme0, const uint4* __restrict__ vfme1, float4* __restrict__ spos,
                       uint4* __restrict__ svfme, const uint32_t* __restrict__ offs,
                       const uint32_t* __restrict__ offs_old, const uint32_t* __restrict__ far,
                       uint32_t* __restrict__ fix_bits, uint4* __restrict__ bands) {
    __shared__ uint32_t s_key[kFarCap], s_slot[kFarCap], s_bloom[kBloomWords];
    griddep_wait();
    griddep_launch();
    const uint32_t F = __ldcg(far);
    if (F > kFarCap) {
        scatter_scenes_range<1>(blockIdx.x, gridDim.x, scenes, tile_scene, keys, n, hist, perm, pos0, pos1, vfme0,
                                vfme1, spos, svfme, offs, fix_bits, bands);
        return;
    }
    const uint32_t tid = threadIdx.x;
    if (F) {
        for (uint32_t t = tid; t < kBloomWords; t += blockDim.x) s_bloom[t] = 0u;
        __syncthreads();
        for (uint32_t t = tid; t < F; t += blockDim.x) {
            const uint32_t sl = min(__ldcg(far + 1u + t), n - 1u), k = __ldg(keys + sl);
            s_slot[t] = sl;
            s_key[t] = k;
            const uint32_t b = bloom_bit(k);
            atomicOr(&s_bloom[b >> 5], 1u << (b & 31u));
        }
        __syncthreads();
    }
    const uint32_t i = blockIdx.x * blockDim.x + tid;
    if (i >= n) return;
    uint32_t sc = __ldg(tile_scene + i / kPhysicsTile);
    while (i >= __ldg(&scenes[sc].agent_end)) ++sc;
    const uint32_t k = __ldg(keys + i), cb = __ldg(&scenes[sc].cell_base), N = __ldg(&scenes[sc].P.N);
    const uint32_t parity = __ldg(&scenes[sc].parity);
    const float4 p = __ldg((parity ? pos1 : pos0) + i);
    const uint4 q = __ldg((parity ? vfme1 : vfme0) + i);
    const uint32_t kl = k - cb;
    if (kl >= N * N) return;  // keys the physics pass cannot emit
    const uint32_t base = __ldg(offs + k);
    const uint32_t kz = kl / N, kx = kl - kz * N;
    const uint32_t c0 = kx > 0u ? kx - 1u : 0u, c1 = (kx + 1u < N ? kx + 1u : kx) + 1u;
    const uint32_t* __restrict__ oo = offs_old + cb;
    uint32_t lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const bool row = d == 0 ? kz > 0u : (d == 2 ? kz + 1u < N : true);
        const uint32_t rw = kz + (uint32_t)d - 1u;
        lo[d] = row ? __ldg(oo + rw * N + c0) : 0u;
        hi[d] = row ? min(__ldg(oo + rw * N + c1), i) : 0u;
    }
    uint32_t cnt = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        for (uint32_t j = lo[d]; j < hi[d]; j += 4u) {
            uint32_t kk[4];
#pragma unroll
            for (uint32_t u = 0; u < 4u; ++u) kk[u] = __ldg(keys + min(j + u, hi[d] - 1u));
#pragma unroll
            for (uint32_t u = 0; u < 4u; ++u) cnt += (j + u < hi[d] && kk[u] == k) ? 1u : 0u;
        }
    }
    if (F) {
        const uint32_t b = bloom_bit(k);
        if (s_bloom[b >> 5] & (1u << (b & 31u)))
            for (uint32_t t = 0; t < F; ++t) cnt += (s_key[t] == k && s_slot[t] < i) ? 1u : 0u;
    }
    if (cnt == 0u) hist[k] = 0u;  // the cell's first sphere
    const uint32_t dst = base + cnt;
    if (dst < n) {
        perm[dst] = i;
        spos[dst] = p;
        svfme[dst] = q;
        if (bands) write_band_bounds(bands, offs + cb, N, n, dst, kl);
    }
}

template <class Src>
__global__ void __launch_bounds__(kCollectThreads)
    k_fix_marked(const uint32_t* __restrict__ fix_bits, const uint32_t* __restrict__ keys, uint32_t n,
                 const uint32_t* __restrict__ offs, uint32_t* perm, FixLists lists, uint32_t* __restrict__ tmp,
                 Src src, float4* __restrict__ spos, uint4* __restrict__ svfme, uint32_t* __restrict__ hist,
                 uint32_t cells, uint32_t* __restrict__ coarse, uint32_t tiles, const uint32_t* __restrict__ gate,
                 uint32_t nvb) {
    __shared__ MarkedSmem S;
    griddep_wait();  // the scatter's bitmap and order are complete
    griddep_launch();
    clear_counts(blockIdx.x, gridDim.x, src, hist, cells, coarse, tiles);
    if (gate && __ldcg(gate) <= kFarCap) return;
    // nvb blocks' worth of the bitmap, taken in turn by the launched blocks
    for (uint32_t vb = blockIdx.x; vb < nvb; vb += gridDim.x) {
        fix_marked_block<Src, false, true>(vb, nvb, fix_bits, keys, n, offs, perm, lists, tmp, src, spos, svfme, S);
        __syncthreads();  // shared lists free for the next one
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
uint32_t fix_words(uint32_t max_keys) { return max_keys / 32u + 1u; }
uint32_t collect_grid(uint32_t n) { return ((n + 31u) / 32u + kCollectWords - 1u) / kCollectWords; }
// Blocks the fixup launches: at most eight per SM, each taking collect_grid's
// blocks of the bitmap in turn (an idle fixup, the usual case under rank
// placement, then costs little to launch).
uint32_t fix_grid(uint32_t n) {
    return std::max(std::min<uint32_t>(collect_grid(n), (uint32_t)device_sm_count() * 8u), 1u);
}
uint32_t scan_tiles(uint32_t cells) { return (cells + kScanTile - 1u) / kScanTile; }
uint32_t fix_capacity(int cls, uint32_t max_cells, uint32_t max_keys) {
    if (cls != kFixListHuge) return 1u;  // only cells above kFixWarp slots are listed
    return std::min(max_cells, max_keys / (kFixWarp + 1u)) + 1u;
}
}  // namespace

uint64_t count_scratch_bytes(uint32_t max_cells, uint32_t max_keys) {
    const uint64_t padded = ((uint64_t)max_cells + kScanTile) & ~(uint64_t)15;
    uint64_t b = 4u * (padded + (max_cells + kScanTile - 1u) / kScanTile + 1u + kFixCtlWords);
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
    if ((e = cudaMalloc(&s.fix_ctl, sizeof(uint32_t) * kFixCtlWords))) return e;
    if ((e = cudaMalloc(&s.fix_tmp, sizeof(uint32_t) * ((size_t)max_keys + 1u)))) return e;
    if ((e = cudaMalloc(&s.fix_bits, sizeof(uint32_t) * fix_words(max_keys)))) return e;
    for (int c = 0; c < kFixLists; ++c) {
        s.fix_cap[c] = fix_capacity(c, max_cells, max_keys);
        if ((e = cudaMalloc(&s.fix[c], sizeof(uint32_t) * s.fix_cap[c]))) return e;
    }
    if ((e = cudaMemset(s.hist, 0, sizeof(uint32_t) * padded))) return e;
    if ((e = cudaMemset(s.coarse, 0, sizeof(uint32_t) * (s.tiles + 1u)))) return e;
    if ((e = cudaMemset(s.fix_ctl, 0, sizeof(uint32_t) * kFixCtlWords))) return e;
    return cudaSuccess;
}

cudaError_t count_rank_alloc(CountScratch& s) {
    if (s.offs_old) return cudaSuccess;
    cudaError_t e;
    const size_t padded = ((size_t)s.max_cells + kScanTile) & ~(size_t)15;
    if ((e = cudaMalloc(&s.offs_old, sizeof(uint32_t) * padded))) return e;
    for (auto*& l : s.far) {
        if ((e = cudaMalloc(&l, sizeof(uint32_t) * kFarWords))) return e;
        if ((e = cudaMemset(l, 0xFF, sizeof(uint32_t)))) return e;  // overflowed: no order to rank from yet
    }
    return cudaSuccess;
}

void count_scratch_free(CountScratch& s) {
    cudaFree(s.hist);
    cudaFree(s.coarse);
    cudaFree(s.fix_ctl);
    cudaFree(s.fix_tmp);
    cudaFree(s.fix_bits);
    cudaFree(s.offs_old);
    for (auto* l : s.far) cudaFree(l);
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

cudaError_t count_scan(CountScratch& s, uint32_t* ctl, uint32_t cells, uint32_t* offs, cudaStream_t st, bool pdl,
                       uint32_t* far_reset) {
    (void)ctl;
    const uint32_t chunks = (cells + kScanChunk - 1u) / kScanChunk;
    return launch_pdl(pdl, k_cell_scan<false>, dim3(chunks), dim3(kScanThreads), 0, st, (const uint32_t*)s.hist,
                      (const uint32_t*)s.coarse, cells, offs, s.fix_ctl, (const SceneDev*)nullptr,
                      (const uint32_t*)nullptr, far_reset);
}

cudaError_t count_rank(CountScratch& s, const uint32_t* keys, uint32_t n, uint32_t cells, const uint32_t* offs,
                       const uint32_t* offs_old, const uint32_t* far, uint32_t* perm, const float4* pos_in,
                       const uint4* vfme_in, float4* spos, uint4* svfme, uint4* bands, uint32_t N, cudaStream_t st,
                       bool pdl, uint32_t per_thread) {
    cudaError_t e;
    if (n) {
        const uint32_t per = per_thread == 4u ? 4u : (per_thread == 2u ? 2u : 1u);
        auto* kern = per == 4u ? k_cell_rank<4> : (per == 2u ? k_cell_rank<2> : k_cell_rank<1>);
        if ((e = launch_pdl(pdl, kern, dim3((n + kRankThreads * per - 1u) / (kRankThreads * per)), dim3(kRankThreads),
                            0, st, keys, n, cells,
                            s.hist, perm, pos_in, vfme_in, spos, svfme, offs, offs_old, far, bands, N, s.fix_bits)))
            return e;
    }
    const OneBuffer src{pos_in, vfme_in};
    return launch_pdl(pdl && n, k_fix_marked<OneBuffer>, dim3(fix_grid(n)),
                      dim3(kCollectThreads), 0, st, (const uint32_t*)s.fix_bits, keys, n, offs, perm, fix_lists(s),
                      s.fix_tmp, src, spos, svfme, s.hist, cells, s.coarse, scan_tiles(cells), far,
                      std::max(collect_grid(n), 1u));
}

cudaError_t count_scatter(CountScratch& s, const uint32_t* keys, uint32_t n, uint32_t cells,
                          const uint32_t* offs, uint32_t* perm, const float4* pos_in, const uint4* vfme_in,
                          float4* spos, uint4* svfme, uint4* bands, uint32_t N, cudaStream_t st, bool pdl,
                          uint32_t per_thread) {
    cudaError_t e;
    if (n) {
        const uint32_t per = per_thread == 4u ? 4u : (per_thread == 2u ? 2u : 1u);
        const uint32_t blocks = std::min<uint32_t>((n + 256u * per - 1u) / (256u * per),
                                                   (uint32_t)device_sm_count() * 8u);
        auto* kern = per == 4u ? k_cell_scatter<4> : (per == 2u ? k_cell_scatter<2> : k_cell_scatter<1>);
        if ((e = launch_pdl(pdl, kern, dim3(blocks), dim3(256), 0, st, keys, n, s.hist, perm, pos_in, vfme_in, spos,
                            svfme, offs, bands, N, s.fix_bits)))
            return e;
    }
    const OneBuffer src{pos_in, vfme_in};
    return launch_pdl(pdl && n, k_fix_marked<OneBuffer>, dim3(fix_grid(n)),
                      dim3(kCollectThreads), 0, st, (const uint32_t*)s.fix_bits, keys, n, offs, perm, fix_lists(s),
                      s.fix_tmp, src, spos, svfme, s.hist, cells, s.coarse, scan_tiles(cells),
                      (const uint32_t*)nullptr, std::max(collect_grid(n), 1u));
}

cudaError_t count_scan_scenes(CountScratch& s, const SceneDev* scenes, const uint32_t* cell_tile_scene,
                              uint32_t cells, uint32_t* offs, cudaStream_t st, uint32_t* far_reset) {
    const uint32_t chunks = (cells + kScanChunk - 1u) / kScanChunk;
    k_cell_scan<true><<<chunks, kScanThreads, 0, st>>>(s.hist, s.coarse, cells, offs, s.fix_ctl, scenes,
                                                      cell_tile_scene, far_reset);
    return cudaGetLastError();
}

cudaError_t count_rank_scenes(CountScratch& s, const SceneDev* scenes, const uint32_t* tile_scene,
                              const uint32_t* cell_tile_scene, const uint32_t* keys, uint32_t n, uint32_t cells,
                              const uint32_t* offs, const uint32_t* offs_old, const uint32_t* far, uint32_t* perm,
                              const float4* pos_buf0, const float4* pos_buf1, const uint4* vfme_buf0,
                              const uint4* vfme_buf1, float4* spos, uint4* svfme, uint4* bands, cudaStream_t st) {
    cudaError_t e;
    if (n) {
        k_cell_rank_scenes<<<(n + kRankThreads - 1u) / kRankThreads, kRankThreads, 0, st>>>(
            scenes, tile_scene, keys, n, s.hist, perm, pos_buf0,
                                                              pos_buf1, vfme_buf0, vfme_buf1, spos, svfme, offs,
                                                              offs_old, far, s.fix_bits, bands);
        if ((e = cudaGetLastError())) return e;
    }
    const SceneBuffers src{scenes, tile_scene, cell_tile_scene, pos_buf0, pos_buf1, vfme_buf0, vfme_buf1, false};
    k_fix_marked<SceneBuffers><<<fix_grid(n), kCollectThreads, 0, st>>>(
        s.fix_bits, keys, n, offs, perm, fix_lists(s), s.fix_tmp, src, spos, svfme, s.hist, cells, s.coarse,
        scan_tiles(cells), far, std::max(collect_grid(n), 1u));
    return cudaGetLastError();
}

cudaError_t count_scatter_scenes(CountScratch& s, const SceneDev* scenes, const uint32_t* tile_scene,
                                 const uint32_t* cell_tile_scene, const uint32_t* keys, uint32_t n, uint32_t cells,
                                 const uint32_t* offs, uint32_t* perm, const float4* pos_buf0,
                                 const float4* pos_buf1, const uint4* vfme_buf0, const uint4* vfme_buf1,
                                 float4* spos, uint4* svfme, uint4* bands, cudaStream_t st, uint32_t per_thread,
                                 bool may_init) {
    cudaError_t e;
    if (n) {
        const uint32_t per = per_thread == 4u ? 4u : (per_thread == 2u ? 2u : 1u);
        const uint32_t blocks = std::min<uint32_t>((n + 256u * per - 1u) / (256u * per),
                                                   (uint32_t)device_sm_count() * 8u);
        auto* kern = per == 4u ? k_cell_scatter_scenes<4>
                               : (per == 2u ? k_cell_scatter_scenes<2> : k_cell_scatter_scenes<1>);
        kern<<<blocks, 256, 0, st>>>(scenes, tile_scene, keys, n, s.hist, perm, pos_buf0, pos_buf1, vfme_buf0,
                                     vfme_buf1, spos, svfme, offs, s.fix_bits, bands);
        if ((e = cudaGetLastError())) return e;
    }
    const SceneBuffers src{scenes, tile_scene, cell_tile_scene, pos_buf0, pos_buf1, vfme_buf0, vfme_buf1, may_init};
    k_fix_marked<SceneBuffers><<<fix_grid(n), kCollectThreads, 0, st>>>(
        s.fix_bits, keys, n, offs, perm, fix_lists(s), s.fix_tmp, src, spos, svfme, s.hist, cells, s.coarse,
        scan_tiles(cells), nullptr, std::max(collect_grid(n), 1u));
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
