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
//      offs[c] (= start of cell c; offs[C] = n) and a cursor copy, and zeroes the
//      counts; each 4096-cell tile takes its base from per-tile counts emitted
//      with the per-cell ones, so tiles never wait on each other;
//   3. k_cell_scatter: each sphere claims a slot of its cell with one atomic per
//      run of equal keys in its warp (match.any), so spheres of one warp keep
//      their order, and its 32-byte state is copied to that slot;
//   4. k_cell_fixup: every cell's slots are put back in ascending input order
//      (what a stable sort yields; only cells filled by several warps need it),
//      re-gathering the state copy of the cells it reorders.
//
// The result is bit-identical to a stable sort; offs[] replaces start/close.

#include <cuda_runtime.h>

#include <algorithm>

#include "mb_internal.h"

namespace mb {
namespace {

// ---------------------------------------------------------------- scan
// Tile t of the scan covers cells [4096 t, 4096 t + 4096).  coarse[t] holds the
// number of spheres in those cells (emitted with the per-cell counts), so a tile
// finds its base by summing coarse[0..t) - no look-back, no waiting on other tiles.
//
// kScenes (a batch): every scene's cell range is padded to whole tiles, so a tile
// belongs to one scene; its base is that scene's first slot plus the coarse
// counts of the scene's earlier tiles, and tiles of HOLD scenes are left alone.
template <bool kScenes>
__global__ void __launch_bounds__(kScanThreads)
    k_cell_scan(uint32_t* __restrict__ hist, const uint32_t* __restrict__ coarse, uint32_t cells,
                uint32_t* __restrict__ offs, uint32_t* __restrict__ cursor, uint32_t* big_ctl,
                const SceneDev* __restrict__ scenes, const uint32_t* __restrict__ cell_tile_scene) {
    constexpr int W = kScanThreads / 32;
    __shared__ uint32_t s_warp[W], s_base[W];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t tile = blockIdx.x;
    if (tile == 0 && tid < 2) big_ctl[tid] = 0u;  // big-cell list of this frame starts empty
    const uint32_t base = tile * kScanTile + tid * kScanItems;

    uint32_t first_tile = 0, base_slot = 0;
    if (kScenes) {
        const uint32_t sc = __ldg(cell_tile_scene + tile);
        if (__ldg(&scenes[sc].mode) == kModeHold) return;
        first_tile = __ldg(&scenes[sc].cell_base) / kScanTile;
        base_slot = __ldg(&scenes[sc].agent_base);
    }
    // exclusive base of this tile: sum of the coarse counts of the earlier tiles
    uint32_t bsum = 0;
    for (uint32_t t = first_tile + tid; t < tile; t += kScanThreads) bsum += __ldg(coarse + t);

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
        uint4* c4 = reinterpret_cast<uint4*>(cursor + base);
        uint4* h4 = reinterpret_cast<uint4*>(hist + base);
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            uint4 x;
            x.x = run; run += v[4 * q];
            x.y = run; run += v[4 * q + 1];
            x.z = run; run += v[4 * q + 2];
            x.w = run; run += v[4 * q + 3];
            o4[q] = x;
            c4[q] = x;
            h4[q] = make_uint4(0u, 0u, 0u, 0u);
        }
        // end of the tile: the next tile's first offset, or the scene's / table's end
        if (base + kScanItems == cells || (kScenes && tid == kScanThreads - 1)) offs[base + kScanItems] = run;
    } else {
        for (int q = 0; q < kScanItems; ++q) {
            uint32_t c = base + q;
            if (c < cells) {
                offs[c] = run;
                cursor[c] = run;
                hist[c] = 0u;
                run += v[q];
                if (c + 1u == cells) offs[cells] = run;
            }
        }
    }
}

// ---------------------------------------------------------------- scatter
// Also moves each sphere's state to its slot (sorted copy for the physics pass)
// and, where a slot begins or ends a physics tile, writes that side of the
// tile's band table entry (the cell of a slot is final here; the fixup only
// reorders slots inside a cell).
__global__ void __launch_bounds__(256)
    k_cell_scatter(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ cursor,
                   uint32_t* __restrict__ perm, const float4* __restrict__ pos_in,
                   const uint4* __restrict__ vfme_in, float4* __restrict__ spos,
                   uint4* __restrict__ svfme, const uint32_t* __restrict__ offs, uint4* __restrict__ bands,
                   uint32_t N) {
    const uint32_t lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        uint32_t i = i0 + threadIdx.x;
        bool valid = i < n;
        uint32_t k = valid ? __ldg(keys + i) : 0xFFFFFFFFu;
        float4 p;
        uint4 q;
        if (valid) {
            p = __ldg(pos_in + i);
            q = __ldg(vfme_in + i);
        }
        // a key flagged kInitKeyBit belongs to a scene in its INIT frame: all its
        // keys are equal, so its stable order is the identity and the slot is i
        const bool ident = valid && (k & kInitKeyBit);
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, ident ? 0xFFFFFFFEu : k);
        uint32_t leader = (uint32_t)(__ffs(peers) - 1);
        uint32_t b = 0;
        if (valid && !ident && lane == leader) b = atomicAdd(cursor + k, (uint32_t)__popc(peers));
        b = __shfl_sync(0xFFFFFFFFu, b, (int)leader);
        if (valid) {
            const uint32_t dst = ident ? i : b + (uint32_t)__popc(peers & lt);
            perm[dst] = i;
            spos[dst] = p;
            svfme[dst] = q;
            if (bands && !ident) write_band_bounds(bands, offs, N, n, dst, k);
        }
    }
}

// The same for a batch: slot i's scene (from the tile table) gives the buffer
// holding its state; spheres of HOLD scenes are left alone.
__global__ void __launch_bounds__(256)
    k_cell_scatter_scenes(const SceneDev* __restrict__ scenes, const uint32_t* __restrict__ tile_scene,
                          const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ cursor,
                          uint32_t* __restrict__ perm, const float4* __restrict__ pos0,
                          const float4* __restrict__ pos1, const uint4* __restrict__ vfme0,
                          const uint4* __restrict__ vfme1, float4* __restrict__ spos, uint4* __restrict__ svfme) {
    const uint32_t lane = threadIdx.x & 31u, lt = (1u << lane) - 1u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += stride) {
        uint32_t i = i0 + threadIdx.x;
        bool valid = i < n;
        uint32_t mode = kModeHold, parity = 0;
        if (valid) {
            uint32_t s = __ldg(tile_scene + i / kPhysicsTile);
            while (i >= __ldg(&scenes[s].agent_end)) ++s;
            mode = __ldg(&scenes[s].mode);
            parity = __ldg(&scenes[s].parity);
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
        if (valid && !ident && lane == leader) b = atomicAdd(cursor + k, (uint32_t)__popc(peers));
        b = __shfl_sync(0xFFFFFFFFu, b, (int)leader);
        if (valid) {
            const uint32_t dst = ident ? i : b + (uint32_t)__popc(peers & lt);
            perm[dst] = i;
            spos[dst] = p;
            svfme[dst] = q;
        }
    }
}

// ---------------------------------------------------------------- fixup
// Cells of up to kSmallCell slots are re-sorted by their own thread (insertion
// sort, after a sortedness check); larger ones go to a list for k_cell_fixup_big.
// A cell whose order changes re-gathers its sorted state copy from the state
// source: one buffer (a world), or each scene's current buffer (a batch, where
// cells and coarse tiles of HOLD scenes are left alone).
constexpr uint32_t kSmallCell = 32;
constexpr uint32_t kBlockSortMax = 8192;

struct OneBuffer {
    const float4* p;
    const uint4* q;
    __device__ __forceinline__ bool tile_active(uint32_t) const { return true; }
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
    __device__ __forceinline__ uint32_t parity(uint32_t o) const {
        uint32_t s = __ldg(slot_tile_scene + o / kPhysicsTile);
        while (o >= __ldg(&scenes[s].agent_end)) ++s;
        return __ldg(&scenes[s].parity);
    }
    __device__ __forceinline__ float4 pos(uint32_t o) const { return __ldg((parity(o) ? p1 : p0) + o); }
    __device__ __forceinline__ uint4 vfme(uint32_t o) const { return __ldg((parity(o) ? q1 : q0) + o); }
};

template <class Src>
__global__ void __launch_bounds__(256)
    k_cell_fixup(const uint32_t* __restrict__ offs, uint32_t cells, uint32_t* perm, uint32_t* coarse,
                 uint32_t tiles, uint32_t* big_ctl, uint32_t* big, Src src, float4* __restrict__ spos,
                 uint4* __restrict__ svfme) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x == 0)  // the scan of this frame is over: clear the tile counts for the next one
        for (uint32_t t = threadIdx.x; t < tiles; t += blockDim.x)
            if (src.tile_active(t)) coarse[t] = 0u;
    if (c >= cells || !src.tile_active(c / kScanTile)) return;
    const uint32_t lo = offs[c], hi = offs[c + 1u];
    if (hi - lo < 2u) return;
    if (hi - lo > kSmallCell) {
        big[atomicAdd(big_ctl, 1u)] = c;
        return;
    }
    bool sorted = true;
    uint32_t prev = perm[lo];
    for (uint32_t j = lo + 1u; j < hi; ++j) {
        uint32_t x = perm[j];
        if (x < prev) { sorted = false; break; }
        prev = x;
    }
    if (sorted) return;
    for (uint32_t a = lo + 1u; a < hi; ++a) {  // insertion sort of this cell's slots
        uint32_t x = perm[a];
        uint32_t b = a;
        while (b > lo) {
            uint32_t y = perm[b - 1u];
            if (y <= x) break;
            perm[b] = y;
            --b;
        }
        perm[b] = x;
    }
    for (uint32_t j = lo; j < hi; ++j) {  // the sorted state copy follows the new order
        const uint32_t o = perm[j];
        spos[j] = src.pos(o);
        svfme[j] = src.vfme(o);
    }
}

__device__ void heap_sift(uint32_t* a, uint32_t root, uint32_t end) {
    while (true) {
        uint32_t child = 2u * root + 1u;
        if (child >= end) return;
        if (child + 1u < end && a[child + 1u] > a[child]) ++child;
        if (a[root] >= a[child]) return;
        uint32_t t = a[root];
        a[root] = a[child];
        a[child] = t;
        root = child;
    }
}

// One block per listed cell: bitonic sort in shared memory (up to kBlockSortMax
// slots), else an O(m log m) heapsort in place by one thread (only degenerate
// scenes with thousands of spheres in one cell get there).
template <class Src>
__global__ void __launch_bounds__(256)
    k_cell_fixup_big(const uint32_t* __restrict__ offs, uint32_t* perm, uint32_t* big_ctl,
                     const uint32_t* __restrict__ big, Src src, float4* __restrict__ spos,
                     uint4* __restrict__ svfme) {
    __shared__ uint32_t s_v[kBlockSortMax];
    __shared__ uint32_t s_idx, s_unsorted;
    const uint32_t tid = threadIdx.x;
    while (true) {
        if (tid == 0) {
            s_idx = atomicAdd(big_ctl + 1, 1u);
            s_unsorted = 0u;
        }
        __syncthreads();
        const uint32_t idx = s_idx;
        if (idx >= __ldcg(big_ctl)) return;
        const uint32_t c = __ldg(big + idx);
        const uint32_t lo = offs[c], m = offs[c + 1u] - lo;
        for (uint32_t j = tid + 1u; j < m; j += blockDim.x)
            if (perm[lo + j] < perm[lo + j - 1u]) s_unsorted = 1u;
        __syncthreads();
        if (s_unsorted) {
            if (m <= kBlockSortMax) {
                uint32_t P = 2u;
                while (P < m) P <<= 1;
                for (uint32_t j = tid; j < P; j += blockDim.x) s_v[j] = j < m ? perm[lo + j] : 0xFFFFFFFFu;
                __syncthreads();
                for (uint32_t k = 2u; k <= P; k <<= 1) {
                    for (uint32_t jj = k >> 1; jj > 0u; jj >>= 1) {
                        for (uint32_t i = tid; i < P; i += blockDim.x) {
                            uint32_t ixj = i ^ jj;
                            if (ixj > i) {
                                uint32_t a = s_v[i], b = s_v[ixj];
                                bool up = (i & k) == 0u;
                                if ((a > b) == up) {
                                    s_v[i] = b;
                                    s_v[ixj] = a;
                                }
                            }
                        }
                        __syncthreads();
                    }
                }
                for (uint32_t j = tid; j < m; j += blockDim.x) perm[lo + j] = s_v[j];
            } else if (tid == 0) {
                uint32_t* a = perm + lo;
                for (uint32_t r = m / 2u; r-- > 0u;) heap_sift(a, r, m);
                for (uint32_t end = m - 1u; end > 0u; --end) {
                    uint32_t t = a[0];
                    a[0] = a[end];
                    a[end] = t;
                    heap_sift(a, 0u, end);
                }
            }
            __syncthreads();
            for (uint32_t j = tid; j < m; j += blockDim.x) {  // sorted state copy follows
                const uint32_t o = perm[lo + j];
                spos[lo + j] = src.pos(o);
                svfme[lo + j] = src.vfme(o);
            }
        }
        __syncthreads();
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

cudaError_t count_scratch_alloc(CountScratch& s, uint32_t max_cells) {
    s.max_cells = max_cells;
    size_t padded = ((size_t)max_cells + kScanTile) & ~(size_t)15;  // uint4-aligned, room for offs[C]
    s.tiles = (max_cells + kScanTile - 1u) / kScanTile;
    cudaError_t e;
    if ((e = cudaMalloc(&s.hist, sizeof(uint32_t) * padded))) return e;
    if ((e = cudaMalloc(&s.cursor, sizeof(uint32_t) * padded))) return e;
    if ((e = cudaMalloc(&s.coarse, sizeof(uint32_t) * (s.tiles + 1u)))) return e;
    if ((e = cudaMalloc(&s.big_ctl, sizeof(uint32_t) * 2u))) return e;
    if ((e = cudaMalloc(&s.big, sizeof(uint32_t) * ((size_t)max_cells + 1u)))) return e;
    if ((e = cudaMemset(s.hist, 0, sizeof(uint32_t) * padded))) return e;
    if ((e = cudaMemset(s.coarse, 0, sizeof(uint32_t) * (s.tiles + 1u)))) return e;
    if ((e = cudaMemset(s.big_ctl, 0, sizeof(uint32_t) * 2u))) return e;
    return cudaSuccess;
}

void count_scratch_free(CountScratch& s) {
    cudaFree(s.hist);
    cudaFree(s.cursor);
    cudaFree(s.coarse);
    cudaFree(s.big_ctl);
    cudaFree(s.big);
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

cudaError_t count_scan(CountScratch& s, uint32_t* ctl, uint32_t cells, uint32_t* offs, cudaStream_t st) {
    (void)ctl;
    uint32_t tiles = (cells + kScanTile - 1u) / kScanTile;
    k_cell_scan<false><<<tiles, kScanThreads, 0, st>>>(s.hist, s.coarse, cells, offs, s.cursor, s.big_ctl,
                                                       nullptr, nullptr);
    return cudaGetLastError();
}

cudaError_t count_scatter(CountScratch& s, const uint32_t* keys, uint32_t n, uint32_t cells,
                          const uint32_t* offs, uint32_t* perm, const float4* pos_in, const uint4* vfme_in,
                          float4* spos, uint4* svfme, uint4* bands, uint32_t N, cudaStream_t st) {
    cudaError_t e;
    if (n) {
        uint32_t blocks = std::min<uint32_t>((n + 255u) / 256u, (uint32_t)device_sm_count() * 8u);
        k_cell_scatter<<<blocks, 256, 0, st>>>(keys, n, s.cursor, perm, pos_in, vfme_in, spos, svfme, offs, bands,
                                               N);
        if ((e = cudaGetLastError())) return e;
    }
    uint32_t tiles = (cells + kScanTile - 1u) / kScanTile;
    OneBuffer src{pos_in, vfme_in};
    k_cell_fixup<OneBuffer><<<(cells + 255u) / 256u, 256, 0, st>>>(offs, cells, perm, s.coarse, tiles, s.big_ctl,
                                                                   s.big, src, spos, svfme);
    if ((e = cudaGetLastError())) return e;
    k_cell_fixup_big<OneBuffer><<<(uint32_t)device_sm_count(), 256, 0, st>>>(offs, perm, s.big_ctl, s.big, src,
                                                                             spos, svfme);
    return cudaGetLastError();
}

cudaError_t count_scan_scenes(CountScratch& s, const SceneDev* scenes, const uint32_t* cell_tile_scene,
                              uint32_t cells, uint32_t* offs, cudaStream_t st) {
    uint32_t tiles = (cells + kScanTile - 1u) / kScanTile;
    k_cell_scan<true><<<tiles, kScanThreads, 0, st>>>(s.hist, s.coarse, cells, offs, s.cursor, s.big_ctl, scenes,
                                                      cell_tile_scene);
    return cudaGetLastError();
}

cudaError_t count_scatter_scenes(CountScratch& s, const SceneDev* scenes, const uint32_t* tile_scene,
                                 const uint32_t* cell_tile_scene, const uint32_t* keys, uint32_t n, uint32_t cells,
                                 const uint32_t* offs, uint32_t* perm, const float4* pos_buf0,
                                 const float4* pos_buf1, const uint4* vfme_buf0, const uint4* vfme_buf1,
                                 float4* spos, uint4* svfme, cudaStream_t st) {
    cudaError_t e;
    if (n) {
        uint32_t blocks = std::min<uint32_t>((n + 255u) / 256u, (uint32_t)device_sm_count() * 8u);
        k_cell_scatter_scenes<<<blocks, 256, 0, st>>>(scenes, tile_scene, keys, n, s.cursor, perm, pos_buf0,
                                                      pos_buf1, vfme_buf0, vfme_buf1, spos, svfme);
        if ((e = cudaGetLastError())) return e;
    }
    uint32_t tiles = (cells + kScanTile - 1u) / kScanTile;
    SceneBuffers src{scenes, tile_scene, cell_tile_scene, pos_buf0, pos_buf1, vfme_buf0, vfme_buf1};
    k_cell_fixup<SceneBuffers><<<(cells + 255u) / 256u, 256, 0, st>>>(offs, cells, perm, s.coarse, tiles,
                                                                      s.big_ctl, s.big, src, spos, svfme);
    if ((e = cudaGetLastError())) return e;
    k_cell_fixup_big<SceneBuffers><<<(uint32_t)device_sm_count(), 256, 0, st>>>(offs, perm, s.big_ctl, s.big,
                                                                                src, spos, svfme);
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
