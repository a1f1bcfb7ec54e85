// mb_segs.cu — compacted segment table of sorted keys.
//
// The reference's segment assembly (src/physics/assemble_segs.rs:314-430,
// assemble_segs.wgsl) turns sorted keys into one entry per run of equal keys:
// segs[s] = first slot of segment s, key_seg_map[key] = s for every key that
// occurs, and the number of segments.  It is the compact alternative to
// per-cell start/close tables when cells far outnumber keys (sparse scenes).
//
// Three kernels: every block counts the run starts of its 4096 keys; one block
// scans the block counts (and writes the total); every block then recounts its
// run starts (per warp, in order, with ballots) and writes its segments at its
// base.  Warps read their keys in coalesced chunks of 32.

#include <cuda_runtime.h>

#include "mb_internal.h"

namespace mb {
namespace {

constexpr uint32_t kSegThreads = 256;
constexpr uint32_t kSegItems = 16;
constexpr uint32_t kSegBlockKeys = kSegThreads * kSegItems;

// key i of the block's range starts a run
__device__ __forceinline__ bool run_start(const uint32_t* __restrict__ keys, uint32_t i) {
    return i == 0u || __ldg(keys + i) != __ldg(keys + i - 1u);
}

// exclusive prefix over the block (thread order) of v; *total = block sum
__device__ __forceinline__ uint32_t block_excl(uint32_t v, uint32_t* s_w, uint32_t& total) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (lane == 31u) s_w[warp] = incl;
    __syncthreads();
    uint32_t base = 0, sum = 0;
    for (uint32_t w = 0; w < blockDim.x / 32u; ++w) {
        if (w < warp) base += s_w[w];
        sum += s_w[w];
    }
    __syncthreads();
    total = sum;
    return base + incl - v;
}

// A block covers kSegBlockKeys consecutive keys; warp w of it the kSegItems
// chunks of 32 keys starting at w * 32 * kSegItems, lane l key l of each chunk
// (coalesced loads).  run_flags returns, per lane, bit q = key l of chunk q starts
// a run, and the warp's number of run starts.
__device__ __forceinline__ uint32_t run_flags(const uint32_t* __restrict__ keys, uint32_t n, uint32_t wfirst,
                                              uint32_t& warp_total) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t flags = 0, total = 0;
#pragma unroll
    for (uint32_t q = 0; q < kSegItems; ++q) {
        const uint32_t i = wfirst + q * 32u + lane;
        const bool f = i < n && run_start(keys, i);
        flags |= (f ? 1u : 0u) << q;
        total += (uint32_t)__popc(__ballot_sync(0xFFFFFFFFu, f));
    }
    warp_total = total;
    return flags;
}

__global__ void __launch_bounds__(kSegThreads)
    k_seg_count(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ block_counts) {
    __shared__ uint32_t s_w[kSegThreads / 32];
    const uint32_t warp = threadIdx.x >> 5;
    uint32_t wt;
    run_flags(keys, n, blockIdx.x * kSegBlockKeys + warp * 32u * kSegItems, wt);
    if ((threadIdx.x & 31u) == 0u) s_w[warp] = wt;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (uint32_t w = 0; w < kSegThreads / 32u; ++w) t += s_w[w];
        block_counts[blockIdx.x] = t;
    }
}

// One block: exclusive scan of the block counts in place, total to *num_segs.
__global__ void __launch_bounds__(1024)
    k_seg_scan(uint32_t* __restrict__ block_counts, uint32_t blocks, uint32_t* __restrict__ num_segs) {
    __shared__ uint32_t s_w[32];
    uint32_t carry = 0;
    for (uint32_t b0 = 0; b0 < blocks; b0 += blockDim.x) {
        const uint32_t b = b0 + threadIdx.x;
        const uint32_t v = b < blocks ? block_counts[b] : 0u;
        uint32_t total;
        const uint32_t ex = block_excl(v, s_w, total);
        if (b < blocks) block_counts[b] = carry + ex;
        carry += total;
    }
    if (threadIdx.x == 0) *num_segs = carry;
}

__global__ void __launch_bounds__(kSegThreads)
    k_seg_assemble(const uint32_t* __restrict__ keys, uint32_t n, const uint32_t* __restrict__ block_base,
                   uint32_t* __restrict__ segs, uint32_t* __restrict__ key_seg_map) {
    __shared__ uint32_t s_w[kSegThreads / 32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, lt = (1u << lane) - 1u;
    const uint32_t wfirst = blockIdx.x * kSegBlockKeys + warp * 32u * kSegItems;
    uint32_t wt;
    const uint32_t flags = run_flags(keys, n, wfirst, wt);
    if (lane == 0u) s_w[warp] = wt;
    __syncthreads();
    uint32_t s = __ldg(block_base + blockIdx.x);  // the warp's first segment: block base + earlier warps
    for (uint32_t w = 0; w < warp; ++w) s += s_w[w];
#pragma unroll
    for (uint32_t q = 0; q < kSegItems; ++q) {
        const bool f = (flags >> q) & 1u;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, f);
        if (f) {
            const uint32_t i = wfirst + q * 32u + lane, at = s + (uint32_t)__popc(m & lt);
            segs[at] = i;
            key_seg_map[__ldg(keys + i)] = at;
        }
        s += (uint32_t)__popc(m);
    }
}

}  // namespace

uint32_t segment_blocks(uint32_t n) { return (n + kSegBlockKeys - 1u) / kSegBlockKeys; }

cudaError_t assemble_segments(const uint32_t* sorted_keys, uint32_t n, uint32_t* block_scratch, uint32_t* segs,
                              uint32_t* key_seg_map, uint32_t* num_segs, cudaStream_t st) {
    const uint32_t blocks = segment_blocks(n);
    cudaError_t e;
    if (blocks) {
        k_seg_count<<<blocks, kSegThreads, 0, st>>>(sorted_keys, n, block_scratch);
        if ((e = cudaGetLastError())) return e;
    }
    k_seg_scan<<<1, 1024, 0, st>>>(block_scratch, blocks, num_segs);
    if ((e = cudaGetLastError())) return e;
    if (blocks) {
        k_seg_assemble<<<blocks, kSegThreads, 0, st>>>(sorted_keys, n, block_scratch, segs, key_seg_map);
        if ((e = cudaGetLastError())) return e;
    }
    return cudaSuccess;
}

}  // namespace mb
