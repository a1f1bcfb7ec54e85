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
// run starts with a block-wide scan and writes its segments at its base.

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

__device__ __forceinline__ uint32_t block_sum(uint32_t v, uint32_t* s_w) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31u) == 0u) s_w[threadIdx.x >> 5] = v;
    __syncthreads();
    uint32_t t = 0;
    for (uint32_t w = 0; w < blockDim.x / 32u; ++w) t += s_w[w];
    __syncthreads();
    return t;
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

// Each thread owns kSegItems consecutive keys of the block's range.
__global__ void __launch_bounds__(kSegThreads)
    k_seg_count(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ block_counts) {
    __shared__ uint32_t s_w[kSegThreads / 32];
    const uint32_t first = blockIdx.x * kSegBlockKeys + threadIdx.x * kSegItems;
    uint32_t c = 0;
    for (uint32_t q = 0; q < kSegItems; ++q)
        if (first + q < n && run_start(keys, first + q)) ++c;
    const uint32_t t = block_sum(c, s_w);
    if (threadIdx.x == 0) block_counts[blockIdx.x] = t;
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
    const uint32_t first = blockIdx.x * kSegBlockKeys + threadIdx.x * kSegItems;
    uint32_t c = 0;
    for (uint32_t q = 0; q < kSegItems; ++q)
        if (first + q < n && run_start(keys, first + q)) ++c;
    uint32_t total;
    uint32_t s = __ldg(block_base + blockIdx.x) + block_excl(c, s_w, total);
    for (uint32_t q = 0; q < kSegItems; ++q) {
        const uint32_t i = first + q;
        if (i < n && run_start(keys, i)) {
            segs[s] = i;
            key_seg_map[__ldg(keys + i)] = s;
            ++s;
        }
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
