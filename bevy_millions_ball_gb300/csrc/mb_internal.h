// mb_internal.h — host-side interfaces between the library's translation units.
#pragma once

#include <nvtx3/nvToolsExt.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/millionsball.h"

namespace mb {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr int kMaxPasses = 4;
constexpr uint32_t kMaxDigitBits = 11;
constexpr uint32_t kMaxRadix = 1u << kMaxDigitBits;
constexpr uint32_t kMaxAgents = (1u << 28) - 1u;   // look-back words keep 28 value bits
constexpr uint32_t kMaxCells = 1u << 28;
// Flag on a cell key of a batched scene in its INIT frame (keys are < 2^28).
constexpr uint32_t kInitKeyBit = 0x80000000u;

// Onesweep tile shape: 256 threads x 16 keys.
#ifndef MB_SORT_ITEMS
#define MB_SORT_ITEMS 16
#endif
constexpr int kSortThreads = 256;
constexpr int kSortItems = MB_SORT_ITEMS;
constexpr uint32_t kSortTile = kSortThreads * kSortItems;

// Control words of a sort plan (device u32 array).
enum : int {
    kCtlTile0 = 0,                // [kMaxPasses] tile tickets
    kCtlDone = kMaxPasses,        // histogram blocks finished
    kCtlError = kMaxPasses + 1,   // nonzero: a bounded wait gave up
    kCtlEpoch = kMaxPasses + 2,   // look-back epoch of the running sort (1..3)
    kCtlGaps = kMaxPasses + 3,    // long cell gaps listed by the cell-offset build
    kCtlWords = 8
};

// Digit schedule of one sort: LSD first; the last (most significant) digit is
// also the chunking of the cell-offset build.
struct SortSchedule {
    uint32_t n = 0;
    uint32_t cells = 0;
    uint32_t total_bits = 0;
    int passes = 0;
    uint32_t shift[kMaxPasses] = {0, 0, 0, 0};
    uint32_t bits[kMaxPasses] = {0, 0, 0, 0};
    uint32_t tiles = 0;
};

SortSchedule make_schedule(uint32_t n, uint32_t cells, uint32_t digit_bits_max);

// Device scratch of the sort + cell-offset build, sized for (max_keys, max_cells).
struct SortScratch {
    uint32_t max_keys = 0;
    uint32_t max_cells = 0;
    uint32_t* alt_keys = nullptr;   // [max_keys]
    uint32_t* alt_vals = nullptr;   // [max_keys]
    uint32_t* counts = nullptr;     // [kMaxPasses][kMaxRadix]   digit counts, zero between sorts
    uint32_t* bases = nullptr;      // [kMaxPasses][kMaxRadix+1] exclusive digit bases
    uint32_t* lookback = nullptr;   // [kMaxPasses][tiles_max * kMaxRadix]
    uint32_t* ctl = nullptr;        // [kCtlWords]
    uint32_t* offs = nullptr;       // [max_cells + 1] cell offsets (CSR)
    uint32_t* gaps = nullptr;       // [3 * gap_capacity(max_cells)] long runs of cells to fill
    size_t lookback_words_per_pass = 0;
    // layout of the previous sort's look-back words (reuse check): a table is
    // reused only when the previous sort wrote every word this one reads
    uint32_t last_tiles = 0;
    int last_passes = 0;
    uint32_t last_bits[kMaxPasses] = {0, 0, 0, 0};
};

// Runs of more than kGapCells cells between consecutive sorted keys are written
// by a fill kernel from a list instead of by one thread each.
constexpr uint32_t kGapCells = 64;
inline uint32_t gap_capacity(uint32_t max_cells) { return max_cells / kGapCells + 2u; }
cudaError_t scratch_alloc(SortScratch& s, uint32_t max_keys, uint32_t max_cells);
void scratch_free(SortScratch& s);

// Stable sort of (keys, vals or iota) -> (sorted_keys, sorted_vals).
// clear_always: clear the look-back words this sort uses on the stream every
// call instead of tracking the previous sort's layout on the host (for scratch
// that calls recorded into graphs may replay in any order).
cudaError_t sort_pairs(SortScratch& s, const SortSchedule& sch, const uint32_t* keys,
                       const uint32_t* vals, uint32_t* sorted_keys, uint32_t* sorted_vals,
                       cudaStream_t st, bool clear_always = false);
// Reads and clears the scratch's error word (synchronises the stream first):
// *flags != 0 when a bounded look-back wait gave up since the last read.  A
// give-up also forces the next sort to start from a cleared look-back table.
cudaError_t sort_take_error(SortScratch& s, cudaStream_t st, uint32_t* flags);
// Test hook: one onesweep block takes tile 1 of a pass whose tile 0 never
// publishes its look-back words, so its wait runs out after spin_limit polls and
// sets the error word; nothing else is written.  The next sort clears the table.
cudaError_t sort_stall_for_test(SortScratch& s, uint32_t spin_limit, cudaStream_t st);
// Cell offsets offs[c] = number of keys < c for c in [0, cells], from the sorted
// keys and the most significant digit's bases of the sort that produced them.
cudaError_t cell_offsets(SortScratch& s, const SortSchedule& sch, const uint32_t* sorted_keys,
                         cudaStream_t st);

// start/close tables (spatial_hashing.wgsl semantics) from cell offsets.
// start/close (nullable) of every cell straight from the sorted keys: 0xFFFFFFFF
// for empty cells, else the first / last slot of the cell's run.
// (scratch: its gap list, whose counter the sort's histogram cleared)
cudaError_t hash_ranges(SortScratch& s, const uint32_t* sorted_keys, uint32_t n, uint32_t cells, uint32_t* start,
                        uint32_t* close, cudaStream_t st);
cudaError_t offsets_to_start_close(const uint32_t* offs, uint32_t cells, uint32_t* start,
                                   uint32_t* close, cudaStream_t st);

// Physics constants as kernel parameters.
struct PhysParams {
    uint32_t N;
    uint32_t grid_size;
    float half_map_size;
    float half_map_height;
    float gx, gy, gz;
    float e_envir, e_agent, k_agent, c_agent, r_agent, dt;
    float neg_c_over_dt;      // -C_AGENT / T_DELTA
    float neg_1pe_over_dt;    // -(1 + E_ENVIR) / T_DELTA
    uint32_t spring;
    uint32_t div_m, div_s1, div_s2;  // exact n / grid_size by multiply-shift
};

PhysParams make_params(const mb_consts& c);

// One scene of a batch (many scenes in one flattened key space).
enum : uint32_t { kModeHold = 0, kModeInit = 1, kModeLoop = 2 };
struct SceneDev {
    PhysParams P;
    uint32_t agent_base, agent_end;  // sorted slots [agent_base, agent_end)
    uint32_t cell_base;              // cells [cell_base, cell_base + N*N)
    uint32_t mode;                   // kModeHold / kModeInit / kModeLoop
    uint32_t parity;                 // which state buffer holds the scene's current state
    uint32_t pad[3];
};
constexpr uint32_t kPhysicsTile = 128;  // slots per block of the physics pass

// Band table of the physics pass: for physics tile t (sorted slots
// [t*kPhysicsTile, t*kPhysicsTile + kPhysicsTile)), bands[2t] = lower and
// bands[2t+1] = upper slot bounds of its three candidate bands (x: row below,
// y: own row, z: row above), each covering the tile's cells one column to either
// side.  The sort writes it while it places the slots: the thread that places
// a tile's first slot writes the lower bounds (from that slot's cell kf), the
// one that places its last slot the upper bounds (from its cell kl).  A band
// whose upper bound is not above its lower bound is empty.
inline uint32_t band_table_entries(uint32_t n) { return 2u * ((n + kPhysicsTile - 1u) / kPhysicsTile); }
#ifdef __CUDACC__
// Programmatic dependent launch.  A kernel launched with launch_pdl may start
// while the kernel before it on the stream is still finishing; it calls
// griddep_wait() before it touches memory that kernel writes (the wait returns
// once that kernel has completed and its writes are visible; without a
// programmatic predecessor it returns at once).  griddep_launch() lets the next
// kernel start launching.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1u : 0u;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Load of data the running kernel does not write.  kCg: the data may have been
// written earlier in the same launch (the fused frame kernel, whose stages are
// separated by grid barriers, not kernel boundaries), so it is read from L2
// (ld.global.cg) instead of through the non-coherent read-only path.
template <bool kCg, typename T>
__device__ __forceinline__ T ld_in(const T* p) {
    if constexpr (kCg)
        return __ldcg(p);
    else
        return __ldg(p);
}

// Load of data that an earlier stage wrote: a plain load after a kernel
// boundary; from L2 (ld.global.cg) inside the fused frame kernel (kCg).
template <bool kCg, typename T>
__device__ __forceinline__ T ld_cur(const T* p) {
    if constexpr (kCg)
        return __ldcg(p);
    else
        return *p;
}

template <bool kCg = false>
__device__ __forceinline__ void write_band_bounds(uint4* __restrict__ bands, const uint32_t* __restrict__ offs,
                                                  uint32_t N, uint32_t n, uint32_t slot, uint32_t key) {
    const uint32_t r = slot % kPhysicsTile;
    const bool first = r == 0u, last = r == kPhysicsTile - 1u || slot + 1u == n;
    if (!first && !last) return;
    const uint32_t t = slot / kPhysicsTile;
    const uint32_t cx = key % N, top = N * (N - 1u);
    if (first) {
        const uint32_t l = cx > 0u ? 1u : 0u;
        const uint32_t f = max(key, N), lf = f % N > 0u ? 1u : 0u;  // row below: from column cx-1 of row cz-1
        bands[2u * t] = make_uint4(ld_in<kCg>(offs + f - N - lf), ld_in<kCg>(offs + key - l),
                                   key < top ? ld_in<kCg>(offs + key + N - l) : n, 0u);
    }
    if (last) {
        const uint32_t rr = cx < N - 1u ? 2u : 1u;
        const uint32_t a = min(key, top - 1u), ra = a % N < N - 1u ? 2u : 1u;  // row above: to column cx+1
        bands[2u * t + 1u] = make_uint4(key >= N ? ld_in<kCg>(offs + key - N + rr) : 0u, ld_in<kCg>(offs + key + rr),
                                        top ? ld_in<kCg>(offs + a + N + ra) : 0u, 0u);
    }
}
#endif

// Physics passes.  `hist` / `coarse` (nullable together) accumulate the per-cell
// and per-4096-cell-tile counts of the keys they emit, for the next frame's
// counting sort; the INIT pass and re-keying emit cell counts only (their tile
// counts come from count_tile_counts).
cudaError_t launch_physics_init(const PhysParams& p, uint32_t n, const uint32_t* perm,
                                const float4* pos_in, const uint4* vfme_in, float4* pos_out,
                                uint4* vfme_out, uint32_t* keys_out, uint32_t* hist, uint32_t* coarse,
                                cudaStream_t st);
// LOOP pass.  perm == NULL: spos/svfme hold the state in sorted order (slot j =
// sorted slot j, a copy the sort wrote); otherwise they hold it in the previous
// frame's slot order and sorted slot j is spos[perm[j]].  `bands` is the band
// table the sort wrote for this order.
// `pdl`: launched as a programmatic dependent of the kernel before it.  tile:
// slots per thread block (64, 128 or 256).
// far (nullable): the far-move list this pass fills for the next frame's rank
// placement (emptied by this frame's scan).
cudaError_t launch_physics_loop(const PhysParams& p, uint32_t n, const uint32_t* offs, const uint4* bands,
                                const float4* spos, const uint4* svfme, const uint32_t* perm, float4* pos_out,
                                uint4* vfme_out, uint32_t* keys_out, uint32_t* hist, uint32_t* coarse, uint32_t* err,
                                cudaStream_t st, bool pdl = false, uint32_t tile = kPhysicsTile,
                                uint32_t* far = nullptr);
// LOOP frames of one world as a single cooperative kernel (all stages of every
// frame, separated by grid barriers): `frames` frames from state buffer `cur`
// (the last one lands in cur ^ (frames & 1)), counting sort, sorted copy or
// (indirect) gather through perm.  bar: two zeroed words; err: the error word
// (bit 8: a grid barrier gave up).
struct CountScratch;
struct FusedFrame {
    PhysParams P;
    uint32_t n, cells, frames, cur;
    bool indirect;
    uint32_t* keys;
    uint32_t* offs;
    uint32_t* perm;
    uint4* bands;
    const CountScratch* cnt;
    float4* pos[2];
    uint4* vfme[2];
    float4* spos;
    uint4* svfme;
    uint32_t* bar;
    uint32_t* err;
};
cudaError_t launch_frame_fused(const FusedFrame& f, cudaStream_t st);
// Resident blocks per SM of the fused frame kernel (0: it cannot run).
int fused_blocks_per_sm();

// Compares the physics pass's division (div_exact) with IEEE division over
// `count` generated cases on the current device (synchronous).
cudaError_t selftest_divide(uint64_t seed, uint64_t count, uint64_t* mismatches, uint32_t* bad4);
cudaError_t launch_rekey(const PhysParams& p, uint32_t n, const float4* pos, uint32_t* keys,
                         uint32_t* hist, uint32_t* coarse, cudaStream_t st);

// Batched LOOP/INIT/HOLD pass: tile_scene[t] = scene of slot t*kPhysicsTile;
// `bands` is the band table the batched scatter wrote (used for tiles inside one
// LOOP scene).
// Batched physics: scene s reads the sorted copy and writes buffer 1 - parity
// (pos_buf[2] / vfme_buf[2]); a HOLD scene only re-emits the counts of its keys.
// far (nullable): the far-move list of the next frame's batched rank placement.
cudaError_t launch_physics_batch(const SceneDev* scenes, const uint32_t* tile_scene, uint32_t n,
                                 const uint32_t* offs, const uint4* bands, const float4* spos, const uint4* svfme,
                                 float4* pos_buf0,
                                 float4* pos_buf1, uint4* vfme_buf0, uint4* vfme_buf1, uint32_t* keys,
                                 uint32_t* hist, uint32_t* coarse, uint32_t* err, cudaStream_t st,
                                 uint32_t tile = kPhysicsTile, uint32_t* far = nullptr);


// Counting sort of cell keys (mb_count.cu).
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr uint32_t kScanChunk = kScanThreads * kScanItems;  // cells per block of the scan
constexpr uint32_t kScanTile = 4096;                        // cells per coarse count (tile base)
static_assert(kScanTile % kScanChunk == 0, "scan chunks tile the coarse tiles");

// Cells the scatter filled from several warp runs are marked (one bit per input
// slot); the fixup puts them back in order by size: up to kFixSmall slots (a
// thread each), up to kFixWarp (a warp each), larger (a block each).
constexpr uint32_t kFixSmall = 8;
constexpr uint32_t kFixWarp = 256;
// fix_ctl words: list lengths (cleared by each frame's scan), then a count of
// finished fixup blocks (kFixListDone: the last one resets it).  Only the list
// of cells above kFixWarp slots is filled.
enum : int { kFixListSmall = 0, kFixListWarp = 1, kFixListHuge = 2, kFixLists = 3, kFixListDone = 3, kFixCtlWords = 4 };

// Rank placement (MB_SORT_RANK).  Once a frame's input is the previous frame's
// sorted order, a sphere that moved at most one cell along x and z sits, in that
// input, inside the old 3 x 3 neighbourhood of its new cell, and so does every
// other such sphere of that cell: its slot is the cell's offset plus the number
// of spheres of its new cell that precede it there.  A sphere that moved
// further (a far move) is listed by the physics pass; up to kFarCap listed far
// moves are counted in from the list, more send the frame down the claim-and-
// fixup path.  A far list is a count word followed by kFarCap input slots.
constexpr uint32_t kFarCap = 256;
constexpr uint32_t kFarWords = 1u + kFarCap;
constexpr uint32_t kBloomWords = 128;  // per-block filter of the listed far moves' cells (4096 bits)

struct CountScratch {
    uint32_t max_cells = 0;
    uint32_t* hist = nullptr;     // [max_cells] counts of the keys of the next sort
    uint32_t* coarse = nullptr;   // [tiles] counts per 4096-cell scan tile
    uint32_t* fix_ctl = nullptr;  // [kFixCtlWords] lengths of the fixup lists, finished fixup blocks
    uint32_t* fix[kFixLists] = {nullptr, nullptr, nullptr};  // listed cells, by size class
    uint32_t fix_cap[kFixLists] = {0u, 0u, 0u};                // their capacities
    uint32_t* fix_tmp = nullptr;  // [max_keys] copy of a large cell's input indices
    uint32_t* fix_bits = nullptr; // [max_keys / 32 + 1] input slots whose run listed its cell
    uint32_t* offs_old = nullptr; // [max_cells + 1] second cell-offset buffer (rank placement alternates)
    uint32_t* far[2] = {nullptr, nullptr};  // [kFarWords] far-move lists, one per state parity
    uint32_t tiles = 0;
};
// Lists are sized from max_keys: a listed cell holds >= 2, > kFixSmall or > kFixWarp keys.
cudaError_t count_scratch_alloc(CountScratch& s, uint32_t max_cells, uint32_t max_keys);
uint64_t count_scratch_bytes(uint32_t max_cells, uint32_t max_keys);
void count_scratch_free(CountScratch& s);
// hist := 0, coarse := 0 for `cells` cells.
cudaError_t count_clear(CountScratch& s, uint32_t cells, cudaStream_t st);
// hist := counts of keys (rebuild, e.g. after an upload or a grid change).
cudaError_t count_keys(CountScratch& s, const uint32_t* keys, uint32_t n, uint32_t cells,
                       cudaStream_t st);
// hist := counts of n all-zero keys (a fresh upload).
cudaError_t count_reset_zero_keys(CountScratch& s, uint32_t n, uint32_t cells, cudaStream_t st);
// offs[0..cells] := exclusive scan of hist (offs[cells] = n); the scatter of
// count_scatter then counts hist back down to zero.
// far_reset (nullable): a far-move list emptied for this frame's physics pass.
cudaError_t count_scan(CountScratch& s, uint32_t* ctl, uint32_t cells, uint32_t* offs, cudaStream_t st,
                       bool pdl = false, uint32_t* far_reset = nullptr);
// coarse[t] := sum of hist over scan tile t (after a pass that emitted cell counts
// only: INIT frames, re-keying); the batched form touches only INIT scenes' tiles.
cudaError_t count_tile_counts(CountScratch& s, uint32_t cells, cudaStream_t st);
cudaError_t count_tile_counts_scenes(CountScratch& s, const SceneDev* scenes, const uint32_t* cell_tile_scene,
                                     uint32_t cells, cudaStream_t st);
// INIT frame after an upload (all keys 0): perm := identity, offs := [0, n, .., n], hist := 0.
cudaError_t count_init_order(CountScratch& s, uint32_t n, uint32_t cells, uint32_t* offs, uint32_t* perm,
                             cudaStream_t st);
// perm := stable permutation sorting keys by cell, from the offsets of count_scan
// and the counts in hist (counted back down to 0); spos/svfme (nullable
// together) := the state in that order (spos[j] = pos_in[perm[j]]); bands
// (nullable) := the band table of that order for an N x N grid; coarse := 0.
// per_thread: inputs each scatter thread takes per step (1, 2 or 4).
cudaError_t count_scatter(CountScratch& s, const uint32_t* keys, uint32_t n, uint32_t cells,
                          const uint32_t* offs, uint32_t* perm, const float4* pos_in, const uint4* vfme_in,
                          float4* spos, uint4* svfme, uint4* bands, uint32_t N, cudaStream_t st,
                          bool pdl = false, uint32_t per_thread = 1);
// Rank placement (MB_SORT_RANK).  count_rank: perm, the sorted copy and the
// band table from the ranks (offs: this frame's offsets, offs_old: the previous
// frame's, which describe this frame's input order; far: the far moves of the
// previous physics pass); when far holds more than kFarCap moves it claims slots
// and fixes cells as count_scatter does.  hist := 0, coarse := 0 either way.
// per_thread: spheres each thread places (1, 2 or 4).
cudaError_t count_rank(CountScratch& s, const uint32_t* keys, uint32_t n, uint32_t cells, const uint32_t* offs,
                       const uint32_t* offs_old, const uint32_t* far, uint32_t* perm, const float4* pos_in,
                       const uint4* vfme_in, float4* spos, uint4* svfme, uint4* bands, uint32_t N, cudaStream_t st,
                       bool pdl = false, uint32_t per_thread = 1);
// Allocates offs_old (the second cell-offset buffer that rank placement
// alternates with the world's own) and the far lists.
cudaError_t count_rank_alloc(CountScratch& s);
// Batched count scan: scene cell ranges are padded to whole scan tiles
// (cell_tile_scene[t] = scene of tile t); tiles of HOLD scenes are skipped.
cudaError_t count_scan_scenes(CountScratch& s, const SceneDev* scenes, const uint32_t* cell_tile_scene,
                              uint32_t cells, uint32_t* offs, cudaStream_t st, uint32_t* far_reset = nullptr);
// Batched rank placement, for frames in which every scene is in LOOP: offs /
// offs_old this frame's and the previous frame's pool-wide offsets, far the
// far moves of the previous batched physics pass (pool-wide slots); an
// overflowed list falls back to the batched scatter and fixup.
cudaError_t count_rank_scenes(CountScratch& s, const SceneDev* scenes, const uint32_t* tile_scene,
                              const uint32_t* cell_tile_scene, const uint32_t* keys, uint32_t n, uint32_t cells,
                              const uint32_t* offs, const uint32_t* offs_old, const uint32_t* far, uint32_t* perm,
                              const float4* pos_buf0, const float4* pos_buf1, const uint4* vfme_buf0,
                              const uint4* vfme_buf1, float4* spos, uint4* svfme, uint4* bands, cudaStream_t st);
// Batched scatter + fixup: like count_scatter, reading each scene's state from its
// parity buffer; spheres and cells of HOLD scenes are left alone.  may_init: a
// scene may be in its INIT frame (its cell counts are then cleared here).
cudaError_t count_scatter_scenes(CountScratch& s, const SceneDev* scenes, const uint32_t* tile_scene,
                                 const uint32_t* cell_tile_scene, const uint32_t* keys, uint32_t n, uint32_t cells,
                                 const uint32_t* offs, uint32_t* perm, const float4* pos_buf0,
                                 const float4* pos_buf1, const uint4* vfme_buf0, const uint4* vfme_buf1,
                                 float4* spos, uint4* svfme, uint4* bands, cudaStream_t st,
                                 uint32_t per_thread = 1, bool may_init = true);
// spos/svfme := pos_in/vfme_in gathered through perm (after the onesweep sort);
// bands (nullable) := the band table of the sorted keys for an N x N grid.
cudaError_t gather_state(const uint32_t* perm, uint32_t n, const float4* pos_in, const uint4* vfme_in,
                         float4* spos, uint4* svfme, const uint32_t* sorted_keys, const uint32_t* offs,
                         uint4* bands, uint32_t N, cudaStream_t st);

// Compacted segment table of sorted keys (mb_segs.cu): segs[s] = first slot of
// run s, key_seg_map[key] = s, *num_segs = runs (device pointers); block_scratch
// holds segment_blocks(n) words.
uint32_t segment_blocks(uint32_t n);
cudaError_t assemble_segments(const uint32_t* sorted_keys, uint32_t n, uint32_t* block_scratch, uint32_t* segs,
                              uint32_t* key_seg_map, uint32_t* num_segs, cudaStream_t st);

// Headless top-down impostor render of n spheres (mb_render.cu): w x h pixels
// over the x/z window [x0, x1) x [z0, z1); zbuf: w*h 64-bit scratch; rgba and
// height: w*h outputs on the device.
cudaError_t render_topdown(const float4* pos, uint32_t n, uint32_t w, uint32_t h, float x0, float z0, float x1,
                           float z1, unsigned long long* zbuf, uint32_t* rgba, float* height, cudaStream_t st);
// Perspective view (mb_render_view): eye and target (+y up), tan of half the
// vertical field of view, unit vector towards the light, the box |x|,|z| <=
// half_map_size, 0 <= y <= map_top; depth (nullable): distance along each
// pixel's ray (0: clear colour).
cudaError_t render_view(const float4* pos, uint32_t n, uint32_t w, uint32_t h, const float eye[3],
                        const float target[3], float tan_half_fov, const float to_light[3], float half_map_size,
                        float map_top, unsigned long long* zbuf, uint32_t* rgba, float* depth, cudaStream_t st);
// The reference view's constants (src/main.rs:65-89): camera (0, 64, 64) looking
// at the origin, Bevy's default vertical field of view (45 degrees), and the unit
// vector towards its directional light (rotation Euler ZYX (0, -0.15 pi,
// -0.15 pi) applied to -z, negated).
void reference_view(float eye[3], float target[3], float* fov_degrees, float to_light[3]);

// SM count of the current device (cached per device id).
int device_sm_count();

// Names the host-side span of a library call (NVTX range) for Nsight tools;
// without a tool attached the push and pop return at once.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Settings checks shared by worlds and batches ("" = valid).
bool settings_valid(const mb_settings* s, std::string& why);

// Sets the message mb_last_error(NULL) returns on this thread.
void set_process_error(const std::string& msg);

}  // namespace mb
