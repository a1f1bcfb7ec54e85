// mb_batch.cu — many independent scenes stepped by one set of launches per
// frame (batching), and a request-serving loop on top of it (serving).
//
// No counterpart in the reference, which runs one scene per app.  Layout: scene
// s owns sorted slots [agent_base, agent_base + n) and cells
// [cell_base, cell_base + N*N) of one flattened key space.  A frame is the same
// three stages as a single world's - count scan, scatter + fixup, physics - run
// once over all scenes: keys of different scenes never mix, so each scene's
// stable order, cell ranges and physics are exactly what it gets alone.  Each
// scene runs its own mode per frame (LOOP, INIT after an upload, or HOLD when
// it has no step to take); the per-scene table is a device buffer that the host
// rewrites between launches, so one captured graph per frame parity serves any
// mix of modes.

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "mb_internal.h"

namespace {

constexpr uint32_t kTile = mb::kPhysicsTile;

__global__ void k_fill_keys(uint32_t* keys, uint32_t n, uint32_t value) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) keys[i] = value;
}

// after a frame: every scene that ran now holds its state in the other buffer
__global__ void k_flip_parity(mb::SceneDev* scenes, uint32_t count) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < count && scenes[s].mode != mb::kModeHold) scenes[s].parity ^= 1u;
}

// cells of a scene are padded to whole scan tiles, so every tile has one scene
uint32_t padded_cells(uint64_t cells) {
    return (uint32_t)((cells + mb::kScanTile - 1u) / mb::kScanTile * mb::kScanTile);
}

// slot-local debug views of one scene
__global__ void k_local_debug(const uint32_t* keys, const uint32_t* perm, const uint32_t* offs, uint32_t n,
                              uint32_t cells, uint32_t agent_base, uint32_t cell_base, uint32_t* okeys,
                              uint32_t* operm, uint32_t* ostart, uint32_t* oclose) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        if (okeys) okeys[i] = (keys[agent_base + i] & ~mb::kInitKeyBit) - cell_base;
        if (operm) operm[i] = perm[agent_base + i] - agent_base;
    }
    if (i < cells) {
        uint32_t a = offs[cell_base + i], b = offs[cell_base + i + 1u];
        bool full = b > a;
        if (ostart) ostart[i] = full ? a - agent_base : mb::kInvalid;
        if (oclose) oclose[i] = full ? b - 1u - agent_base : mb::kInvalid;
    }
}

struct SceneHost {
    mb_settings s{};
    mb_consts c{};
    uint32_t agent_base = 0, n = 0, cell_base = 0, cells = 0;
    bool has_state = false;
    bool init_pending = false;
    bool active = true;
    bool frame_done = false;
    uint32_t parity = 0;   // state buffer holding the current state
    int64_t time = -1;
};

}  // namespace

struct mb_batch {
    uint32_t cap_agents = 0, cap_cells = 0, cap_scenes = 0;
    cudaStream_t stream = nullptr, cap_stream = nullptr;
    float4* pos[2] = {nullptr, nullptr};
    uint4* vfme[2] = {nullptr, nullptr};
    float4* spos = nullptr;
    uint4* svfme = nullptr;
    uint4* bands = nullptr;  // band table of the sorted order (written by the batched scatter)
    uint32_t *keys = nullptr, *perm = nullptr, *offs = nullptr, *ctl = nullptr, *d_tile_scene = nullptr;
    uint32_t* d_cell_tile_scene = nullptr;  // scene of each 4096-cell scan tile
    uint32_t* h_cell_tile_scene = nullptr;  // pinned
    mb::SceneDev* d_scenes = nullptr;
    mb::SceneDev* h_scenes = nullptr;     // pinned mirror of the scene table
    uint32_t* h_tile_scene = nullptr;     // pinned
    cudaEvent_t table_ev = nullptr;       // last table upload has been read
    mb::CountScratch cnt;
    std::vector<SceneHost> scenes;
    uint32_t n_total = 0, cells_total = 0;  // cells_total: padded to whole scan tiles
    bool counts_valid = true;             // hist/coarse match keys
    bool layout_dirty = true;             // scene ranges changed: re-upload tiles, re-capture
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    // rank placement (frames in which every scene is in LOOP): [one frame / a chain]
    // x [offsets buffer the first frame writes]; ob: the buffer (0: offs, 1:
    // cnt.offs_old) holding the last frame's offsets; rank_ready: cnt.far[ob ^ 1]
    // lists the far moves of the last frame, which was ranked too
    cudaGraphExec_t rgraph[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    int ob = 0;
    bool rank_ready = false;
    std::vector<uint32_t> last_modes;
    mb_tuning tuning{};                   // frames_per_launch (chain length) and collide_block are used
    std::string err;
};

namespace {

mb_status bfail(mb_batch* b, mb_status st, const std::string& msg) {
    if (b) b->err = msg;
    mb::set_process_error(msg);
    return st;
}
mb_status bcuda(mb_batch* b, const char* what, cudaError_t e) {
    return bfail(b, e == cudaErrorMemoryAllocation ? MB_ERR_OOM : MB_ERR_CUDA,
                 std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

void drop_graphs(mb_batch* b) {
    for (auto& g : b->graph) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
    for (auto& set : b->rgraph)
        for (auto& g : set) {
            if (g) cudaGraphExecDestroy(g);
            g = nullptr;
        }
}

uint32_t* offs_buf(const mb_batch* b, int i) { return i ? b->cnt.offs_old : b->offs; }

uint64_t bytes_for(uint64_t agents, uint64_t cells, uint64_t scenes) {
    // state x2, sorted copy, keys, perm; offs x2; counts, fixup lists; tile and band tables
    return agents * (32u * 3u + 8u) + cells * 8u + mb::count_scratch_bytes((uint32_t)cells, (uint32_t)agents) +
           scenes * sizeof(mb::SceneDev) + (agents / kTile + 1u) * (4u + 32u) + 64u * 1024u;
}

cudaError_t alloc_pool(mb_batch* b) {
    const size_t A = std::max<uint32_t>(b->cap_agents, 1u), Cc = std::max<uint32_t>(b->cap_cells, 1u);
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking))) return e;
    for (int i = 0; i < 2; ++i) {
        if ((e = cudaMalloc(&b->pos[i], sizeof(float4) * A))) return e;
        if ((e = cudaMalloc(&b->vfme[i], sizeof(uint4) * A))) return e;
    }
    if ((e = cudaMalloc(&b->spos, sizeof(float4) * A))) return e;
    if ((e = cudaMalloc(&b->svfme, sizeof(uint4) * A))) return e;
    if ((e = cudaMalloc(&b->bands, sizeof(uint4) * mb::band_table_entries((uint32_t)A)))) return e;
    if ((e = cudaMalloc(&b->keys, sizeof(uint32_t) * A))) return e;
    if ((e = cudaMalloc(&b->perm, sizeof(uint32_t) * A))) return e;
    if ((e = cudaMalloc(&b->offs, sizeof(uint32_t) * (Cc + 1u)))) return e;
    if ((e = cudaMalloc(&b->ctl, sizeof(uint32_t) * mb::kCtlWords))) return e;
    if ((e = cudaMemset(b->ctl, 0, sizeof(uint32_t) * mb::kCtlWords))) return e;
    if ((e = cudaMalloc(&b->d_tile_scene, sizeof(uint32_t) * (A / kTile + 1u)))) return e;
    if ((e = cudaMalloc(&b->d_cell_tile_scene, sizeof(uint32_t) * (Cc / mb::kScanTile + 1u)))) return e;
    if ((e = cudaMallocHost(&b->h_cell_tile_scene, sizeof(uint32_t) * (Cc / mb::kScanTile + 1u)))) return e;
    if ((e = cudaMalloc(&b->d_scenes, sizeof(mb::SceneDev) * std::max<uint32_t>(b->cap_scenes, 1u)))) return e;
    if ((e = cudaMallocHost(&b->h_scenes, sizeof(mb::SceneDev) * std::max<uint32_t>(b->cap_scenes, 1u)))) return e;
    if ((e = cudaMallocHost(&b->h_tile_scene, sizeof(uint32_t) * (A / kTile + 1u)))) return e;
    if ((e = cudaEventCreateWithFlags(&b->table_ev, cudaEventDisableTiming))) return e;
    if ((e = cudaMemset(b->keys, 0, sizeof(uint32_t) * A))) return e;
    if ((e = mb::count_scratch_alloc(b->cnt, (uint32_t)Cc, (uint32_t)A))) return e;
    return mb::count_rank_alloc(b->cnt);
}

void free_pool(mb_batch* b) {
    drop_graphs(b);
    for (int i = 0; i < 2; ++i) {
        cudaFree(b->pos[i]);
        cudaFree(b->vfme[i]);
    }
    cudaFree(b->spos);
    cudaFree(b->svfme);
    cudaFree(b->bands);
    cudaFree(b->keys);
    cudaFree(b->perm);
    cudaFree(b->offs);
    cudaFree(b->ctl);
    cudaFree(b->d_tile_scene);
    cudaFree(b->d_cell_tile_scene);
    if (b->h_cell_tile_scene) cudaFreeHost(b->h_cell_tile_scene);
    cudaFree(b->d_scenes);
    if (b->h_scenes) cudaFreeHost(b->h_scenes);
    if (b->h_tile_scene) cudaFreeHost(b->h_tile_scene);
    if (b->table_ev) cudaEventDestroy(b->table_ev);
    mb::count_scratch_free(b->cnt);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
}

mb_status add_scene(mb_batch* b, const mb_settings* s, uint32_t* index) {
    std::string why;
    if (!mb::settings_valid(s, why)) return bfail(b, MB_ERR_INVALID_ARG, why);
    const uint64_t cells = (uint64_t)s->number_of_grids_one_dimension * s->number_of_grids_one_dimension;
    if (b->scenes.size() >= b->cap_scenes || (uint64_t)b->n_total + s->max_number_of_agents > b->cap_agents ||
        (uint64_t)b->cells_total + padded_cells(cells) > b->cap_cells)
        return bfail(b, MB_ERR_BUDGET_EXCEEDED, "batch capacity exhausted (scenes, spheres or cells)");
    SceneHost h;
    h.s = *s;
    mb_quantize_settings(s, &h.c);
    h.agent_base = b->n_total;
    h.n = s->max_number_of_agents;
    h.cell_base = b->cells_total;
    h.cells = (uint32_t)cells;
    b->scenes.push_back(h);
    b->n_total += h.n;
    b->cells_total += padded_cells(h.cells);
    b->layout_dirty = true;
    b->counts_valid = false;
    if (index) *index = (uint32_t)(b->scenes.size() - 1u);
    return MB_OK;
}

// Upload the scene table (and tile table after a layout change) if it differs
// from what the device holds.
cudaError_t sync_tables(mb_batch* b, const std::vector<uint32_t>& modes) {
    const bool layout = b->layout_dirty;
    if (!layout && modes == b->last_modes) return cudaSuccess;
    cudaError_t e = cudaEventSynchronize(b->table_ev);  // pinned mirrors free to rewrite
    if (e) return e;
    const uint32_t S = (uint32_t)b->scenes.size();
    for (uint32_t i = 0; i < S; ++i) {
        const SceneHost& h = b->scenes[i];
        mb::SceneDev& d = b->h_scenes[i];
        d.P = mb::make_params(h.c);
        d.agent_base = h.agent_base;
        d.agent_end = h.agent_base + h.n;
        d.cell_base = h.cell_base;
        d.mode = modes[i];
        d.parity = h.parity;
    }
    if ((e = cudaMemcpyAsync(b->d_scenes, b->h_scenes, sizeof(mb::SceneDev) * S, cudaMemcpyHostToDevice,
                             b->stream)))
        return e;
    if (layout) {
        const uint32_t tiles = (b->n_total + kTile - 1u) / kTile;
        uint32_t sc = 0;
        for (uint32_t t = 0; t < tiles; ++t) {
            while (sc + 1u < S && t * kTile >= b->scenes[sc].agent_base + b->scenes[sc].n) ++sc;
            b->h_tile_scene[t] = sc;
        }
        if ((e = cudaMemcpyAsync(b->d_tile_scene, b->h_tile_scene, sizeof(uint32_t) * std::max(tiles, 1u),
                                 cudaMemcpyHostToDevice, b->stream)))
            return e;
        const uint32_t ctiles = b->cells_total / mb::kScanTile;
        sc = 0;
        for (uint32_t t = 0; t < ctiles; ++t) {
            while (sc + 1u < S && t * mb::kScanTile >= b->scenes[sc].cell_base + padded_cells(b->scenes[sc].cells))
                ++sc;
            b->h_cell_tile_scene[t] = sc;
        }
        if ((e = cudaMemcpyAsync(b->d_cell_tile_scene, b->h_cell_tile_scene, sizeof(uint32_t) * std::max(ctiles, 1u),
                                 cudaMemcpyHostToDevice, b->stream)))
            return e;
        drop_graphs(b);
        b->layout_dirty = false;
    }
    b->last_modes = modes;
    return cudaEventRecord(b->table_ev, b->stream);
}

// may_init: a scene can be in its INIT frame (false for chained frames, which
// never hold one), so the tile counts of INIT scenes are summed afterwards.
cudaError_t enqueue_frame(mb_batch* b, cudaStream_t st, bool may_init) {
    cudaError_t e;
    if ((e = mb::count_scan_scenes(b->cnt, b->d_scenes, b->d_cell_tile_scene, b->cells_total, b->offs, st)))
        return e;
    if ((e = mb::count_scatter_scenes(b->cnt, b->d_scenes, b->d_tile_scene, b->d_cell_tile_scene, b->keys, b->n_total,
                                      b->cells_total, b->offs, b->perm, b->pos[0], b->pos[1], b->vfme[0],
                                      b->vfme[1], b->spos, b->svfme, b->bands, st, b->tuning.scatter_agents,
                                      may_init)))
        return e;
    if ((e = mb::launch_physics_batch(b->d_scenes, b->d_tile_scene, b->n_total, b->offs, b->bands, b->spos, b->svfme,
                                      b->pos[0], b->pos[1], b->vfme[0], b->vfme[1], b->keys, b->cnt.hist,
                                      b->cnt.coarse, b->ctl + mb::kCtlError, st, b->tuning.collide_block)))
        return e;
    // INIT scenes emitted cell counts only: their tile counts from the cell counts
    if (may_init &&
        (e = mb::count_tile_counts_scenes(b->cnt, b->d_scenes, b->d_cell_tile_scene, b->cells_total, st)))
        return e;
    const uint32_t S = (uint32_t)b->scenes.size();
    k_flip_parity<<<(S + 127u) / 128u, 128, 0, st>>>(b->d_scenes, S);
    return cudaGetLastError();
}

// A frame in which every scene is in LOOP, sorted by rank placement: writes the
// offsets buffer q, reads the previous frame's from q ^ 1, ranks the far moves
// listed in cnt.far[q] and lists this frame's in cnt.far[q ^ 1] (emptied by the scan).
cudaError_t enqueue_rank_frame(mb_batch* b, cudaStream_t st, int q) {
    cudaError_t e;
    if ((e = mb::count_scan_scenes(b->cnt, b->d_scenes, b->d_cell_tile_scene, b->cells_total, offs_buf(b, q), st,
                                   b->cnt.far[q ^ 1])))
        return e;
    if ((e = mb::count_rank_scenes(b->cnt, b->d_scenes, b->d_tile_scene, b->d_cell_tile_scene, b->keys, b->n_total,
                                   b->cells_total, offs_buf(b, q), offs_buf(b, q ^ 1), b->cnt.far[q], b->perm,
                                   b->pos[0], b->pos[1], b->vfme[0], b->vfme[1], b->spos, b->svfme, b->bands, st)))
        return e;
    if ((e = mb::launch_physics_batch(b->d_scenes, b->d_tile_scene, b->n_total, offs_buf(b, q), b->bands, b->spos,
                                      b->svfme, b->pos[0], b->pos[1], b->vfme[0], b->vfme[1], b->keys, b->cnt.hist,
                                      b->cnt.coarse, b->ctl + mb::kCtlError, st, b->tuning.collide_block,
                                      b->cnt.far[q ^ 1])))
        return e;
    const uint32_t S = (uint32_t)b->scenes.size();
    k_flip_parity<<<(S + 127u) / 128u, 128, 0, st>>>(b->d_scenes, S);
    return cudaGetLastError();
}

// graph[0]: one frame; graph[1]: chain_frames(b) frames back to back (used while
// no scene changes mode; 1, 2, 4, 8 (default) or 16).
uint32_t chain_frames(const mb_batch* b) {
    return b->tuning.frames_per_launch ? b->tuning.frames_per_launch : 8u;
}

// rank >= 0: rank-placement frames, the first writing offsets buffer `rank`
// (into rgraph[which][rank]).
cudaError_t build_graph(mb_batch* b, int which = 0, int rank = -1) {
    cudaError_t e = cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal);
    if (e) return e;
    cudaError_t fe = cudaSuccess;
    for (uint32_t f = 0; f < (which ? chain_frames(b) : 1u) && !fe; ++f)
        fe = rank >= 0 ? enqueue_rank_frame(b, b->cap_stream, rank ^ (int)(f & 1u))
                       : enqueue_frame(b, b->cap_stream, !which);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->cap_stream, &g);
    if (fe) {
        if (g) cudaGraphDestroy(g);
        return fe;
    }
    if (e) return e;
    e = cudaGraphInstantiate(rank >= 0 ? &b->rgraph[which][rank] : &b->graph[which], g, 0);
    cudaGraphDestroy(g);
    return e;
}

// Rebuild per-cell counts from the keys of every scene (after an upload).
cudaError_t recount(mb_batch* b) {
    cudaError_t e = mb::count_keys(b->cnt, b->keys, b->n_total, b->cells_total, b->stream);
    if (!e) b->counts_valid = true;
    return e;
}

// One frame over every scene (frames = 1), or chain_frames(b) frames with the same
// modes and no INIT among them; modes[i] is scene i's mode.
mb_status run_frame(mb_batch* b, const std::vector<uint32_t>& modes, uint32_t frames = 1) {
    cudaError_t e;
    const int which = frames == 1 ? 0 : 1;  // (a chain of one frame is graph 0)
    if (!b->counts_valid && (e = recount(b))) {
        b->rank_ready = false;
        return bcuda(b, "batch recount", e);
    }
    if ((e = sync_tables(b, modes))) return bcuda(b, "batch tables", e);
    const bool all_loop = std::all_of(modes.begin(), modes.end(), [](uint32_t m) { return m == mb::kModeLoop; });
    if (b->tuning.sort_algorithm == MB_SORT_RANK && all_loop && b->counts_valid) {
        const int q = b->ob ^ 1;  // offsets buffer of the first frame
        if (!b->rank_ready) {
            // no far list describes this input yet: mark it overflowed, so the first
            // frame claims slots and fixes cells (its physics pass then lists far moves)
            if ((e = cudaMemsetAsync(b->cnt.far[q], 0xFF, sizeof(uint32_t), b->stream)))
                return bcuda(b, "batch frame", e);
            b->rank_ready = true;
        }
        if (!b->rgraph[which][q] && (e = build_graph(b, which, q))) return bcuda(b, "batch capture", e);
        if ((e = cudaGraphLaunch(b->rgraph[which][q], b->stream))) return bcuda(b, "batch frame", e);
        b->ob = q ^ (int)((frames - 1u) & 1u);
    } else {
        if (!b->graph[which] && (e = build_graph(b, which))) return bcuda(b, "batch capture", e);
        if ((e = cudaGraphLaunch(b->graph[which], b->stream))) return bcuda(b, "batch frame", e);
        b->ob = 0;
        b->rank_ready = false;
    }
    for (size_t i = 0; i < b->scenes.size(); ++i) {
        SceneHost& h = b->scenes[i];
        if (modes[i] != mb::kModeHold) {
            h.time += frames;
            h.frame_done = true;
            h.parity ^= frames & 1u;  // mirrors k_flip_parity
        }
        if (modes[i] == mb::kModeInit) h.init_pending = false;
    }
    return MB_OK;
}

// Copy a scene's state in the pool's current buffers (every scene lives in the
// same parity).
mb_status set_scene_state(mb_batch* b, uint32_t si, const float* pos, const uint32_t* vfme, mb_memory where) {
    if (si >= b->scenes.size()) return bfail(b, MB_ERR_INVALID_ARG, "scene index out of range");
    if (!pos || !vfme) return bfail(b, MB_ERR_INVALID_ARG, "NULL state");
    SceneHost& h = b->scenes[si];
    cudaMemcpyKind kind = where == MB_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(b->pos[h.parity] + h.agent_base, pos, sizeof(float4) * h.n, kind, b->stream)))
        return bcuda(b, "batch set_state", e);
    if ((e = cudaMemcpyAsync(b->vfme[h.parity] + h.agent_base, vfme, sizeof(uint4) * h.n, kind, b->stream)))
        return bcuda(b, "batch set_state", e);
    k_fill_keys<<<(h.n + 255u) / 256u, 256, 0, b->stream>>>(b->keys + h.agent_base, h.n,
                                                             h.cell_base | mb::kInitKeyBit);
    if ((e = cudaGetLastError())) return bcuda(b, "batch set_state", e);
    if (where == MB_HOST && (e = cudaStreamSynchronize(b->stream))) return bcuda(b, "batch set_state", e);
    h.has_state = true;
    h.init_pending = true;
    h.frame_done = false;
    h.time = 0;
    b->counts_valid = false;
    return MB_OK;
}

}  // namespace

extern "C" {

mb_status mb_batch_create(const mb_settings* scenes, uint32_t num_scenes, uint32_t capacity_agents,
                          uint32_t capacity_cells, uint32_t capacity_scenes, void* cuda_stream, mb_batch** out) {
    if (!out) return bfail(nullptr, MB_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (num_scenes && !scenes) return bfail(nullptr, MB_ERR_INVALID_ARG, "scenes is NULL");
    uint64_t agents = 0, cells = 0;
    std::string why;
    for (uint32_t i = 0; i < num_scenes; ++i) {
        if (!mb::settings_valid(&scenes[i], why)) return bfail(nullptr, MB_ERR_INVALID_ARG, why);
        agents += scenes[i].max_number_of_agents;
        cells += padded_cells((uint64_t)scenes[i].number_of_grids_one_dimension * scenes[i].number_of_grids_one_dimension);
    }
    agents = std::max<uint64_t>(agents, capacity_agents);
    // capacity_cells counts N*N cells; each scene may add up to one scan tile of padding
    const uint64_t scenes_cap = std::max(num_scenes, capacity_scenes);
    if (capacity_cells) cells = std::max<uint64_t>(cells, capacity_cells + scenes_cap * (mb::kScanTile - 1u));
    if (agents > mb::kMaxAgents || cells > mb::kMaxCells)
        return bfail(nullptr, MB_ERR_INVALID_ARG, "batch exceeds 2^28 spheres or cells");
    mb_batch* b = new (std::nothrow) mb_batch();
    if (!b) return bfail(nullptr, MB_ERR_OOM, "host allocation failed");
    b->cap_agents = (uint32_t)agents;
    b->cap_cells = (uint32_t)cells;
    b->cap_scenes = std::max(num_scenes, capacity_scenes);
    b->stream = (cudaStream_t)cuda_stream;
    b->tuning.digit_bits_max = 8;
    b->tuning.collide_block = mb::kPhysicsTile;
    b->tuning.frames_per_launch = 8;
    b->tuning.sort_algorithm = MB_SORT_RANK;
    cudaError_t e = alloc_pool(b);
    if (e) {
        mb_status st = bcuda(nullptr, "mb_batch_create", e);
        free_pool(b);
        delete b;
        return st;
    }
    for (uint32_t i = 0; i < num_scenes; ++i) add_scene(b, &scenes[i], nullptr);
    *out = b;
    return MB_OK;
}

mb_status mb_batch_add_scene(mb_batch* b, const mb_settings* s, uint32_t* index) {
    if (!b) return bfail(nullptr, MB_ERR_INVALID_ARG, "batch is NULL");
    return add_scene(b, s, index);
}

mb_status mb_batch_destroy(mb_batch* b) {
    if (!b) return MB_OK;
    cudaStreamSynchronize(b->stream);
    free_pool(b);
    delete b;
    return MB_OK;
}

uint32_t mb_batch_num_scenes(const mb_batch* b) { return b ? (uint32_t)b->scenes.size() : 0u; }

mb_status mb_batch_memory(const mb_batch* b, uint64_t* bytes) {
    if (!b || !bytes) return MB_ERR_INVALID_ARG;
    *bytes = bytes_for(b->cap_agents, b->cap_cells, b->cap_scenes);
    return MB_OK;
}

mb_status mb_batch_set_state(mb_batch* b, uint32_t scene, const float* pos_scale, const uint32_t* vfme,
                             mb_memory where) {
    if (!b) return bfail(nullptr, MB_ERR_INVALID_ARG, "batch is NULL");
    return set_scene_state(b, scene, pos_scale, vfme, where);
}

mb_status mb_batch_get_state(mb_batch* b, uint32_t scene, float* pos_scale, uint32_t* vfme, mb_memory where) {
    if (!b) return bfail(nullptr, MB_ERR_INVALID_ARG, "batch is NULL");
    if (scene >= b->scenes.size()) return bfail(b, MB_ERR_INVALID_ARG, "scene index out of range");
    const SceneHost& h = b->scenes[scene];
    if (!h.has_state) return bfail(b, MB_ERR_NOT_READY, "scene has no state");
    cudaMemcpyKind kind = where == MB_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    cudaError_t e;
    if (pos_scale &&
        (e = cudaMemcpyAsync(pos_scale, b->pos[h.parity] + h.agent_base, sizeof(float4) * h.n, kind, b->stream)))
        return bcuda(b, "batch get_state", e);
    if (vfme && (e = cudaMemcpyAsync(vfme, b->vfme[h.parity] + h.agent_base, sizeof(uint4) * h.n, kind, b->stream)))
        return bcuda(b, "batch get_state", e);
    if (where == MB_HOST && (e = cudaStreamSynchronize(b->stream))) return bcuda(b, "batch get_state", e);
    return MB_OK;
}

mb_status mb_batch_set_active(mb_batch* b, uint32_t scene, int active) {
    if (!b) return bfail(nullptr, MB_ERR_INVALID_ARG, "batch is NULL");
    if (scene >= b->scenes.size()) return bfail(b, MB_ERR_INVALID_ARG, "scene index out of range");
    b->scenes[scene].active = active != 0;
    return MB_OK;
}

mb_status mb_batch_step(mb_batch* b, uint32_t k) {
    mb::NvtxRange nvtx_range("mb_batch_step");
    if (!b) return bfail(nullptr, MB_ERR_INVALID_ARG, "batch is NULL");
    for (const SceneHost& h : b->scenes)
        if (!h.has_state) return bfail(b, MB_ERR_NOT_READY, "every scene needs a state before stepping");
    std::vector<uint32_t> modes(b->scenes.size());
    for (uint32_t f = 0; f < k;) {
        bool init = false;
        for (size_t i = 0; i < b->scenes.size(); ++i) {
            const SceneHost& h = b->scenes[i];
            const bool run = h.active && h.s.enable_simulation;
            modes[i] = !run ? mb::kModeHold : (h.init_pending ? mb::kModeInit : mb::kModeLoop);
            init = init || modes[i] == mb::kModeInit;
        }
        const uint32_t cf = chain_frames(b);
        const uint32_t frames = (!init && cf > 1u && k - f >= cf) ? cf : 1u;
        mb_status st = run_frame(b, modes, frames);
        if (st != MB_OK) return st;
        f += frames;
    }
    return MB_OK;
}

mb_status mb_batch_sync(mb_batch* b) {
    if (!b) return bfail(nullptr, MB_ERR_INVALID_ARG, "batch is NULL");
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e) return bcuda(b, "mb_batch_sync", e);
    uint32_t flag = 0;
    if ((e = cudaMemcpy(&flag, b->ctl + mb::kCtlError, sizeof(uint32_t), cudaMemcpyDeviceToHost)))
        return bcuda(b, "mb_batch_sync", e);
    if (flag) {
        cudaMemset(b->ctl + mb::kCtlError, 0, sizeof(uint32_t));
        return bfail(b, MB_ERR_TIMEOUT, "a bounded device-side wait gave up; results since the last sync are invalid");
    }
    return MB_OK;
}

int64_t mb_batch_time(const mb_batch* b, uint32_t scene) {
    return (b && scene < b->scenes.size()) ? b->scenes[scene].time : -1;
}

mb_status mb_batch_get_debug(mb_batch* b, uint32_t scene, uint32_t* keys, uint32_t* perm, uint32_t* start,
                             uint32_t* close, mb_memory where) {
    if (!b) return bfail(nullptr, MB_ERR_INVALID_ARG, "batch is NULL");
    if (scene >= b->scenes.size()) return bfail(b, MB_ERR_INVALID_ARG, "scene index out of range");
    const SceneHost& h = b->scenes[scene];
    if (!h.frame_done) return bfail(b, MB_ERR_NOT_READY, "no frame has run for this scene since its upload");
    const uint32_t m = std::max(h.n, h.cells);
    uint32_t* tmp = nullptr;  // device staging for host requests
    cudaError_t e;
    uint32_t *dk = keys, *dp = perm, *ds = start, *dc = close;
    if (where == MB_HOST) {
        if ((e = cudaMalloc(&tmp, sizeof(uint32_t) * (2u * (size_t)h.n + 2u * (size_t)h.cells))))
            return bcuda(b, "batch debug", e);
        dk = keys ? tmp : nullptr;
        dp = perm ? tmp + h.n : nullptr;
        ds = start ? tmp + 2u * h.n : nullptr;
        dc = close ? tmp + 2u * h.n + h.cells : nullptr;
    }
    k_local_debug<<<(m + 255u) / 256u, 256, 0, b->stream>>>(b->keys, b->perm, offs_buf(b, b->ob), h.n, h.cells,
                                                             h.agent_base, h.cell_base, dk, dp, ds, dc);
    e = cudaGetLastError();
    if (!e && where == MB_HOST) {
        if (keys) e = cudaMemcpyAsync(keys, dk, sizeof(uint32_t) * h.n, cudaMemcpyDeviceToHost, b->stream);
        if (!e && perm) e = cudaMemcpyAsync(perm, dp, sizeof(uint32_t) * h.n, cudaMemcpyDeviceToHost, b->stream);
        if (!e && start) e = cudaMemcpyAsync(start, ds, sizeof(uint32_t) * h.cells, cudaMemcpyDeviceToHost, b->stream);
        if (!e && close) e = cudaMemcpyAsync(close, dc, sizeof(uint32_t) * h.cells, cudaMemcpyDeviceToHost, b->stream);
        if (!e) e = cudaStreamSynchronize(b->stream);
        cudaFree(tmp);
    }
    if (e) return bcuda(b, "batch debug", e);
    return MB_OK;
}

mb_status mb_batch_get_tuning(const mb_batch* b, mb_tuning* out) {
    if (!b || !out) return MB_ERR_INVALID_ARG;
    *out = b->tuning;
    return MB_OK;
}

mb_status mb_batch_set_tuning(mb_batch* b, const mb_tuning* t) {
    if (!b || !t) return bfail(b, MB_ERR_INVALID_ARG, "NULL argument");
    const uint32_t fpl = t->frames_per_launch;
    if (!(fpl == 0 || fpl == 1 || fpl == 2 || fpl == 4 || fpl == 8 || fpl == 16))
        return bfail(b, MB_ERR_INVALID_ARG, "frames_per_launch must be 0, 1, 2, 4, 8 or 16");
    if (t->collide_block != 64u && t->collide_block != 128u && t->collide_block != 256u)
        return bfail(b, MB_ERR_INVALID_ARG, "collide_block must be 64, 128 or 256");
    if (t->scatter_agents > 4u || t->scatter_agents == 3u)
        return bfail(b, MB_ERR_INVALID_ARG, "scatter_agents must be 0, 1, 2 or 4");
    if ((t->sort_algorithm != MB_SORT_RANK && t->sort_algorithm != MB_SORT_COUNTING) ||
        t->state_gather != MB_GATHER_COPY || t->frame_kernel != MB_FRAME_GRAPH)
        return bfail(b, MB_ERR_INVALID_ARG,
                     "a batch runs rank placement or the counting sort, the sorted copy and per-stage kernels");
    drop_graphs(b);
    b->tuning = *t;
    b->rank_ready = false;
    return MB_OK;
}

mb_status mb_batch_autotune(mb_batch* b, uint32_t frames, mb_tuning* best, float* frame_ms, mb_tuning* tried) {
    mb::NvtxRange nvtx_range("mb_batch_autotune");
    if (!b || !best) return bfail(b, MB_ERR_INVALID_ARG, "NULL argument");
    if (frames == 0) return bfail(b, MB_ERR_INVALID_ARG, "frames must be positive");
    if (b->scenes.empty()) return bfail(b, MB_ERR_NOT_READY, "the batch has no scene");
    for (const SceneHost& h : b->scenes)
        if (!h.has_state || h.init_pending || !h.frame_done)
            return bfail(b, MB_ERR_NOT_READY, "run a frame of every scene before autotuning");
    const mb_tuning start = b->tuning;
    mb_tuning cand[MB_BATCH_TUNE_CANDIDATES];
    {
        const uint32_t fpl[3] = {1u, 8u, 16u}, tiles[3] = {64u, 128u, 256u};
        uint32_t c = 0;
        for (uint32_t f : fpl)
            for (uint32_t t : tiles) {
                cand[c] = start;
                cand[c].sort_algorithm = MB_SORT_RANK;
                cand[c].frames_per_launch = f;
                cand[c].collide_block = t;
                cand[c].scatter_agents = 1u;
                ++c;
            }
        for (uint32_t a : {1u, 2u, 4u}) {  // the counting sort, spheres per scatter thread
            cand[c] = start;
            cand[c].sort_algorithm = MB_SORT_COUNTING;
            cand[c].frames_per_launch = 8u;
            cand[c].collide_block = 128u;
            cand[c].scatter_agents = a;
            ++c;
        }
    }
    // save what the frames overwrite: both state buffers (scenes keep their own
    // parity), keys, order, cell offsets and the host view of every scene
    const size_t A = b->n_total, Cc = (size_t)b->cells_total + 1u;
    float4* pos[2] = {nullptr, nullptr};
    uint4* vfme[2] = {nullptr, nullptr};
    uint32_t *keys = nullptr, *perm = nullptr, *offs = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    auto release = [&]() {
        for (int i = 0; i < 2; ++i) {
            cudaFree(pos[i]);
            cudaFree(vfme[i]);
        }
        cudaFree(keys);
        cudaFree(perm);
        cudaFree(offs);
        for (auto& x : ev)
            if (x) cudaEventDestroy(x);
    };
    const std::vector<SceneHost> saved = b->scenes;
    const int ob0 = b->ob;  // the offsets buffer holding the saved frame's offsets
    auto snap = [&](bool save) -> cudaError_t {
        cudaError_t r;
        auto cp = [&](void* a, void* d, size_t bytes) {
            return cudaMemcpyAsync(save ? a : d, save ? d : a, bytes, cudaMemcpyDeviceToDevice, b->stream);
        };
        for (int i = 0; i < 2; ++i) {
            if ((r = cp(pos[i], b->pos[i], sizeof(float4) * A))) return r;
            if ((r = cp(vfme[i], b->vfme[i], sizeof(uint4) * A))) return r;
        }
        if ((r = cp(keys, b->keys, sizeof(uint32_t) * A))) return r;
        if ((r = cp(perm, b->perm, sizeof(uint32_t) * A))) return r;
        return cp(offs, offs_buf(b, ob0), sizeof(uint32_t) * Cc);
    };
    auto restore_host = [&]() {
        b->scenes = saved;
        b->last_modes.clear();  // the scene table (parities) is uploaded again before the next frame
        b->counts_valid = false;
        b->ob = ob0;
        b->rank_ready = false;
    };
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 2 && !e; ++i) {
        if (!e) e = cudaMalloc(&pos[i], sizeof(float4) * A);
        if (!e) e = cudaMalloc(&vfme[i], sizeof(uint4) * A);
    }
    if (!e) e = cudaMalloc(&keys, sizeof(uint32_t) * A);
    if (!e) e = cudaMalloc(&perm, sizeof(uint32_t) * A);
    if (!e) e = cudaMalloc(&offs, sizeof(uint32_t) * Cc);
    if (!e) e = cudaEventCreate(&ev[0]);
    if (!e) e = cudaEventCreate(&ev[1]);
    if (!e) e = snap(true);
    if (e) {
        release();
        return bcuda(b, "mb_batch_autotune", e);
    }
    float best_ms = 0.0f;
    uint32_t best_i = 0;
    mb_status st = MB_OK;
    for (uint32_t c = 0; c < MB_BATCH_TUNE_CANDIDATES && st == MB_OK; ++c) {
        if ((e = snap(false))) break;  // every candidate starts from the saved frame
        restore_host();
        if ((st = mb_batch_set_tuning(b, &cand[c])) != MB_OK) break;
        if ((st = mb_batch_step(b, 1)) != MB_OK) break;  // warm-up: graphs built
        if ((e = cudaEventRecord(ev[0], b->stream))) break;
        if ((st = mb_batch_step(b, frames)) != MB_OK) break;
        if ((e = cudaEventRecord(ev[1], b->stream)) || (e = cudaEventSynchronize(ev[1]))) break;
        float ms = 0.0f;
        if ((e = cudaEventElapsedTime(&ms, ev[0], ev[1]))) break;
        ms /= (float)frames;
        if (frame_ms) frame_ms[c] = ms;
        if (tried) tried[c] = cand[c];
        if (c == 0 || ms < best_ms) {
            best_ms = ms;
            best_i = c;
        }
    }
    cudaError_t e2 = snap(false);
    restore_host();
    const mb_status st2 = mb_batch_set_tuning(b, (e || st != MB_OK) ? &start : &cand[best_i]);
    if (!e2) e2 = cudaStreamSynchronize(b->stream);
    release();
    if (e) return bcuda(b, "mb_batch_autotune", e);
    if (st != MB_OK) return st;
    if (e2) return bcuda(b, "mb_batch_autotune", e2);
    if (st2 != MB_OK) return st2;
    *best = cand[best_i];
    return MB_OK;
}

}  // extern "C"

// ============================================================================
// Serving: a request loop over one batch pool.
//
// create-scene requests are admitted in arrival order while the pool's memory
// budget (spheres, cells, scenes reserved at start-up) has room; scenes stay
// resident, so a create that does not fit is rejected (MB_ERR_BUDGET_EXCEEDED)
// and so are later requests on it.  Advance requests add steps to their scene.  A worker thread runs frames over the
// pool: every scene with a pending step runs LOOP (INIT first after an
// upload), the others HOLD.  Requests that arrive while frames are on the GPU
// join at the next frame.  A request completes when its scene has taken all
// its steps; its latency is completion minus submission (host clock).
// ============================================================================

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t id = 0;
    bool create = false;
    uint32_t scene = 0;
    uint32_t steps = 0;
    mb_settings settings{};
    std::vector<float> pos;
    std::vector<uint32_t> vfme;
    Clock::time_point submitted;
    int64_t target_time = -1;  // scene time at which the request is done
    bool done = false;
    double latency = 0.0;
    mb_status status = MB_OK;
};

struct ServerScene {
    bool admitted = false;
    bool rejected = false;
    uint32_t pool = 0;          // index of the scene in the batch pool
    int64_t pending = 0;        // steps owed (incl. INIT)
    int64_t scheduled_time = 0; // scene time after every step owed so far
};

}  // namespace

struct mb_server {
    mb_batch* pool = nullptr;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> incoming;        // not yet seen by the worker
    std::unordered_map<uint64_t, Request*> requests;
    std::vector<ServerScene> sscenes;     // by scene handle (submission order)
    std::vector<uint32_t> pool_handle;    // scene handle of each pool scene
    std::vector<Request*> in_flight;      // advance/create requests not yet complete
    uint64_t next_id = 1;
    uint32_t next_scene = 0;              // scene handles handed out (admission order)
    bool stop = false;
    mb_server_stats stats{};
    std::string err;
};

namespace {

void complete(mb_server* s, Request* r, Clock::time_point now) {
    r->done = true;
    r->latency = std::chrono::duration<double>(now - r->submitted).count();
    s->stats.requests_done += 1;
}

void worker_loop(mb_server* s) {
    mb_batch* b = s->pool;
    std::vector<uint32_t> modes;
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        bool idle = true;
        for (const ServerScene& sc : s->sscenes)
            if (sc.admitted && sc.pending > 0) idle = false;
        if (idle && s->incoming.empty()) s->cv_work.wait(lk, [&] { return s->stop || !s->incoming.empty(); });
        if (s->stop) return;
        // admit creates in arrival order; queue advances on their scenes
        std::deque<Request*> fresh;
        fresh.swap(s->incoming);
        for (Request* r : fresh) {
            if (s->sscenes.size() <= r->scene) s->sscenes.resize(r->scene + 1u);
            ServerScene& sc = s->sscenes[r->scene];
            if (r->create) {
                uint32_t idx = 0;
                mb_status st = add_scene(b, &r->settings, &idx);
                if (st == MB_OK) st = set_scene_state(b, idx, r->pos.data(), r->vfme.data(), MB_HOST);
                r->pos = std::vector<float>();
                r->vfme = std::vector<uint32_t>();
                if (st != MB_OK) {  // no room (scenes stay resident) or bad input: rejected
                    r->status = st;
                    sc.rejected = true;
                    complete(s, r, Clock::now());
                    continue;
                }
                if (s->pool_handle.size() <= idx) s->pool_handle.resize(idx + 1u);
                s->pool_handle[idx] = r->scene;
                sc.admitted = true;
                sc.pool = idx;
                sc.pending = 1;  // the INIT frame
                sc.scheduled_time = 1;
                r->target_time = 1;
                s->in_flight.push_back(r);
            } else {
                if (sc.rejected || !sc.admitted) {
                    r->status = sc.rejected ? MB_ERR_BUDGET_EXCEEDED : MB_ERR_INVALID_ARG;
                    complete(s, r, Clock::now());
                    continue;
                }
                sc.pending += r->steps;
                sc.scheduled_time += r->steps;
                r->target_time = sc.scheduled_time;
                s->in_flight.push_back(r);
            }
        }
        s->cv_done.notify_all();
        // a round of up to 16 frames; each frame runs the scenes that still have
        // frames owed (INIT first after an upload), the others are held
        const size_t S = b->scenes.size();
        int64_t frames = 0;
        for (size_t i = 0; i < S; ++i) {
            const ServerScene& sc = s->sscenes[s->pool_handle[i]];
            if (sc.admitted && sc.pending > 0) frames = std::max<int64_t>(frames, std::min<int64_t>(sc.pending, 16));
        }
        if (frames == 0) continue;
        const auto t0 = Clock::now();
        uint64_t agent_steps = 0;
        modes.assign(S, mb::kModeHold);
        for (int64_t f = 0; f < frames;) {
            bool init = false;
            int64_t least = INT64_MAX;  // fewest frames owed by a scene that runs
            for (size_t i = 0; i < S; ++i) {
                const ServerScene& sc = s->sscenes[s->pool_handle[i]];
                const bool run = sc.admitted && sc.pending > 0 && b->scenes[i].s.enable_simulation;
                modes[i] = !run ? mb::kModeHold : (b->scenes[i].init_pending ? mb::kModeInit : mb::kModeLoop);
                init = init || modes[i] == mb::kModeInit;
                if (run) least = std::min<int64_t>(least, sc.pending);
            }
            // a chain of frames while every running scene owes that many and none is new
            const int64_t cf = (int64_t)chain_frames(b);
            const uint32_t chain = (!init && cf > 1 && least >= cf && frames - f >= cf) ? (uint32_t)cf : 1u;
            for (size_t i = 0; i < S; ++i)
                if (modes[i] == mb::kModeLoop) agent_steps += (uint64_t)b->scenes[i].n * chain;
            if (run_frame(b, modes, chain) != MB_OK) {
                s->err = b->err;
                break;
            }
            for (size_t i = 0; i < S; ++i)
                if (modes[i] != mb::kModeHold) s->sscenes[s->pool_handle[i]].pending -= chain;
            f += chain;
        }
        lk.unlock();  // submitters keep queueing while the GPU works
        cudaStreamSynchronize(b->stream);
        const auto t1 = Clock::now();
        lk.lock();
        s->stats.frames += (uint64_t)frames;
        s->stats.agent_steps += agent_steps;
        s->stats.busy_seconds += std::chrono::duration<double>(t1 - t0).count();
        for (auto it = s->in_flight.begin(); it != s->in_flight.end();) {
            Request* r = *it;
            if (b->scenes[s->sscenes[r->scene].pool].time >= r->target_time) {
                complete(s, r, t1);
                it = s->in_flight.erase(it);
            } else {
                ++it;
            }
        }
        s->cv_done.notify_all();
    }
}

}  // namespace

extern "C" {

mb_status mb_server_create(const mb_server_config* cfg, void* cuda_stream, mb_server** out) {
    if (!out || !cfg) return bfail(nullptr, MB_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    // split the budget: per sphere ~104 B, per cell 16 B (cells ~ 2 x spheres)
    uint64_t budget = cfg->budget_bytes;
    uint64_t agents = cfg->max_agents, cells = cfg->max_cells;
    if (!agents || !cells) {
        const uint64_t fixed = bytes_for(0, 0, cfg->max_scenes);
        const uint64_t per = 104u + 2u * 16u + 1u;  // a sphere and two cells, plus tile tables
        agents = budget > fixed ? std::min<uint64_t>((budget - fixed) / per, mb::kMaxAgents) : 0u;
        // room for each scene's padding to whole scan tiles inside the 2^28-cell key space
        const uint64_t pad = (uint64_t)std::max<uint32_t>(cfg->max_scenes, 1u) * (mb::kScanTile - 1u);
        cells = std::min<uint64_t>(2u * agents, mb::kMaxCells > pad ? mb::kMaxCells - pad : 0u);
    }
    if (bytes_for(agents, cells, cfg->max_scenes) > budget)
        return bfail(nullptr, MB_ERR_BUDGET_EXCEEDED, "configured capacity exceeds the memory budget");
    mb_server* s = new (std::nothrow) mb_server();
    if (!s) return bfail(nullptr, MB_ERR_OOM, "host allocation failed");
    mb_status st = mb_batch_create(nullptr, 0, (uint32_t)agents, (uint32_t)cells,
                                   std::max<uint32_t>(cfg->max_scenes, 1u), cuda_stream, &s->pool);
    if (st != MB_OK) {
        delete s;
        return st;
    }
    s->worker = std::thread(worker_loop, s);
    *out = s;
    return MB_OK;
}

mb_status mb_server_destroy(mb_server* s) {
    if (!s) return MB_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    mb_batch_destroy(s->pool);
    for (auto& kv : s->requests) delete kv.second;
    delete s;
    return MB_OK;
}

mb_status mb_server_submit_create(mb_server* s, const mb_settings* settings, const float* pos_scale,
                                  const uint32_t* vfme, uint32_t* scene, uint64_t* request) {
    if (!s || !settings || !pos_scale || !vfme) return bfail(nullptr, MB_ERR_INVALID_ARG, "NULL argument");
    std::string why;
    if (!mb::settings_valid(settings, why)) return bfail(nullptr, MB_ERR_INVALID_ARG, why);
    Request* r = new (std::nothrow) Request();
    if (!r) return bfail(nullptr, MB_ERR_OOM, "host allocation failed");
    r->create = true;
    r->settings = *settings;
    const size_t n = settings->max_number_of_agents;
    r->pos.assign(pos_scale, pos_scale + 4u * n);
    r->vfme.assign(vfme, vfme + 4u * n);
    r->submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        r->scene = s->next_scene++;
        s->requests[r->id] = r;
        s->incoming.push_back(r);
    }
    s->cv_work.notify_all();
    if (scene) *scene = r->scene;
    if (request) *request = r->id;
    return MB_OK;
}

mb_status mb_server_submit_advance(mb_server* s, uint32_t scene, uint32_t k, uint64_t* request) {
    if (!s) return bfail(nullptr, MB_ERR_INVALID_ARG, "server is NULL");
    Request* r = new (std::nothrow) Request();
    if (!r) return bfail(nullptr, MB_ERR_OOM, "host allocation failed");
    r->scene = scene;
    r->steps = k;
    r->submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (scene >= s->next_scene) {
            delete r;
            return bfail(nullptr, MB_ERR_INVALID_ARG, "unknown scene");
        }
        r->id = s->next_id++;
        s->requests[r->id] = r;
        s->incoming.push_back(r);
    }
    s->cv_work.notify_all();
    if (request) *request = r->id;
    return MB_OK;
}

mb_status mb_server_wait(mb_server* s, uint64_t request, double timeout_s, double* latency_s) {
    if (!s) return bfail(nullptr, MB_ERR_INVALID_ARG, "server is NULL");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(request);
    if (it == s->requests.end()) return bfail(nullptr, MB_ERR_INVALID_ARG, "unknown request");
    Request* r = it->second;
    bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return r->done; });
    if (!ok) return MB_ERR_NOT_READY;
    if (latency_s) *latency_s = r->latency;
    mb_status st = r->status;
    s->requests.erase(it);
    delete r;
    return st;
}

mb_status mb_server_get_state(mb_server* s, uint32_t scene, float* pos_scale, uint32_t* vfme) {
    if (!s) return bfail(nullptr, MB_ERR_INVALID_ARG, "server is NULL");
    // wait until the scene owes no step, then copy under the lock (frames are
    // only launched by the worker, which takes the lock between rounds)
    std::unique_lock<std::mutex> lk(s->mu);
    if (scene >= s->next_scene) return bfail(nullptr, MB_ERR_INVALID_ARG, "unknown scene");
    s->cv_done.wait(lk, [&] {
        if (scene >= s->sscenes.size()) return false;
        const ServerScene& sc = s->sscenes[scene];
        return sc.rejected || (sc.admitted && sc.pending == 0);
    });
    if (s->sscenes[scene].rejected) return bfail(nullptr, MB_ERR_BUDGET_EXCEEDED, "scene was not admitted");
    return mb_batch_get_state(s->pool, s->sscenes[scene].pool, pos_scale, vfme, MB_HOST);
}

mb_status mb_server_get_stats(mb_server* s, mb_server_stats* out) {
    if (!s || !out) return MB_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->scenes = (uint32_t)s->pool->scenes.size();
    return MB_OK;
}

}  // extern "C"
