// mb_api.cu — the C ABI (include/millionsball.h): worlds, frames, graphs, stages.
//
// One frame = PhysicsNode::run (src/physics/mod.rs:846-912): sort the cell keys
// emitted by the previous frame, build the cell offsets, run the physics pass
// (INIT on frame 0 after an upload, LOOP afterwards, mod.rs:929-939).  The
// reference's eve/odd bind groups (mod.rs:659-705) become two state buffers that
// swap every frame; each LOOP frame parity is one captured CUDA graph.

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "mb_internal.h"

namespace {

thread_local std::string g_last_error;

std::string cuda_msg(const char* what, cudaError_t e) {
    return std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
}

// (x * 1000.) as i32 / as u32: truncation toward zero, saturating, NaN -> 0
// (src/physics/mod.rs:473-481).
int32_t q_i32(float x) {
    float v = x * 1000.0f;
    if (std::isnan(v)) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v <= -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}
uint32_t q_u32(float x) {
    float v = x * 1000.0f;
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)v;
}

}  // namespace

void mb::set_process_error(const std::string& msg) { g_last_error = msg; }

struct mb_world {
    mb_settings s{};
    mb_consts c{};
    mb::PhysParams P{};
    uint32_t n = 0;
    uint32_t cells = 0;
    int device = 0;
    cudaStream_t stream = nullptr;     // caller's stream: all work is ordered on it
    cudaStream_t cap_stream = nullptr; // private stream used only to capture graphs
    float4* pos[2] = {nullptr, nullptr};
    uint4* vfme[2] = {nullptr, nullptr};
    float4* spos = nullptr;            // state in sorted order (input of the LOOP pass)
    uint4* svfme = nullptr;
    uint32_t* keys = nullptr;          // unsorted keys emitted by the last physics pass
    uint32_t* sorted_keys = nullptr;
    uint4* bands = nullptr;            // band table of the sorted order (written by the sort)
    uint32_t* perm = nullptr;
    uint32_t* fused_bar = nullptr;     // grid barrier words of the fused frame kernel (2, zero between launches)
    mb::SortScratch scratch;      // onesweep sort scratch + the cell offsets (offs)
    mb::CountScratch cnt;         // counting-sort scratch (per-cell and per-tile counts, fixup lists)
    mb::SortSchedule sched;
    mb_tuning tuning{};
    int cur = 0;
    int64_t time = -1;
    bool has_state = false;
    bool frame_done = false;           // a frame ran since the last upload
    bool rank_ready = false;           // cnt.far[cur] lists the far moves of the frame before (MB_SORT_RANK)
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    cudaGraphExec_t chain[2] = {nullptr, nullptr};  // chained LOOP frames from each parity
    unsigned long long* zbuf = nullptr;             // render depth buffer (grown on demand)
    size_t zbuf_pixels = 0;
    uint32_t* img = nullptr;                        // render outputs for MB_HOST
    float* img_h = nullptr;
    bool profiling = false;
    cudaEvent_t prof_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::string err;
};

namespace {

mb_status fail(mb_world* w, mb_status st, const std::string& msg) {
    if (w) w->err = msg;
    g_last_error = msg;
    return st;
}
mb_status cuda_fail(mb_world* w, const char* what, cudaError_t e) {
    return fail(w, e == cudaErrorMemoryAllocation ? MB_ERR_OOM : MB_ERR_CUDA, cuda_msg(what, e));
}

}  // namespace

bool mb::settings_valid(const mb_settings* s, std::string& why) {
    if (!s) { why = "settings is NULL"; return false; }
    if (s->max_number_of_agents == 0 || s->max_number_of_agents > mb::kMaxAgents) {
        why = "max_number_of_agents must be in [1, 2^28-1]";
        return false;
    }
    if (s->number_of_grids_one_dimension == 0 || s->grid_size == 0) {
        why = "number_of_grids_one_dimension and grid_size must be >= 1";
        return false;
    }
    uint64_t cells = (uint64_t)s->number_of_grids_one_dimension * s->number_of_grids_one_dimension;
    if (cells > mb::kMaxCells) { why = "number_of_grids_one_dimension^2 must be <= 2^28"; return false; }
    if ((uint64_t)s->number_of_grids_one_dimension * s->grid_size > 0xFFFFFFFFull) {
        why = "number_of_grids_one_dimension * grid_size overflows u32";
        return false;
    }
    mb_consts c;
    mb_quantize_settings(s, &c);
    if (!(c.time_delta > 0.0f)) { why = "time_delta quantises to 0 (needs >= 0.001)"; return false; }
    return true;
}

namespace {
using mb::settings_valid;

// LOOP frames captured back to back in one graph for multi-frame steps: the
// tuning's frames_per_launch (even, or 1; so a chain ends in the parity it
// started from), 8 by default.
uint32_t chain_frames(const mb_world* w) {
    return w->tuning.frames_per_launch ? w->tuning.frames_per_launch : 8u;
}

void drop_graphs(mb_world* w) {
    for (auto* set : {w->graph, w->chain})
        for (int i = 0; i < 2; ++i) {
            if (set[i]) cudaGraphExecDestroy(set[i]);
            set[i] = nullptr;
        }
}

void apply_settings(mb_world* w, const mb_settings& s) {
    w->s = s;
    mb_quantize_settings(&s, &w->c);
    w->P = mb::make_params(w->c);
    w->cells = s.number_of_grids_one_dimension * s.number_of_grids_one_dimension;
    w->sched = mb::make_schedule(w->n, w->cells, w->tuning.digit_bits_max);
}

// Record a profiling event; inside a stream capture it becomes an event-record
// node that fires on every graph launch.
cudaError_t mark(mb_world* w, int i, cudaStream_t st, bool capturing) {
    if (!w->profiling) return cudaSuccess;
    return capturing ? cudaEventRecordWithFlags(w->prof_ev[i], st, cudaEventRecordExternal)
                     : cudaEventRecord(w->prof_ev[i], st);
}

// Counting sort (claim-and-fixup or rank placement) rather than the radix sort.
bool counting(const mb_world* w) { return w->tuning.sort_algorithm != MB_SORT_ONESWEEP; }
// LOOP frames place spheres by rank (falling back to claim-and-fixup by themselves).
bool rank(const mb_world* w) { return w->tuning.sort_algorithm == MB_SORT_RANK; }
// Cell offsets a frame reading state buffer `cur` writes.  Rank placement reads
// the previous frame's offsets while the scan writes new ones, so it alternates
// two buffers by state parity; the other sorts keep one.
uint32_t* frame_offs(const mb_world* w, int cur) {
    return rank(w) && cur ? w->cnt.offs_old : w->scratch.offs;
}
// The offsets of the last frame run (the current order's cell ranges).
uint32_t* cur_offs(const mb_world* w) { return frame_offs(w, w->cur ^ 1); }
// The physics pass reads the state through the permutation instead of a sorted copy.
bool indirect(const mb_world* w) { return w->tuning.state_gather == MB_GATHER_INDIRECT; }
// LOOP frames run as one cooperative kernel per step (profiling needs the
// per-stage kernels, so it falls back to them).
bool fused(const mb_world* w) { return w->tuning.frame_kernel == MB_FRAME_FUSED && !w->profiling; }
constexpr uint32_t kFusedFramesPerLaunch = 256;

cudaError_t enqueue_fused(mb_world* w, uint32_t frames) {
    mb::FusedFrame f;
    f.P = w->P;
    f.n = w->n;
    f.cells = w->cells;
    f.frames = frames;
    f.cur = (uint32_t)w->cur;
    f.indirect = indirect(w);
    f.keys = w->keys;
    f.offs = w->scratch.offs;
    f.perm = w->perm;
    f.bands = w->bands;
    f.cnt = &w->cnt;
    for (int b = 0; b < 2; ++b) {
        f.pos[b] = w->pos[b];
        f.vfme[b] = w->vfme[b];
    }
    f.spos = w->spos;
    f.svfme = w->svfme;
    f.bar = w->fused_bar;
    f.err = w->scratch.ctl + mb::kCtlError;
    return mb::launch_frame_fused(f, w->stream);
}

// Enqueue one frame on `st`.  Profiling marks: [0] frame start, [1] after the
// first ordering stage, [2] after the second, [3] after physics.  `chained`: the
// frame follows another frame in the same capture.
cudaError_t enqueue_frame(mb_world* w, cudaStream_t st, int cur, bool init, bool capturing = false,
                          bool chained = false) {
    cudaError_t e;
    // kernels after the first start while their predecessor drains (programmatic
    // dependent launch) in captured LOOP frames without profiling marks between them
    const bool pdl = capturing && !init && !w->profiling;
    uint32_t* hist = nullptr;
    uint32_t* coarse = nullptr;
    if ((e = mark(w, 0, st, capturing))) return e;
    if (counting(w) && init) {
        // frame 0 after an upload sorts all-zero keys: identity order, one full cell
        if ((e = mb::count_init_order(w->cnt, w->n, w->cells, frame_offs(w, cur), w->perm, st))) return e;
        if ((e = mark(w, 1, st, capturing))) return e;
        hist = w->cnt.hist;
        coarse = w->cnt.coarse;
    } else if (rank(w)) {
        // cell offsets (into the buffer of this parity: the other holds the
        // previous frame's), then the order by rank in the old neighbourhoods;
        // this frame's physics pass lists its far moves in cnt.far[cur ^ 1]
        if ((e = mb::count_scan(w->cnt, w->scratch.ctl, w->cells, frame_offs(w, cur), st, pdl && chained,
                                w->cnt.far[cur ^ 1])))
            return e;
        if ((e = mark(w, 1, st, capturing))) return e;
        if ((e = mb::count_rank(w->cnt, w->keys, w->n, w->cells, frame_offs(w, cur), frame_offs(w, cur ^ 1),
                                w->cnt.far[cur], w->perm, w->pos[cur], w->vfme[cur], indirect(w) ? nullptr : w->spos,
                                indirect(w) ? nullptr : w->svfme, w->bands, w->P.N, st, pdl,
                                w->tuning.scatter_agents)))
            return e;
        hist = w->cnt.hist;
        coarse = w->cnt.coarse;
    } else if (counting(w)) {
        // cell offsets first (scan of the counts), then the permutation
        if ((e = mb::count_scan(w->cnt, w->scratch.ctl, w->cells, w->scratch.offs, st, pdl && chained))) return e;
        if ((e = mark(w, 1, st, capturing))) return e;
        if ((e = mb::count_scatter(w->cnt, w->keys, w->n, w->cells, w->scratch.offs, w->perm, w->pos[cur],
                                   w->vfme[cur], indirect(w) ? nullptr : w->spos, indirect(w) ? nullptr : w->svfme,
                                   w->bands, w->P.N, st, pdl, w->tuning.scatter_agents)))
            return e;
        hist = w->cnt.hist;
        coarse = w->cnt.coarse;
    } else {
        if ((e = mb::sort_pairs(w->scratch, w->sched, w->keys, nullptr, w->sorted_keys, w->perm, st))) return e;
        if ((e = mark(w, 1, st, capturing))) return e;
        if ((e = mb::cell_offsets(w->scratch, w->sched, w->sorted_keys, st))) return e;
        if (!init && (e = mb::gather_state(w->perm, w->n, w->pos[cur], w->vfme[cur],
                                           indirect(w) ? nullptr : w->spos, indirect(w) ? nullptr : w->svfme,
                                           w->sorted_keys, w->scratch.offs, w->bands, w->P.N, st)))
            return e;
    }
    if ((e = mark(w, 2, st, capturing))) return e;
    int nxt = cur ^ 1;
    if (init) {
        e = mb::launch_physics_init(w->P, w->n, w->perm, w->pos[cur], w->vfme[cur], w->pos[nxt],
                                    w->vfme[nxt], w->keys, hist, coarse, st);
        if (!e && hist) e = mb::count_tile_counts(w->cnt, w->cells, st);
    } else if (indirect(w)) {
        e = mb::launch_physics_loop(w->P, w->n, frame_offs(w, cur), w->bands, w->pos[cur], w->vfme[cur], w->perm,
                                    w->pos[nxt], w->vfme[nxt], w->keys, hist, coarse, w->scratch.ctl + mb::kCtlError,
                                    st, pdl && counting(w), w->tuning.collide_block,
                                    rank(w) ? w->cnt.far[nxt] : nullptr);
    } else {
        e = mb::launch_physics_loop(w->P, w->n, frame_offs(w, cur), w->bands, w->spos, w->svfme, nullptr, w->pos[nxt],
                                    w->vfme[nxt], w->keys, hist, coarse, w->scratch.ctl + mb::kCtlError, st,
                                    pdl && counting(w), w->tuning.collide_block,
                                    rank(w) ? w->cnt.far[nxt] : nullptr);
    }
    if (e) return e;
    return mark(w, 3, st, capturing);
}

// Rebuild the per-cell counts of the current keys (counting mode only).
cudaError_t recount(mb_world* w) {
    if (!counting(w)) return cudaSuccess;
    if (!w->frame_done) return mb::count_reset_zero_keys(w->cnt, w->n, w->cells, w->stream);
    return mb::count_keys(w->cnt, w->keys, w->n, w->cells, w->stream);
}

// One LOOP frame (frames = 1, into graph[cur]) or a chain of kChainFrames LOOP
// frames (into chain[cur]) captured from parity `cur`.
cudaError_t build_graph(mb_world* w, int cur, uint32_t frames = 1) {
    cudaError_t e = cudaStreamBeginCapture(w->cap_stream, cudaStreamCaptureModeThreadLocal);
    if (e) return e;
    cudaError_t fe = cudaSuccess;
    for (uint32_t f = 0; f < frames && !fe; ++f) fe = enqueue_frame(w, w->cap_stream, cur ^ (int)(f & 1u), false, true, f > 0);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(w->cap_stream, &g);
    if (fe) {
        if (g) cudaGraphDestroy(g);
        return fe;
    }
    if (e) return e;
    e = cudaGraphInstantiate(frames == 1 ? &w->graph[cur] : &w->chain[cur], g, 0);
    cudaGraphDestroy(g);
    return e;
}

}  // namespace

extern "C" {

void mb_settings_default(mb_settings* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    // PhysicsPlugin::default (src/physics/mod.rs:87-109)
    o->enable_simulation = 1;
    o->enable_spring = 0;
    o->number_of_grids_one_dimension = 128;
    o->grid_size = 8;
    o->half_map_height = 16;
    o->gravity[0] = 0.0f;
    o->gravity[1] = -9.8f;
    o->gravity[2] = 0.0f;
    o->e_envir = 0.90f;
    o->e_agent = 0.95f;
    o->k_agent = 25.0f;
    o->c_agent = 0.1f;
    o->r_agent = 0.9f;
    o->max_number_of_agents = 16 * 1024;
    o->time_delta = 1.0f / 120.0f;
}

mb_status mb_quantize_settings(const mb_settings* s, mb_consts* c) {
    if (!s || !c) return MB_ERR_INVALID_ARG;
    std::memset(c, 0, sizeof(*c));
    c->number_of_grids_one_dimension = s->number_of_grids_one_dimension;
    c->grid_size = s->grid_size;
    c->half_map_height = (float)s->half_map_height;  // HALF_MAP_HEIGHT = f32(u32)
    c->half_map_size = (float)((s->number_of_grids_one_dimension * s->grid_size) / 2u);
    if (s->exact_constants) {
        for (int i = 0; i < 3; ++i) c->gravity[i] = s->gravity[i];
        c->e_envir = s->e_envir;
        c->e_agent = s->e_agent;
        c->k_agent = s->k_agent;
        c->c_agent = s->c_agent;
        c->r_agent = s->r_agent;
        c->time_delta = s->time_delta;
    } else {
        // f32(#DEF) / 1000. (physics.wgsl:7-16)
        for (int i = 0; i < 3; ++i) c->gravity[i] = (float)q_i32(s->gravity[i]) / 1000.0f;
        c->e_envir = (float)q_u32(s->e_envir) / 1000.0f;
        c->e_agent = (float)q_u32(s->e_agent) / 1000.0f;
        c->k_agent = (float)q_u32(s->k_agent) / 1000.0f;
        c->c_agent = (float)q_u32(s->c_agent) / 1000.0f;
        c->r_agent = (float)q_u32(s->r_agent) / 1000.0f;
        c->time_delta = (float)q_u32(s->time_delta) / 1000.0f;
    }
    c->enable_spring = s->enable_spring ? 1u : 0u;
    return MB_OK;
}

mb_status mb_create(const mb_settings* s, void* cuda_stream, mb_world** out) {
    if (!out) return fail(nullptr, MB_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    std::string why;
    if (!settings_valid(s, why)) return fail(nullptr, MB_ERR_INVALID_ARG, why);
    mb_world* w = new (std::nothrow) mb_world();
    if (!w) return fail(nullptr, MB_ERR_OOM, "host allocation failed");
    cudaGetDevice(&w->device);
    w->stream = (cudaStream_t)cuda_stream;
    w->n = s->max_number_of_agents;
    w->tuning.digit_bits_max = 8;
    w->tuning.collide_block = 128;
    w->tuning.sort_algorithm = MB_SORT_RANK;
    apply_settings(w, *s);
    const size_t n = w->n;
    auto alloc_all = [&]() -> cudaError_t {
        cudaError_t e;
        if ((e = cudaStreamCreateWithFlags(&w->cap_stream, cudaStreamNonBlocking))) return e;
        for (int i = 0; i < 2; ++i) {
            if ((e = cudaMalloc(&w->pos[i], sizeof(float4) * n))) return e;
            if ((e = cudaMalloc(&w->vfme[i], sizeof(uint4) * n))) return e;
        }
        if ((e = cudaMalloc(&w->spos, sizeof(float4) * n))) return e;
        if ((e = cudaMalloc(&w->svfme, sizeof(uint4) * n))) return e;
        if ((e = cudaMalloc(&w->keys, sizeof(uint32_t) * n))) return e;
        if ((e = cudaMalloc(&w->sorted_keys, sizeof(uint32_t) * n))) return e;
        if ((e = cudaMalloc(&w->bands, sizeof(uint4) * mb::band_table_entries(n)))) return e;
        if ((e = cudaMalloc(&w->perm, sizeof(uint32_t) * n))) return e;
        if ((e = cudaMalloc(&w->fused_bar, sizeof(uint32_t) * 2u))) return e;
        if ((e = cudaMemset(w->fused_bar, 0, sizeof(uint32_t) * 2u))) return e;
        if ((e = mb::scratch_alloc(w->scratch, w->n, w->cells))) return e;
        if ((e = mb::count_scratch_alloc(w->cnt, w->cells, w->n))) return e;
        return mb::count_rank_alloc(w->cnt);
    };
    cudaError_t e = alloc_all();
    if (e) {
        mb_status st = cuda_fail(nullptr, "mb_create", e);
        mb_destroy(w);
        return st;
    }
    *out = w;
    return MB_OK;
}

mb_status mb_destroy(mb_world* w) {
    if (!w) return MB_OK;
    if (w->stream || w->cap_stream) cudaStreamSynchronize(w->stream);
    drop_graphs(w);
    for (int i = 0; i < 2; ++i) {
        cudaFree(w->pos[i]);
        cudaFree(w->vfme[i]);
    }
    cudaFree(w->spos);
    cudaFree(w->svfme);
    cudaFree(w->keys);
    cudaFree(w->sorted_keys);
    cudaFree(w->bands);
    cudaFree(w->zbuf);
    cudaFree(w->img);
    cudaFree(w->img_h);
    cudaFree(w->perm);
    cudaFree(w->fused_bar);
    mb::scratch_free(w->scratch);
    mb::count_scratch_free(w->cnt);
    if (w->cap_stream) cudaStreamDestroy(w->cap_stream);
    for (auto& ev : w->prof_ev)
        if (ev) cudaEventDestroy(ev);
    delete w;
    return MB_OK;
}

mb_status mb_set_settings(mb_world* w, const mb_settings* s) {
    if (!w) return fail(nullptr, MB_ERR_INVALID_ARG, "world is NULL");
    std::string why;
    if (!settings_valid(s, why)) return fail(w, MB_ERR_INVALID_ARG, why);
    if (s->max_number_of_agents != w->n)
        return fail(w, MB_ERR_INVALID_ARG, "max_number_of_agents is fixed for a world");
    bool grid_changed = s->number_of_grids_one_dimension != w->s.number_of_grids_one_dimension ||
                        s->grid_size != w->s.grid_size;
    uint32_t new_cells = s->number_of_grids_one_dimension * s->number_of_grids_one_dimension;
    if (new_cells > w->scratch.max_cells) {
        cudaError_t e = cudaStreamSynchronize(w->stream);
        if (e) return cuda_fail(w, "mb_set_settings", e);
        uint32_t* offs = nullptr;
        if ((e = cudaMalloc(&offs, sizeof(uint32_t) * ((size_t)new_cells + 1u))))
            return cuda_fail(w, "mb_set_settings", e);
        mb::CountScratch cnt;
        if ((e = mb::count_scratch_alloc(cnt, new_cells, w->n)) || (e = mb::count_rank_alloc(cnt))) {
            cudaFree(offs);
            mb::count_scratch_free(cnt);
            return cuda_fail(w, "mb_set_settings", e);
        }
        cudaFree(w->scratch.offs);
        w->scratch.offs = offs;
        w->scratch.max_cells = new_cells;
        mb::count_scratch_free(w->cnt);
        w->cnt = cnt;
    }
    drop_graphs(w);
    apply_settings(w, *s);
    w->rank_ready = false;
    // keys emitted under the old grid are re-derived under the new one
    if (grid_changed && w->has_state) {
        cudaError_t e = cudaSuccess;
        if (!w->frame_done) {
            e = recount(w);  // still the all-zero keys of the upload
        } else {
            uint32_t* hist = counting(w) ? w->cnt.hist : nullptr;
            uint32_t* coarse = counting(w) ? w->cnt.coarse : nullptr;
            if (hist) e = mb::count_clear(w->cnt, w->cells, w->stream);
            if (!e) e = mb::launch_rekey(w->P, w->n, w->pos[w->cur], w->keys, hist, coarse, w->stream);
            if (!e && hist) e = mb::count_tile_counts(w->cnt, w->cells, w->stream);
        }
        if (e) return cuda_fail(w, "mb_set_settings", e);
    }
    return MB_OK;
}

mb_status mb_get_settings(const mb_world* w, mb_settings* out) {
    if (!w || !out) return MB_ERR_INVALID_ARG;
    *out = w->s;
    return MB_OK;
}

mb_status mb_set_state(mb_world* w, const float* pos_scale, const uint32_t* vfme, mb_memory where) {
    if (!w || !pos_scale || !vfme) return fail(w, MB_ERR_INVALID_ARG, "NULL argument");
    cudaMemcpyKind kind = where == MB_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(w->pos[0], pos_scale, sizeof(float4) * w->n, kind, w->stream)))
        return cuda_fail(w, "mb_set_state", e);
    if ((e = cudaMemcpyAsync(w->vfme[0], vfme, sizeof(uint4) * w->n, kind, w->stream)))
        return cuda_fail(w, "mb_set_state", e);
    // fresh sort buffers hold zeros: frame 0 sorts all-zero keys (identity order)
    if ((e = cudaMemsetAsync(w->keys, 0, sizeof(uint32_t) * w->n, w->stream)))
        return cuda_fail(w, "mb_set_state", e);
    w->frame_done = false;
    w->rank_ready = false;
    if ((e = recount(w))) return cuda_fail(w, "mb_set_state", e);
    if (where == MB_HOST && (e = cudaStreamSynchronize(w->stream)))
        return cuda_fail(w, "mb_set_state", e);
    w->cur = 0;
    w->time = 0;
    w->has_state = true;
    return MB_OK;
}

mb_status mb_get_state(mb_world* w, float* pos_scale, uint32_t* vfme, mb_memory where) {
    if (!w) return fail(nullptr, MB_ERR_INVALID_ARG, "world is NULL");
    if (!w->has_state) return fail(w, MB_ERR_NOT_READY, "no state uploaded");
    cudaMemcpyKind kind = where == MB_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    cudaError_t e;
    if (pos_scale && (e = cudaMemcpyAsync(pos_scale, w->pos[w->cur], sizeof(float4) * w->n, kind, w->stream)))
        return cuda_fail(w, "mb_get_state", e);
    if (vfme && (e = cudaMemcpyAsync(vfme, w->vfme[w->cur], sizeof(uint4) * w->n, kind, w->stream)))
        return cuda_fail(w, "mb_get_state", e);
    if (where == MB_HOST && (e = cudaStreamSynchronize(w->stream))) return cuda_fail(w, "mb_get_state", e);
    return MB_OK;
}

mb_status mb_step(mb_world* w, uint32_t k) {
    mb::NvtxRange nvtx_range("mb_step");
    if (!w) return fail(nullptr, MB_ERR_INVALID_ARG, "world is NULL");
    if (!w->has_state) return fail(w, MB_ERR_NOT_READY, "no state uploaded");
    if (!w->s.enable_simulation) return MB_OK;
    cudaError_t e;
    for (uint32_t f = 0; f < k;) {
        if (w->time == 0) {
            if ((e = enqueue_frame(w, w->stream, w->cur, true))) return cuda_fail(w, "mb_step(init)", e);
            w->rank_ready = false;  // the next frame sorts keys in upload order
        } else if (fused(w)) {  // the remaining LOOP frames, one cooperative launch per 256
            const uint32_t fr = std::min(k - f, kFusedFramesPerLaunch);
            if ((e = enqueue_fused(w, fr))) return cuda_fail(w, "mb_step(fused)", e);
            f += fr;
            w->time += fr;
            w->cur ^= (int)(fr & 1u);
            w->frame_done = true;
            w->rank_ready = false;
            continue;
        } else if (rank(w) && !w->rank_ready) {
            // no far list describes this frame's input yet: mark it overflowed, so the
            // frame claims slots and fixes cells (its physics pass then lists far moves)
            if ((e = cudaMemsetAsync(w->cnt.far[w->cur], 0xFF, sizeof(uint32_t), w->stream)))
                return cuda_fail(w, "mb_step", e);
            w->rank_ready = true;
            continue;
        } else if (chain_frames(w) > 1u && k - f >= chain_frames(w) && !w->profiling) {
            // a chain of LOOP frames, one launch
            const uint32_t cf = chain_frames(w);
            if (!w->chain[w->cur] && (e = build_graph(w, w->cur, cf))) return cuda_fail(w, "mb_step(capture)", e);
            if ((e = cudaGraphLaunch(w->chain[w->cur], w->stream))) return cuda_fail(w, "mb_step", e);
            f += cf;
            w->time += cf;
            w->frame_done = true;
            continue;
        } else {
            if (!w->graph[w->cur] && (e = build_graph(w, w->cur)))
                return cuda_fail(w, "mb_step(capture)", e);
            if ((e = cudaGraphLaunch(w->graph[w->cur], w->stream))) return cuda_fail(w, "mb_step", e);
        }
        w->cur ^= 1;
        w->time += 1;
        w->frame_done = true;
        ++f;
    }
    return MB_OK;
}

mb_status mb_sync(mb_world* w) {
    if (!w) return fail(nullptr, MB_ERR_INVALID_ARG, "world is NULL");
    cudaError_t e = cudaStreamSynchronize(w->stream);
    if (e) return cuda_fail(w, "mb_sync", e);
    uint32_t flag = 0;
    if ((e = cudaMemcpy(&flag, w->scratch.ctl + mb::kCtlError, sizeof(uint32_t), cudaMemcpyDeviceToHost)))
        return cuda_fail(w, "mb_sync", e);
    if (flag) {
        cudaMemset(w->scratch.ctl + mb::kCtlError, 0, sizeof(uint32_t));
        cudaMemset(w->fused_bar, 0, sizeof(uint32_t) * 2u);  // a barrier that gave up leaves its count
        w->scratch.last_tiles = 0;  // force a clean look-back table next sort
        drop_graphs(w);
        char msg[192];
        std::snprintf(msg, sizeof msg,
                      "a bounded device-side wait gave up (flags 0x%x: 1 sort look-back, 4 band copy, 8 grid "
                      "barrier of the fused frame); results since the last sync are invalid",
                      flag);
        return fail(w, MB_ERR_TIMEOUT, msg);
    }
    return MB_OK;
}

mb_status mb_get_debug(mb_world* w, uint32_t* keys, uint32_t* perm, uint32_t* start, uint32_t* close,
                       mb_memory where) {
    if (!w) return fail(nullptr, MB_ERR_INVALID_ARG, "world is NULL");
    if (!w->frame_done) return fail(w, MB_ERR_NOT_READY, "no frame has run since the upload");
    cudaError_t e;
    cudaMemcpyKind kind = where == MB_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (keys && (e = cudaMemcpyAsync(keys, w->keys, sizeof(uint32_t) * w->n, kind, w->stream)))
        return cuda_fail(w, "mb_get_debug", e);
    if (perm && (e = cudaMemcpyAsync(perm, w->perm, sizeof(uint32_t) * w->n, kind, w->stream)))
        return cuda_fail(w, "mb_get_debug", e);
    if (start || close) {
        if (where == MB_DEVICE) {
            if ((e = mb::offsets_to_start_close(cur_offs(w), w->cells, start, close, w->stream)))
                return cuda_fail(w, "mb_get_debug", e);
        } else {
            std::vector<uint32_t> offs((size_t)w->cells + 1u);
            if ((e = cudaMemcpyAsync(offs.data(), cur_offs(w), sizeof(uint32_t) * offs.size(),
                                     cudaMemcpyDeviceToHost, w->stream)))
                return cuda_fail(w, "mb_get_debug", e);
            if ((e = cudaStreamSynchronize(w->stream))) return cuda_fail(w, "mb_get_debug", e);
            for (uint32_t c = 0; c < w->cells; ++c) {
                bool full = offs[c + 1] > offs[c];
                if (start) start[c] = full ? offs[c] : mb::kInvalid;
                if (close) close[c] = full ? offs[c + 1] - 1u : mb::kInvalid;
            }
        }
    }
    if (where == MB_HOST && (e = cudaStreamSynchronize(w->stream))) return cuda_fail(w, "mb_get_debug", e);
    return MB_OK;
}

mb_status mb_device_buffers(mb_world* w, const float** pos_scale, const uint32_t** vfme) {
    if (!w) return fail(nullptr, MB_ERR_INVALID_ARG, "world is NULL");
    if (pos_scale) *pos_scale = reinterpret_cast<const float*>(w->pos[w->cur]);
    if (vfme) *vfme = reinterpret_cast<const uint32_t*>(w->vfme[w->cur]);
    return MB_OK;
}

int64_t mb_time(const mb_world* w) { return w ? w->time : -1; }

const char* mb_last_error(const mb_world* w) { return w ? w->err.c_str() : g_last_error.c_str(); }

mb_status mb_get_tuning(const mb_world* w, mb_tuning* out) {
    if (!w || !out) return MB_ERR_INVALID_ARG;
    *out = w->tuning;
    return MB_OK;
}

mb_status mb_set_tuning(mb_world* w, const mb_tuning* t) {
    if (!w || !t) return fail(w, MB_ERR_INVALID_ARG, "NULL argument");
    if (t->digit_bits_max < 4 || t->digit_bits_max > mb::kMaxDigitBits)
        return fail(w, MB_ERR_INVALID_ARG, "digit_bits_max must be in [4, 11]");
    if (t->collide_block != 64u && t->collide_block != 128u && t->collide_block != 256u)
        return fail(w, MB_ERR_INVALID_ARG, "collide_block must be 64, 128 or 256");
    if (t->sort_algorithm != MB_SORT_COUNTING && t->sort_algorithm != MB_SORT_ONESWEEP &&
        t->sort_algorithm != MB_SORT_RANK)
        return fail(w, MB_ERR_INVALID_ARG, "sort_algorithm must be MB_SORT_COUNTING, MB_SORT_ONESWEEP or MB_SORT_RANK");
    const uint32_t fpl = t->frames_per_launch;
    if (!(fpl == 0 || fpl == 1 || fpl == 2 || fpl == 4 || fpl == 8 || fpl == 16))
        return fail(w, MB_ERR_INVALID_ARG, "frames_per_launch must be 0, 1, 2, 4, 8 or 16");
    if (t->state_gather != MB_GATHER_COPY && t->state_gather != MB_GATHER_INDIRECT)
        return fail(w, MB_ERR_INVALID_ARG, "state_gather must be MB_GATHER_COPY or MB_GATHER_INDIRECT");
    if (t->frame_kernel != MB_FRAME_GRAPH && t->frame_kernel != MB_FRAME_FUSED)
        return fail(w, MB_ERR_INVALID_ARG, "frame_kernel must be MB_FRAME_GRAPH or MB_FRAME_FUSED");
    if (t->scatter_agents > 4u || t->scatter_agents == 3u)
        return fail(w, MB_ERR_INVALID_ARG, "scatter_agents must be 0, 1, 2 or 4");
    if (t->frame_kernel == MB_FRAME_FUSED && t->sort_algorithm != MB_SORT_COUNTING)
        return fail(w, MB_ERR_INVALID_ARG, "MB_FRAME_FUSED runs the counting sort (sort_algorithm 0)");
    if (t->frame_kernel == MB_FRAME_FUSED && mb::fused_blocks_per_sm() <= 0)
        return fail(w, MB_ERR_INVALID_ARG, "the fused frame kernel cannot be resident on this device");
    drop_graphs(w);
    bool to_counting = t->sort_algorithm != MB_SORT_ONESWEEP && !counting(w);
    uint32_t* offs_before = cur_offs(w);
    w->tuning = *t;
    w->rank_ready = false;
    if (cur_offs(w) != offs_before) {  // the current cell ranges move to this sort's buffer
        cudaError_t e = cudaMemcpyAsync(cur_offs(w), offs_before, sizeof(uint32_t) * ((size_t)w->cells + 1u),
                                        cudaMemcpyDeviceToDevice, w->stream);
        if (e) return cuda_fail(w, "mb_set_tuning", e);
    }
    w->sched = mb::make_schedule(w->n, w->cells, w->tuning.digit_bits_max);
    if (to_counting && w->has_state) {  // counts were not kept while the radix sort ran
        cudaError_t e = recount(w);
        if (e) return cuda_fail(w, "mb_set_tuning", e);
    }
    return MB_OK;
}

// The per-world image buffers of the renderers, grown on demand.
cudaError_t image_buffers(mb_world* w, size_t px) {
    if (px <= w->zbuf_pixels) return cudaSuccess;
    cudaFree(w->zbuf);
    cudaFree(w->img);
    cudaFree(w->img_h);
    w->zbuf = nullptr;
    w->img = nullptr;
    w->img_h = nullptr;
    w->zbuf_pixels = 0;
    cudaError_t e;
    if ((e = cudaMalloc(&w->zbuf, sizeof(unsigned long long) * px)) ||
        (e = cudaMalloc(&w->img, sizeof(uint32_t) * px)) || (e = cudaMalloc(&w->img_h, sizeof(float) * px)))
        return e;
    w->zbuf_pixels = px;
    return cudaSuccess;
}

// Copies a rendered image (and its float plane) back to the host, synchronously.
cudaError_t image_to_host(mb_world* w, size_t px, uint32_t* rgba, const uint32_t* out, float* plane,
                          const float* out_plane) {
    cudaError_t e = cudaMemcpyAsync(rgba, out, sizeof(uint32_t) * px, cudaMemcpyDeviceToHost, w->stream);
    if (!e && plane) e = cudaMemcpyAsync(plane, out_plane, sizeof(float) * px, cudaMemcpyDeviceToHost, w->stream);
    if (!e) e = cudaStreamSynchronize(w->stream);
    return e;
}

mb_status mb_render_topdown(mb_world* w, uint32_t width, uint32_t height, float x0, float z0, float x1, float z1,
                            uint32_t* rgba, float* height_map, mb_memory where) {
    mb::NvtxRange nvtx_range("mb_render_topdown");
    if (!w || !rgba) return fail(w, MB_ERR_INVALID_ARG, "NULL argument");
    if (!w->has_state) return fail(w, MB_ERR_NOT_READY, "no state uploaded");
    if (width == 0 || height == 0 || (uint64_t)width * height > (1ull << 28))
        return fail(w, MB_ERR_INVALID_ARG, "image must have 1 .. 2^28 pixels");
    if (!(x1 > x0) || !(z1 > z0) || !std::isfinite(x0) || !std::isfinite(x1) || !std::isfinite(z0) ||
        !std::isfinite(z1))
        return fail(w, MB_ERR_INVALID_ARG, "window must satisfy x0 < x1, z0 < z1 (finite)");
    const size_t px = (size_t)width * height;
    cudaError_t e;
    if ((e = image_buffers(w, px))) return cuda_fail(w, "mb_render_topdown", e);
    const bool host = where == MB_HOST;
    uint32_t* out = host ? w->img : rgba;
    float* out_h = host ? w->img_h : (height_map ? height_map : w->img_h);
    if ((e = mb::render_topdown(w->pos[w->cur], w->n, width, height, x0, z0, x1, z1, w->zbuf, out, out_h,
                                w->stream)))
        return cuda_fail(w, "mb_render_topdown", e);
    if (host && (e = image_to_host(w, px, rgba, out, height_map, out_h))) return cuda_fail(w, "mb_render_topdown", e);
    return MB_OK;
}

mb_status mb_render_view(mb_world* w, uint32_t width, uint32_t height, const float* eye, const float* target,
                         float fov_y_degrees, uint32_t* rgba, float* depth, mb_memory where) {
    mb::NvtxRange nvtx_range("mb_render_view");
    if (!w || !rgba) return fail(w, MB_ERR_INVALID_ARG, "NULL argument");
    if (!w->has_state) return fail(w, MB_ERR_NOT_READY, "no state uploaded");
    if (width == 0 || height == 0 || (uint64_t)width * height > (1ull << 28))
        return fail(w, MB_ERR_INVALID_ARG, "image must have 1 .. 2^28 pixels");
    float e3[3], t3[3], fov, to_light[3];
    mb::reference_view(e3, t3, &fov, to_light);
    if (eye) std::copy(eye, eye + 3, e3);
    if (target) std::copy(target, target + 3, t3);
    if (fov_y_degrees > 0.0f) fov = fov_y_degrees;
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(e3[k]) || !std::isfinite(t3[k]))
            return fail(w, MB_ERR_INVALID_ARG, "eye and target must be finite");
    const float fx = t3[0] - e3[0], fy = t3[1] - e3[1], fz = t3[2] - e3[2];
    if (!(fx * fx + fz * fz > 1e-12f * (fx * fx + fy * fy + fz * fz)))  // also eye == target
        return fail(w, MB_ERR_INVALID_ARG, "the view direction must not be vertical (the image's up is +y)");
    if (!(fov < 180.0f) || !std::isfinite(fov))
        return fail(w, MB_ERR_INVALID_ARG, "fov_y_degrees must be below 180 (0 or less: 45)");
    const float tan_half = (float)std::tan((double)fov * 3.14159265358979323846 / 360.0);
    const size_t px = (size_t)width * height;
    cudaError_t e;
    if ((e = image_buffers(w, px))) return cuda_fail(w, "mb_render_view", e);
    const bool host = where == MB_HOST;
    uint32_t* out = host ? w->img : rgba;
    float* out_d = host ? (depth ? w->img_h : nullptr) : depth;
    if ((e = mb::render_view(w->pos[w->cur], w->n, width, height, e3, t3, tan_half, to_light, w->c.half_map_size,
                             2.0f * w->c.half_map_height, w->zbuf, out, out_d, w->stream)))
        return cuda_fail(w, "mb_render_view", e);
    if (host && (e = image_to_host(w, px, rgba, out, depth, out_d))) return cuda_fail(w, "mb_render_view", e);
    return MB_OK;
}

mb_status mb_autotune(mb_world* w, uint32_t frames, mb_tuning* best, float* frame_ms, mb_tuning* tried) {
    mb::NvtxRange nvtx_range("mb_autotune");
    if (!w || !best) return fail(w, MB_ERR_INVALID_ARG, "NULL argument");
    if (frames == 0) return fail(w, MB_ERR_INVALID_ARG, "frames must be positive");
    if (!w->frame_done || w->time == 0) return fail(w, MB_ERR_NOT_READY, "run a frame before autotuning");
    if (w->profiling) return fail(w, MB_ERR_INVALID_ARG, "turn profiling off before autotuning");
    const mb_tuning start = w->tuning;
    mb_tuning cand[MB_TUNE_CANDIDATES];
    {
        // {sort, digit bits, frames per graph launch, state gather, frame kernel, physics tile,
        //  scatter spheres per thread}
        const uint32_t C = MB_SORT_COUNTING, O = MB_SORT_ONESWEEP, R = MB_SORT_RANK, CP = MB_GATHER_COPY,
                       IN = MB_GATHER_INDIRECT, G = MB_FRAME_GRAPH, F = MB_FRAME_FUSED;
        const uint32_t c6[MB_TUNE_CANDIDATES][7] = {
            {R, 8u, 8u, CP, G, 128u, 1u},  {R, 8u, 16u, CP, G, 128u, 1u}, {R, 8u, 8u, CP, G, 256u, 1u},
            {R, 8u, 8u, CP, G, 128u, 2u},  {R, 8u, 8u, IN, G, 128u, 1u},
            {C, 8u, 1u, CP, G, 128u, 1u},  {C, 8u, 8u, CP, G, 128u, 1u},  {C, 8u, 16u, CP, G, 128u, 1u},
            {C, 8u, 8u, CP, G, 64u, 1u},   {C, 8u, 8u, CP, G, 256u, 1u},  {C, 8u, 16u, CP, G, 256u, 1u},
            {C, 8u, 8u, CP, G, 128u, 2u},  {C, 8u, 8u, CP, G, 128u, 4u},  {C, 8u, 16u, CP, G, 256u, 2u},
            {C, 8u, 8u, CP, F, 128u, 1u},  {C, 8u, 8u, IN, G, 128u, 1u},  {C, 8u, 16u, IN, G, 128u, 1u},
            {C, 8u, 8u, IN, G, 256u, 1u},  {C, 8u, 8u, IN, F, 128u, 1u},  {O, 6u, 8u, CP, G, 128u, 1u},
            {O, 8u, 1u, CP, G, 128u, 1u},  {O, 8u, 8u, CP, G, 128u, 1u},  {O, 8u, 8u, IN, G, 128u, 1u},
            {O, 11u, 8u, CP, G, 128u, 1u},
        };
        for (uint32_t c = 0; c < MB_TUNE_CANDIDATES; ++c) {
            cand[c] = start;
            cand[c].sort_algorithm = c6[c][0];
            cand[c].digit_bits_max = c6[c][1];
            cand[c].frames_per_launch = c6[c][2];
            cand[c].state_gather = c6[c][3];
            cand[c].frame_kernel = c6[c][4];
            cand[c].collide_block = c6[c][5];
            cand[c].scatter_agents = c6[c][6];
        }
    }
    // save what the frames overwrite
    const size_t n = w->n, C = w->cells;
    float4* pos = nullptr;
    uint4* vfme = nullptr;
    uint32_t *keys = nullptr, *perm = nullptr, *offs = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    auto release = [&]() {
        cudaFree(pos);
        cudaFree(vfme);
        cudaFree(keys);
        cudaFree(perm);
        cudaFree(offs);
        for (auto& x : ev)
            if (x) cudaEventDestroy(x);
    };
    const int cur0 = w->cur;
    const int64_t time0 = w->time;
    cudaError_t e = cudaSuccess;
    auto snap = [&](bool save) -> cudaError_t {
        cudaError_t r;
        auto cp = [&](void* a, void* b, size_t bytes) {
            return cudaMemcpyAsync(save ? a : b, save ? b : a, bytes, cudaMemcpyDeviceToDevice, w->stream);
        };
        if ((r = cp(pos, w->pos[cur0], sizeof(float4) * n))) return r;
        if ((r = cp(vfme, w->vfme[cur0], sizeof(uint4) * n))) return r;
        if ((r = cp(keys, w->keys, sizeof(uint32_t) * n))) return r;
        if ((r = cp(perm, w->perm, sizeof(uint32_t) * n))) return r;
        return cp(offs, cur_offs(w), sizeof(uint32_t) * (C + 1u));
    };
    if ((e = cudaMalloc(&pos, sizeof(float4) * std::max<size_t>(n, 1))) ||
        (e = cudaMalloc(&vfme, sizeof(uint4) * std::max<size_t>(n, 1))) ||
        (e = cudaMalloc(&keys, sizeof(uint32_t) * std::max<size_t>(n, 1))) ||
        (e = cudaMalloc(&perm, sizeof(uint32_t) * std::max<size_t>(n, 1))) ||
        (e = cudaMalloc(&offs, sizeof(uint32_t) * (C + 1u))) || (e = cudaEventCreate(&ev[0])) ||
        (e = cudaEventCreate(&ev[1])) || (e = snap(true))) {
        release();
        return cuda_fail(w, "mb_autotune", e);
    }
    float best_ms = 0.0f;
    uint32_t best_i = 0;
    mb_status st = MB_OK;
    for (uint32_t c = 0; c < MB_TUNE_CANDIDATES && st == MB_OK; ++c) {
        w->cur = cur0;  // before the restore: it writes the offsets buffer of this parity
        w->time = time0;
        if ((e = snap(false))) break;  // every candidate starts from the saved frame
        if ((st = mb_set_tuning(w, &cand[c])) != MB_OK) break;
        if ((e = recount(w))) break;  // counts of the restored keys
        if ((st = mb_step(w, 1)) != MB_OK) break;  // warm-up: graphs built, caches touched
        if ((e = cudaEventRecord(ev[0], w->stream))) break;
        if ((st = mb_step(w, frames)) != MB_OK) break;
        if ((e = cudaEventRecord(ev[1], w->stream)) || (e = cudaEventSynchronize(ev[1]))) break;
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
    // restore the saved frame under the winning tuning
    w->cur = cur0;
    w->time = time0;
    cudaError_t e2 = snap(false);
    mb_status st2 = mb_set_tuning(w, (e || st != MB_OK) ? &start : &cand[best_i]);
    if (!e2) e2 = recount(w);
    if (!e2) e2 = cudaStreamSynchronize(w->stream);
    release();
    if (e) return cuda_fail(w, "mb_autotune", e);
    if (st != MB_OK) return st;
    if (e2) return cuda_fail(w, "mb_autotune", e2);
    if (st2 != MB_OK) return st2;
    *best = cand[best_i];
    return MB_OK;
}

// ------------------------------------------------------------------ stages
struct mb_sort_plan {
    mb::SortScratch scratch;
    uint32_t digit_bits_max = 8;
    uint32_t* seg_blocks = nullptr;  // per-block segment counts of mb_assemble_segments
};

mb_status mb_sort_plan_create(uint32_t max_keys, uint32_t max_cells, mb_sort_plan** out) {
    if (!out) return fail(nullptr, MB_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (max_keys > mb::kMaxAgents || max_cells == 0 || max_cells > mb::kMaxCells)
        return fail(nullptr, MB_ERR_INVALID_ARG, "max_keys must be < 2^28 and max_cells in [1, 2^28]");
    mb_sort_plan* p = new (std::nothrow) mb_sort_plan();
    if (!p) return fail(nullptr, MB_ERR_OOM, "host allocation failed");
    cudaError_t e = mb::scratch_alloc(p->scratch, max_keys, max_cells);
    if (!e) e = cudaMalloc(&p->seg_blocks, sizeof(uint32_t) * (mb::segment_blocks(max_keys) + 1u));
    if (e) {
        cudaFree(p->seg_blocks);
        mb::scratch_free(p->scratch);
        delete p;
        return cuda_fail(nullptr, "mb_sort_plan_create", e);
    }
    *out = p;
    return MB_OK;
}

mb_status mb_sort_plan_destroy(mb_sort_plan* p) {
    if (!p) return MB_OK;
    cudaDeviceSynchronize();
    cudaFree(p->seg_blocks);
    mb::scratch_free(p->scratch);
    delete p;
    return MB_OK;
}

mb_status mb_sort_and_hash(mb_sort_plan* p, const uint32_t* keys, const uint32_t* vals, uint32_t n,
                           uint32_t number_of_cells, uint32_t* sorted_keys, uint32_t* sorted_vals,
                           uint32_t* start, uint32_t* close, void* cuda_stream) {
    mb::NvtxRange nvtx_range("mb_sort_and_hash");
    if (!p) return fail(nullptr, MB_ERR_INVALID_ARG, "plan is NULL");
    if (n > p->scratch.max_keys || number_of_cells == 0 || number_of_cells > p->scratch.max_cells)
        return fail(nullptr, MB_ERR_INVALID_ARG, "n or number_of_cells exceeds the plan");
    if (n && (!keys || !sorted_keys || !sorted_vals))
        return fail(nullptr, MB_ERR_INVALID_ARG, "NULL key/value buffer");
    cudaStream_t st = (cudaStream_t)cuda_stream;
    mb::SortSchedule sch = mb::make_schedule(n, number_of_cells, p->digit_bits_max);
    cudaError_t e = mb::sort_pairs(p->scratch, sch, keys, vals, sorted_keys, sorted_vals, st);
    if (e) return cuda_fail(nullptr, "mb_sort_and_hash", e);
    if ((start || close) && (e = mb::hash_ranges(p->scratch, sorted_keys, n, number_of_cells, start, close, st)))
        return cuda_fail(nullptr, "mb_sort_and_hash", e);
    return MB_OK;
}

mb_status mb_sort_plan_status(mb_sort_plan* p, void* cuda_stream) {
    if (!p) return fail(nullptr, MB_ERR_INVALID_ARG, "plan is NULL");
    uint32_t flags = 0;
    cudaError_t e = mb::sort_take_error(p->scratch, (cudaStream_t)cuda_stream, &flags);
    if (e) return cuda_fail(nullptr, "mb_sort_plan_status", e);
    if (flags)
        return fail(nullptr, MB_ERR_TIMEOUT,
                    "mb_sort_plan_status: a bounded look-back wait of the sort gave up; the results of the "
                    "plan's calls since the last status check are invalid");
    return MB_OK;
}

mb_status mb_sort_plan_selftest_stall(mb_sort_plan* p, uint32_t spin_limit, void* cuda_stream) {
    if (!p) return fail(nullptr, MB_ERR_INVALID_ARG, "plan is NULL");
    if (spin_limit == 0 || spin_limit > (1u << 20))
        return fail(nullptr, MB_ERR_INVALID_ARG, "spin_limit must be in [1, 2^20]");
    cudaError_t e = mb::sort_stall_for_test(p->scratch, spin_limit, (cudaStream_t)cuda_stream);
    if (e) return cuda_fail(nullptr, "mb_sort_plan_selftest_stall", e);
    return MB_OK;
}

mb_status mb_assemble_segments(mb_sort_plan* p, const uint32_t* sorted_keys, uint32_t n, uint32_t* segs,
                               uint32_t* key_seg_map, uint32_t* num_segs, void* cuda_stream) {
    if (!p) return fail(nullptr, MB_ERR_INVALID_ARG, "plan is NULL");
    if (n > p->scratch.max_keys) return fail(nullptr, MB_ERR_INVALID_ARG, "n exceeds the plan");
    if (!num_segs || (n && (!sorted_keys || !segs || !key_seg_map)))
        return fail(nullptr, MB_ERR_INVALID_ARG, "NULL buffer");
    cudaError_t e = mb::assemble_segments(sorted_keys, n, p->seg_blocks, segs, key_seg_map, num_segs,
                              static_cast<cudaStream_t>(cuda_stream));
    if (e) return cuda_fail(nullptr, "mb_assemble_segments", e);
    return MB_OK;
}

mb_status mb_set_profiling(mb_world* w, int enable) {
    if (!w) return fail(nullptr, MB_ERR_INVALID_ARG, "world is NULL");
    if (enable) {
        for (auto& ev : w->prof_ev) {
            if (ev) continue;
            cudaError_t e = cudaEventCreate(&ev);
            if (e) return cuda_fail(w, "mb_set_profiling", e);
        }
    }
    drop_graphs(w);
    w->profiling = enable != 0;
    return MB_OK;
}

mb_status mb_last_frame_times(mb_world* w, float* ms) {
    if (!w || !ms) return fail(w, MB_ERR_INVALID_ARG, "NULL argument");
    if (!w->profiling || !w->frame_done) return fail(w, MB_ERR_NOT_READY, "profiling off or no frame yet");
    cudaError_t e = cudaEventSynchronize(w->prof_ev[3]);
    if (e) return cuda_fail(w, "mb_last_frame_times", e);
    float t[3];
    for (int i = 0; i < 3; ++i) {
        if ((e = cudaEventElapsedTime(&t[i], w->prof_ev[i], w->prof_ev[i + 1])))
            return cuda_fail(w, "mb_last_frame_times", e);
    }
    // counting mode runs the cell-offset scan before the permutation
    ms[0] = counting(w) ? t[1] : t[0];
    ms[1] = counting(w) ? t[0] : t[1];
    ms[2] = t[2];
    return MB_OK;
}

uint32_t mb_kernels_per_frame(const mb_world* w) {
    if (!w) return 0u;
    if (fused(w)) return 1u;  // one launch per step, whatever its frame count
    // counting and rank placement: scan + scatter or rank + marked-cell fixup (idle unless the rank
    // placement fell back) + physics;
    // onesweep: histogram + one kernel per digit pass + cell offsets + gap fill + gather + physics
    return counting(w) ? 4u : (uint32_t)w->sched.passes + 5u;
}

mb_status mb_selftest_divide(uint64_t seed, uint64_t count, uint64_t* mismatches, uint32_t* first_bad) {
    if (!mismatches) return MB_ERR_INVALID_ARG;
    const cudaError_t e = mb::selftest_divide(seed, count, mismatches, first_bad);
    if (e == cudaErrorMemoryAllocation) return MB_ERR_OOM;
    return e ? MB_ERR_CUDA : MB_OK;
}

const char* mb_version(void) { return "millionsball-gb300 " __DATE__ " sm_103a"; }

}  // extern "C"
