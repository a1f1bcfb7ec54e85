/*
 * millionsball.h — C ABI of the GB300 (sm_103a) sphere-collision step library.
 *
 * This header is the drop-in boundary for the per-frame compute passes of
 * bevy_millions_ball's physics plugin.  The reference drives those passes from a
 * Bevy render-graph node once per rendered frame:
 *
 *     radix sort      bevy_radix_sort::run(.., n, 0..3, true, is_even)   src/physics/mod.rs:880-890
 *     cell ranges     spatial_hashing::run(.., n, !is_even)              src/physics/mod.rs:892-900
 *     physics         physics::run(..)   (INIT on frame 0, LOOP after)   src/physics/mod.rs:902-909, 915-956
 *
 * Here the same three stages are hand-written CUDA kernels behind a headless
 * step() call.  All functions return an mb_status and never abort the process.
 *
 * Threading: one mb_world per host thread (a world is not internally locked).
 * All device work of a world is issued on the CUDA stream given at creation;
 * mb_step() is asynchronous with respect to the host.
 */
#ifndef MILLIONSBALL_H
#define MILLIONSBALL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MB_ABI_VERSION 1u

/* Status codes.  The reference panics / unwraps on every failure
 * (src/physics/mod.rs:788-798, 930-937); this library reports instead. */
typedef enum mb_status {
    MB_OK = 0,
    MB_ERR_INVALID_ARG = 1,     /* bad pointer, size or setting                         */
    MB_ERR_OOM = 2,             /* device or host allocation failed                     */
    MB_ERR_CUDA = 3,            /* a CUDA runtime call failed (see mb_last_error)       */
    MB_ERR_TIMEOUT = 4,         /* a bounded device-side wait gave up (sort look-back or band copy) */
    MB_ERR_BUDGET_EXCEEDED = 5, /* the request does not fit the device-memory budget    */
    MB_ERR_NOT_READY = 6        /* state was never uploaded / request still running     */
} mb_status;

/* Where a caller's buffer lives. */
typedef enum mb_memory {
    MB_HOST = 0,   /* host memory (pageable or pinned); copied synchronously on the world's stream */
    MB_DEVICE = 1  /* device memory of the world's GPU; copied on the world's stream, asynchronously */
} mb_memory;

/*
 * Physics settings.  Field-for-field the reference's PhysicsPlugin /
 * PhysicsSettings (src/physics/mod.rs:53-85 and 294-363), with the same meaning:
 *
 *   max_number_of_agents            number of simulated spheres n (fixed per world,
 *                                   like the private field at mod.rs:362)
 *   number_of_grids_one_dimension   N; the grid has N*N square collision cells
 *   grid_size                       integer edge length of one cell
 *   half_map_height                 H; the box is y in [0, 2H]
 *   gravity                         acceleration, m/s^2
 *   e_envir / e_agent               restitution against the walls / other spheres
 *   k_agent / c_agent / r_agent     spring stiffness, damping and rigid threshold
 *   time_delta                      step length, seconds
 *   enable_simulation               0 makes mb_step() a no-op (mod.rs:778, 854)
 *   enable_spring                   spring response instead of rigid restitution
 *
 * The reference bakes every real-valued setting into its shaders as
 * (value * 1000) truncated to an integer and divides by 1000 again on the GPU
 * (mod.rs:460-484, physics.wgsl:7-16); so dt = 1/60 runs as 0.016.  This library
 * applies exactly that quantisation unless `exact_constants` is set, in which
 * case the f32 values are used as given (no counterpart in the reference).
 */
typedef struct mb_settings {
    uint32_t max_number_of_agents;
    uint32_t number_of_grids_one_dimension;
    uint32_t grid_size;
    uint32_t half_map_height;
    float gravity[3];
    float e_envir;
    float e_agent;
    float k_agent;
    float c_agent;
    float r_agent;
    float time_delta;
    uint8_t enable_simulation;
    uint8_t enable_spring;
    uint8_t exact_constants;
    uint8_t reserved0;
} mb_settings;

/* PhysicsPlugin::default() (src/physics/mod.rs:87-109). */
void mb_settings_default(mb_settings* out);

/*
 * Constants exactly as the kernels use them after quantisation
 * (CompiledConsts::shader_defs, src/physics/mod.rs:459-485; physics.wgsl:2-16).
 */
typedef struct mb_consts {
    uint32_t number_of_grids_one_dimension;
    uint32_t grid_size;
    float half_map_height;   /* HALF_MAP_HEIGHT */
    float half_map_size;     /* HALF_MAP_SIZE = f32(N * grid_size / 2) */
    float gravity[3];
    float e_envir, e_agent, k_agent, c_agent, r_agent, time_delta;
    uint32_t enable_spring;
} mb_consts;

mb_status mb_quantize_settings(const mb_settings* s, mb_consts* out);

/* ------------------------------------------------------------------------- */
/* World: one scene, resident in device memory.                               */
/* ------------------------------------------------------------------------- */
typedef struct mb_world mb_world;

/*
 * Create a world for s->max_number_of_agents spheres on the current CUDA device.
 * `cuda_stream` is a cudaStream_t (NULL = the legacy default stream).  Replaces
 * PhysicsPlugin::build + create_shader_storage_buffers + RadixSortPlugin buffer
 * set-up (src/physics/mod.rs:111-125, 241-292).
 */
mb_status mb_create(const mb_settings* s, void* cuda_stream, mb_world** out);
mb_status mb_destroy(mb_world* w);

/*
 * Replace the runtime settings (the egui path, src/main.rs:155-210 and the
 * recompile at src/physics/mod.rs:808-837).  No recompilation: settings are
 * kernel parameters.  max_number_of_agents cannot change (mod.rs:362).
 */
mb_status mb_set_settings(mb_world* w, const mb_settings* s);
mb_status mb_get_settings(const mb_world* w, mb_settings* out);

/*
 * Upload n = max_number_of_agents agent states.
 *   pos_scale : n x float4  (x, y, z, radius)            physics.wgsl:25 position_with_scale
 *   vfme      : n x uint4   f16 pairs (vx,vy) (vz,fx)    physics.wgsl:26 packed_vfme,
 *                           (fy,fz) (mass,0); velocity is the displacement per step
 * The frame counter restarts: the next step is the INIT frame (mod.rs:929-933),
 * which reorders nothing and only emits cell keys.
 */
mb_status mb_set_state(mb_world* w, const float* pos_scale, const uint32_t* vfme, mb_memory where);

/* Download the current state, in the current slot (sorted-cell) order. */
mb_status mb_get_state(mb_world* w, float* pos_scale, uint32_t* vfme, mb_memory where);

/* Advance k frames (sort -> cell ranges -> physics per frame).  Asynchronous. */
mb_status mb_step(mb_world* w, uint32_t k);

/* Wait for the world's stream; reports a device-side timeout as MB_ERR_TIMEOUT. */
mb_status mb_sync(mb_world* w);

/*
 * Debug view of the last frame, each array optional (NULL = skip):
 *   keys  : n  u32  unsorted cell keys emitted by the last physics pass (the next sort's input)
 *   perm  : n  u32  sorted permutation of the last frame (old slot of each sorted slot)
 *   start : N*N u32 first sorted slot of each cell, 0xFFFFFFFF if the cell is empty
 *   close : N*N u32 last sorted slot of each cell (inclusive); 0xFFFFFFFF if empty
 * start/close follow spatial_hashing.wgsl:29-70 (ZEROING + HASHING).
 */
mb_status mb_get_debug(mb_world* w, uint32_t* keys, uint32_t* perm, uint32_t* start,
                       uint32_t* close, mb_memory where);

/*
 * Device pointers of the current state (headless replacement of the buffer
 * handles the renderer binds, src/physics/mod.rs:40-51 and
 * src/custom_materials/physics_ball/mod.rs:709-740).  Valid until the next
 * mb_step / mb_set_state / mb_destroy on this world.
 */
mb_status mb_device_buffers(mb_world* w, const float** pos_scale, const uint32_t** vfme);

/* Frames run since the last mb_set_state (PhysicsBindGroup::time, mod.rs:711-743). */
int64_t mb_time(const mb_world* w);

/* Last error message of this world ("" if none).  Pass NULL for process-wide errors. */
const char* mb_last_error(const mb_world* w);

/* ------------------------------------------------------------------------- */
/* Stage entry points (device pointers, caller's stream).                     */
/* ------------------------------------------------------------------------- */

/*
 * Stable key/index sort followed by the cell-range build: what one frame runs
 * before physics (bevy_radix_sort::run, src/physics/mod.rs:880-890, then
 * spatial_hashing::run, src/physics/spatial_hashing.rs:191-243).  The reference's
 * own test drives exactly this pair (spatial_hashing.rs:408-600).
 *
 *   keys        : n u32, every key < number_of_cells
 *   vals        : n u32 or NULL; NULL sorts the identity 0..n-1 (the `true`
 *                 argument at mod.rs:888)
 *   sorted_keys, sorted_vals : n u32 outputs
 *   start, close: number_of_cells u32 outputs (as in mb_get_debug); either may be NULL
 *
 * Scratch comes from a plan sized by mb_sort_plan_create (max keys, max cells).
 */
typedef struct mb_sort_plan mb_sort_plan;
mb_status mb_sort_plan_create(uint32_t max_keys, uint32_t max_cells, mb_sort_plan** out);
mb_status mb_sort_plan_destroy(mb_sort_plan* p);
mb_status mb_sort_and_hash(mb_sort_plan* p, const uint32_t* keys, const uint32_t* vals, uint32_t n,
                           uint32_t number_of_cells, uint32_t* sorted_keys, uint32_t* sorted_vals,
                           uint32_t* start, uint32_t* close, void* cuda_stream);

/*
 * Status of a plan's sorts (the reference panics where a pass fails,
 * src/physics/mod.rs:788-798; this reports instead).  Every wait of the sort's
 * decoupled look-back is bounded: a wait that gives up sets an error word in the
 * plan and the call's results are invalid.  mb_sort_plan_status waits for
 * `cuda_stream`, reads and clears that word, and returns MB_ERR_TIMEOUT if it was
 * set (the next sort then starts from a cleared look-back table), else MB_OK.
 * Allocates nothing.
 */
mb_status mb_sort_plan_status(mb_sort_plan* p, void* cuda_stream);

/*
 * Diagnostic (no counterpart in the reference): makes one look-back wait of the
 * plan's sort run out on purpose - a lone block takes the second tile of a pass
 * whose first tile never publishes - with a wait limit of spin_limit polls
 * (1 .. 2^20), so that the timeout path can be tested without a fault: the block
 * gives up, sets the plan's error word and exits; mb_sort_plan_status then
 * returns MB_ERR_TIMEOUT.  Synchronous.  Writes nothing the caller owns.
 */
mb_status mb_sort_plan_selftest_stall(mb_sort_plan* p, uint32_t spin_limit, void* cuda_stream);

/*
 * Compacted segment table of sorted keys, the reference's segment assembly
 * (src/physics/assemble_segs.rs:314-430, assemble_segs.wgsl): each run of equal
 * keys in sorted_keys[0..n) is one segment, in slot order.  Device pointers:
 *   segs        : receives the first slot of every segment (at most n entries)
 *   key_seg_map : key_seg_map[key] = its segment, for every key that occurs
 *                 (entries of absent keys are left as they were; the map must
 *                 hold max key + 1 entries)
 *   num_segs    : one u32, receives the number of segments (0 for n = 0)
 * Scratch comes from the plan (n <= its max_keys).
 */
mb_status mb_assemble_segments(mb_sort_plan* p, const uint32_t* sorted_keys, uint32_t n, uint32_t* segs,
                               uint32_t* key_seg_map, uint32_t* num_segs, void* cuda_stream);

/*
 * mb_sort_and_hash without any device allocation (no counterpart in the
 * reference).  For callers that may not allocate device memory where they issue
 * GPU work: a frame loop that forbids allocation after start-up (allocator
 * stalls cause frame-time spikes and break fixed memory budgets), or code
 * recording into a CUDA stream capture, where cudaMalloc cannot be recorded.
 * Same arguments and results as mb_sort_and_hash minus the plan: the scratch is
 * one fixed array inside the library (about 3.5 MB on every GPU that loads it).
 *   - n <= MB_STATIC_MAX_KEYS and 1 <= number_of_cells <= MB_STATIC_MAX_CELLS,
 *     else MB_ERR_INVALID_ARG (message via mb_last_error(NULL));
 *   - the first call on a device sets the scratch up (looks up its device
 *     address and zeroes it on `cuda_stream`): make that first call before any
 *     stream capture;
 *   - all calls on a device share the scratch and it keeps the last call's
 *     contents: calls that overlap on the GPU race and corrupt each other, so
 *     order them (e.g. issue them on one stream).
 */
#define MB_STATIC_MAX_KEYS 262144u
#define MB_STATIC_MAX_CELLS 262144u
mb_status mb_sort_and_hash_static(const uint32_t* keys, const uint32_t* vals, uint32_t n,
                                  uint32_t number_of_cells, uint32_t* sorted_keys, uint32_t* sorted_vals,
                                  uint32_t* start, uint32_t* close, void* cuda_stream);
/* mb_sort_plan_status for the fixed scratch of mb_sort_and_hash_static on the
 * current device (MB_OK if no call ran there yet).  Allocates nothing. */
mb_status mb_sort_static_status(void* cuda_stream);

/* Per-world kernel choices (the autotuner's knobs). */
typedef struct mb_tuning {
    uint32_t digit_bits_max;   /* widest radix digit of the onesweep sort, 4..11 */
    uint32_t collide_block;    /* sorted slots per thread block of the physics pass: 64, 128
                                  (default) or 256; MB_FRAME_FUSED frames run 128 */
    uint32_t sort_algorithm;   /* MB_SORT_RANK (default), MB_SORT_COUNTING or MB_SORT_ONESWEEP */
    uint32_t frames_per_launch; /* LOOP frames captured per graph launch in multi-frame steps:
                                   1, 2, 4, 8 (default; 0 reads as 8) or 16 */
    uint32_t state_gather;     /* MB_GATHER_COPY or MB_GATHER_INDIRECT (below) */
    uint32_t frame_kernel;     /* MB_FRAME_GRAPH or MB_FRAME_FUSED (below) */
    uint32_t scatter_agents;   /* spheres each thread of the counting sort's scatter (or of the
                                  rank placement) takes: 1 (default; 0 reads as 1), 2 or 4;
                                  MB_FRAME_FUSED frames run 1 */
    uint32_t reserved;
} mb_tuning;

/* How LOOP frames are launched:
 *   MB_FRAME_GRAPH: one kernel per stage (count scan, rank placement or scatter,
 *                   marked-cell fixup, physics), captured in CUDA graphs (default);
 *   MB_FRAME_FUSED: every stage of every frame of an mb_step call in one
 *                   cooperative kernel, the stages separated by grid barriers
 *                   (bounded waits: a barrier that gives up is reported by
 *                   mb_sync as MB_ERR_TIMEOUT).  MB_SORT_COUNTING only; with
 *                   profiling on, frames run as MB_FRAME_GRAPH.
 * Both give identical results. */
#define MB_FRAME_GRAPH 0u
#define MB_FRAME_FUSED 1u

/* How the physics pass reads the state in this frame's sorted order:
 *   MB_GATHER_COPY:     the sort writes a sorted copy of the state (32 B per
 *                       sphere); the physics pass copies its tile's neighbour
 *                       bands from it with bulk copies;
 *   MB_GATHER_INDIRECT: the sort writes only the permutation; the physics pass
 *                       gathers its bands (and its own spheres) through it.
 * Both give identical results. */
#define MB_GATHER_COPY 0u
#define MB_GATHER_INDIRECT 1u

/* Frame sort: all three produce the identical stable permutation and cell ranges.
 *   MB_SORT_COUNTING: per-cell counts (emitted by the previous physics pass) ->
 *                     scan = cell offsets -> scatter -> in-cell fixup
 *   MB_SORT_ONESWEEP: onesweep LSD radix sort of the keys, then the cell-offset build
 *   MB_SORT_RANK:     counts -> scan -> each sphere placed at its cell's offset plus
 *                     its rank among the spheres of its new cell in its old 3 x 3
 *                     cell neighbourhood (no atomics, no fixup); spheres that moved
 *                     more than one cell are listed by the physics pass and ranked
 *                     from the list (up to 256 per frame; beyond that, and in the
 *                     first LOOP frame after an upload, a grid change or a tuning
 *                     change, the frame runs the MB_SORT_COUNTING scatter and fixup) */
#define MB_SORT_COUNTING 0u
#define MB_SORT_ONESWEEP 1u
#define MB_SORT_RANK 2u
mb_status mb_get_tuning(const mb_world* w, mb_tuning* out);
mb_status mb_set_tuning(mb_world* w, const mb_tuning* t);

/*
 * Headless sphere-impostor render of the current state (the reference draws the
 * spheres with src/custom_materials/physics_ball/deferred_physics_ball.wgsl and
 * src/custom_materials/sdf.wgsl through Bevy's renderer): an orthographic view
 * straight down onto the x/z window [x0, x1) x [z0, z1), width x height pixels,
 * row v covering z = z0 + (v + 0.5)(z1 - z0)/height.  Per pixel the highest
 * sphere surface (radius grown near the floor as the shader does) is marched 16
 * steps on the smooth maximum (k = 0.08) of the sphere's and the floor's signed
 * distances and lit by one directional light.  rgba: width*height u32 (R in the
 * low byte, A = 255); height_map (nullable): width*height f32 surface heights
 * (0 for the floor).  where: MB_DEVICE (device pointers, asynchronous on the
 * world's stream) or MB_HOST (copied back, synchronous).  Keeps a per-world
 * 8-byte-per-pixel depth buffer, grown on demand (allocates).
 */
mb_status mb_render_topdown(mb_world* w, uint32_t width, uint32_t height, float x0, float z0, float x1, float z1,
                            uint32_t* rgba, float* height_map, mb_memory where);

/*
 * The same impostors seen through a perspective camera: by default the
 * reference's own view (src/main.rs:65-89: eye (0, 64, 64) looking at the
 * origin with +y up, Bevy's default 45-degree vertical field of view, clear
 * colour sRGB (248, 151, 184), its directional light); eye / target (nullable,
 * 3 floats each) and fov_y_degrees (> 0) override it.  Per pixel the nearest
 * sphere along the pixel's ray is marched and its normal taken as the shader
 * does; the light is a GGX lobe (the material's roughness 0.435, F0 0.04) plus
 * Lambert and ambient terms standing in for Bevy's PBR pass, sRGB-encoded; the
 * box interior (base colour 0.8, 0.7, 0.6) shows behind the spheres.  rgba:
 * width*height u32 (R in the low byte, A = 255); depth (nullable): distance
 * along each pixel's ray (0 where only the clear colour shows).  The view
 * direction must not be vertical.  where and buffers as for mb_render_topdown.
 */
mb_status mb_render_view(mb_world* w, uint32_t width, uint32_t height, const float* eye, const float* target,
                         float fov_y_degrees, uint32_t* rgba, float* depth, mb_memory where);

/*
 * Autotuner (no counterpart in the reference, whose sort and passes have fixed
 * workgroup shapes, NUMBER_OF_THREADS_PER_WORKGROUP = 256 at src/physics/mod.rs:35).
 * Times every candidate tuning on the world's own scene for `frames` LOOP frames
 * each (CUDA events on the world's stream, one warm-up frame per candidate):
 * twenty-four combinations of the sort (rank placement, counting, or onesweep
 * with 6-, 8- or 11-bit digits), frames per graph launch (1, 8, 16), state gather
 * (sorted copy or through the permutation), frame kernel (per-stage graph or
 * fused), physics tile (64, 128 or 256 slots per thread block) and spheres per
 * thread of the scatter or the rank placement (1, 2, 4).  The world's
 * state, keys, permutation, cell ranges and time are saved first and restored
 * afterwards, so the simulation continues exactly as if the tuner had not run.
 * The fastest candidate is applied and written to *best; frame_ms (nullable,
 * MB_TUNE_CANDIDATES entries) receives each candidate's mean frame time, in the
 * order of tried[] (nullable, same length).  Needs a frame to have run since the
 * last upload (MB_ERR_NOT_READY otherwise).  Allocates temporary device memory.
 */
#define MB_TUNE_CANDIDATES 24u
mb_status mb_autotune(mb_world* w, uint32_t frames, mb_tuning* best, float* frame_ms, mb_tuning* tried);

/*
 * Per-stage device timing (no counterpart in the reference, which only labels
 * its passes, src/physics/mod.rs:925).  With profiling on, every frame records
 * CUDA events around its three stages; mb_last_frame_times waits for the most
 * recent frame and reports milliseconds: [0] sort (histogram + digit passes),
 * [1] cell-range build, [2] physics pass.  Enabling or disabling re-captures the
 * frame graphs.
 */
mb_status mb_set_profiling(mb_world* w, int enable);
mb_status mb_last_frame_times(mb_world* w, float* stage_ms3);

/* Kernels one frame launches (graph nodes that are kernels). */
uint32_t mb_kernels_per_frame(const mb_world* w);

/* ------------------------------------------------------------------------- */
/* Batching: many independent scenes, one set of launches per frame.         */
/* No counterpart in the reference (one scene per app).                       */
/* ------------------------------------------------------------------------- */
/*
 * A batch is a pool of scenes sharing device buffers; every frame sorts, builds
 * cell ranges and runs physics for all of them at once, and each scene evolves
 * exactly as it would in its own mb_world (same state, keys, order, bit for
 * bit).  Per frame each scene runs its own mode: LOOP, INIT (its first frame
 * after mb_batch_set_state) or HOLD (inactive: state kept, nothing advances).
 *
 *   mb_batch_create    scenes[0..num_scenes) plus room for later
 *                      mb_batch_add_scene calls (capacity_* >= the initial sum,
 *                      capacity_cells counted as N*N per scene; 0 = just the
 *                      initial scenes)
 *   mb_batch_step      k frames for every active scene with a state
 *   mb_batch_get_debug slot-local keys / perm / start / close of one scene (as of
 *                      its last frame; a held scene is not touched at all)
 */
typedef struct mb_batch mb_batch;
mb_status mb_batch_create(const mb_settings* scenes, uint32_t num_scenes, uint32_t capacity_agents,
                          uint32_t capacity_cells, uint32_t capacity_scenes, void* cuda_stream,
                          mb_batch** out);
mb_status mb_batch_add_scene(mb_batch* b, const mb_settings* s, uint32_t* scene_index);
mb_status mb_batch_destroy(mb_batch* b);
uint32_t mb_batch_num_scenes(const mb_batch* b);
mb_status mb_batch_memory(const mb_batch* b, uint64_t* device_bytes);
mb_status mb_batch_set_state(mb_batch* b, uint32_t scene, const float* pos_scale, const uint32_t* vfme,
                             mb_memory where);
mb_status mb_batch_get_state(mb_batch* b, uint32_t scene, float* pos_scale, uint32_t* vfme, mb_memory where);
mb_status mb_batch_set_active(mb_batch* b, uint32_t scene, int active);
mb_status mb_batch_step(mb_batch* b, uint32_t k);
mb_status mb_batch_sync(mb_batch* b);
int64_t mb_batch_time(const mb_batch* b, uint32_t scene);
mb_status mb_batch_get_debug(mb_batch* b, uint32_t scene, uint32_t* keys, uint32_t* perm, uint32_t* start,
                             uint32_t* close, mb_memory where);

/*
 * Kernel choices of a batch (the knobs of mb_tuning that apply to a pool):
 * sort_algorithm (MB_SORT_RANK, the default: frames in which every scene is
 * in LOOP place spheres by rank, other frames claim and fix; or
 * MB_SORT_COUNTING: every frame claims and fixes), frames_per_launch (frames
 * captured per graph launch while no scene changes mode: 1, 2, 4, 8 (default)
 * or 16), collide_block (physics tile: 64, 128 (default) or 256 slots) and
 * scatter_agents (spheres per thread of the counting scatter: 1, 2 or 4).  The
 * other fields must keep their defaults (sorted copy, per-stage kernels).
 *
 * mb_batch_autotune: the world autotuner's counterpart for a pool (no
 * counterpart in the reference, whose passes have fixed workgroup shapes,
 * src/physics/mod.rs:35): times rank placement with frames_per_launch
 * {1, 8, 16} x collide_block {64, 128, 256}, then the counting sort with
 * scatter_agents 1, 2 and 4 at 8 frames per launch and 128-slot tiles, on the
 * pool's own scenes for `frames` frames each (one warm-up
 * frame per candidate), restoring every scene's state, keys, order, cell ranges
 * and time before each and at the end, then applies the fastest.  Every scene
 * needs a frame since its upload.  frame_ms / tried (nullable) receive
 * MB_BATCH_TUNE_CANDIDATES entries.  Allocates temporary device memory.
 */
#define MB_BATCH_TUNE_CANDIDATES 12u
mb_status mb_batch_get_tuning(const mb_batch* b, mb_tuning* out);
mb_status mb_batch_set_tuning(mb_batch* b, const mb_tuning* t);
mb_status mb_batch_autotune(mb_batch* b, uint32_t frames, mb_tuning* best, float* frame_ms, mb_tuning* tried);

/* ------------------------------------------------------------------------- */
/* Serving: a request loop over one batch pool (no counterpart in the         */
/* reference).                                                                */
/* ------------------------------------------------------------------------- */
/*
 * Requests are submitted from any thread and run by a worker thread:
 *   create  - admitted in arrival order while the memory budget has room (the
 *             pool's spheres / cells / scenes are reserved at mb_server_create);
 *             scenes stay resident, so one that does not fit is rejected
 *             (MB_ERR_BUDGET_EXCEEDED), and so are later requests on it;
 *   advance - k more frames for a scene.
 * Requests that arrive while frames run join at the next frame (continuous
 * batching); each frame advances every scene that owes a step.  A request is
 * done when its scene has taken its steps; latency = done - submitted.
 */
typedef struct mb_server_config {
    uint64_t budget_bytes;   /* device memory the pool may take */
    uint32_t max_scenes;
    uint32_t max_agents;     /* 0: derived from the budget */
    uint32_t max_cells;      /* 0: derived from the budget */
    uint32_t reserved[3];
} mb_server_config;

typedef struct mb_server_stats {
    uint64_t requests_done;
    uint64_t frames;
    uint64_t agent_steps;    /* sphere-steps taken by LOOP frames */
    double busy_seconds;     /* wall time with frames on the GPU */
    uint32_t scenes;
    uint32_t reserved[3];
} mb_server_stats;

typedef struct mb_server mb_server;
mb_status mb_server_create(const mb_server_config* cfg, void* cuda_stream, mb_server** out);
mb_status mb_server_destroy(mb_server* s);
mb_status mb_server_submit_create(mb_server* s, const mb_settings* settings, const float* pos_scale,
                                  const uint32_t* vfme, uint32_t* scene, uint64_t* request);
mb_status mb_server_submit_advance(mb_server* s, uint32_t scene, uint32_t k, uint64_t* request);
/* MB_ERR_NOT_READY if the request is not done within timeout_s (it stays queued). */
mb_status mb_server_wait(mb_server* s, uint64_t request, double timeout_s, double* latency_s);
/* Waits until the scene owes no step, then copies its state to host memory. */
mb_status mb_server_get_state(mb_server* s, uint32_t scene, float* pos_scale, uint32_t* vfme);
mb_status mb_server_get_stats(mb_server* s, mb_server_stats* out);

/* Diagnostic: compares the physics pass's division (an exact reciprocal
 * multiply for power-of-two divisors, IEEE division otherwise) with IEEE
 * division on `count` generated operand pairs on the current device; *mismatches = the
 * number of differing results (0 expected), first_bad (nullable, 4 words) =
 * the first mismatch's a, d, result, IEEE result as float bit patterns.
 * Synchronous. */
mb_status mb_selftest_divide(uint64_t seed, uint64_t count, uint64_t* mismatches, uint32_t* first_bad);

/* Library version string (build id). */
const char* mb_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MILLIONSBALL_H */
