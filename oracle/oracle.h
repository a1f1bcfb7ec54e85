/*
 * oracle.h — CPU restatement of bevy_millions_ball's per-frame physics passes.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the correctness oracle: the checker that the
 * CUDA library is compared against, and the timed CPU baseline of the benchmark.
 * The product (libmillionsball) never links, loads or calls it.
 *
 * What it restates (paths relative to the reference project):
 *   - src/physics/physics.wgsl:57-337      INIT / LOOP physics pass, every helper
 *   - src/physics/spatial_hashing.wgsl:29-70  ZEROING + HASHING (cell ranges)
 *   - src/physics/mod.rs:460-484           x1000 constant quantisation
 *   - src/physics/mod.rs:214-239           f16 packing of velocity / force / mass
 *   - src/physics/mod.rs:659-705, 929-939  ping-pong routing, INIT on frame 0
 *   - bevy_radix_sort 0.15.0 (crates.io, not vendored) as called at mod.rs:880-890:
 *     a stable LSD key/value sort over 8-bit digits with values = 0..n-1.
 *
 * Parity status: the sort + cell-range half is pinned against the reference's own
 * known-answer test (src/physics/spatial_hashing.rs:536-632, restated under
 * tests/golden/).  The physics half has no golden vectors in the reference and the
 * reference cannot run here (Rust/wgpu), so it is "parity unpinned" against the
 * reference itself; it is cross-checked against a second, independent Python
 * restatement and against analytic known answers.
 *
 * Floating-point model: IEEE-754 binary32, round-to-nearest-even, no contraction
 * (built with -ffp-contract=off), WGSL built-ins restated from their definitions
 * (length = sqrt(dot), normalize = v / length, clamp = min(max())), f32->f16 RNE.
 */
#ifndef MB_ORACLE_H
#define MB_ORACLE_H

#include <stdint.h>

#include "../include/millionsball.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mbo_world mbo_world;

/* Quantised constants (CompiledConsts, mod.rs:459-485). Returns 0 on success. */
int mbo_quantize(const mb_settings* s, mb_consts* out);

/* f32 <-> f16, IEEE round-to-nearest-even (pack2x16float / unpack2x16float). */
uint16_t mbo_f32_to_f16(float f);
float mbo_f16_to_f32(uint16_t h);

/* Cell key of a position (physics.wgsl:107-117). */
uint32_t mbo_cell_key(const mb_consts* c, float x, float z);

/* hash3f1u (physics.wgsl:334-337). */
void mbo_hash3f1u(uint32_t n, float out[3]);

/* Stable LSD radix sort, 8-bit digits, `passes` passes from the least
 * significant digit; vals == NULL sorts 0..n-1.  threads <= 0: all cores. */
void mbo_radix_sort(const uint32_t* keys, const uint32_t* vals, uint32_t n, uint32_t passes,
                    uint32_t* keys_out, uint32_t* vals_out, int threads);

/* ZEROING over all number_of_cells cells, then HASHING over the sorted keys.
 * close[] of an empty cell is written 0xFFFFFFFF (the reference leaves it stale
 * and never reads it). */
void mbo_spatial_hash(const uint32_t* sorted_keys, uint32_t n, uint32_t number_of_cells,
                      uint32_t* start, uint32_t* close);

/* One physics pass (INIT if init != 0, else LOOP) over n sorted slots. */
void mbo_physics(const mb_consts* c, int init, uint32_t n, const uint32_t* perm,
                 const uint32_t* start, const uint32_t* close, const float* pos_in,
                 const uint32_t* vfme_in, float* pos_out, uint32_t* vfme_out,
                 uint32_t* keys_out, int threads);

/* A whole scene with the reference's frame semantics. */
mbo_world* mbo_create(const mb_settings* s);
void mbo_destroy(mbo_world* w);
int mbo_set_settings(mbo_world* w, const mb_settings* s);
int mbo_set_state(mbo_world* w, const float* pos_scale, const uint32_t* vfme);
int mbo_get_state(const mbo_world* w, float* pos_scale, uint32_t* vfme);
int mbo_step(mbo_world* w, uint32_t k, int threads);
int mbo_get_debug(const mbo_world* w, uint32_t* keys, uint32_t* perm, uint32_t* start,
                  uint32_t* close);
int64_t mbo_time(const mbo_world* w);
int mbo_hardware_threads(void);

/* Top-down impostor render (deferred_physics_ball.wgsl + sdf.wgsl per-pixel
 * math, orthographic view down -y onto [x0, x1) x [z0, z1)): rgba u32 and
 * surface height per pixel; winner (nullable) = sphere index + 1, 0 = floor. */
void mbo_render_topdown(const float* pos4, uint32_t n, uint32_t w, uint32_t h, float x0, float z0, float x1,
                        float z1, uint32_t* rgba, float* height, uint32_t* winner);

#ifdef __cplusplus
}
#endif

#endif
