// mb_physics.cu — INIT / LOOP physics pass (fused Verlet + neighbour-stencil
// contacts + jitter + wall constraint + f16 pack + next cell key).
//
// Restates src/physics/physics.wgsl:57-337 as CUDA for sm_103a.  This translation
// unit is compiled with --fmad=false and IEEE division / square root so every
// arithmetic step rounds exactly like the WGSL expression it follows; with that,
// positions, packed velocities and keys are bit-identical to the CPU oracle.
//
// Neighbour ranges come from cell offsets (offs[c] = number of agents in cells
// < c): the reference's three-cell merge with its INVALID-skipping logic
// (physics.wgsl:122-147, 171-206) always yields [offs[first], offs[last + 1]),
// because empty cells have zero width.

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "mb_count_dev.cuh"
#include "mb_internal.h"

namespace mb {
namespace {

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ V3 splat(float s) { return {s, s, s}; }
__device__ __forceinline__ float dot3(V3 a, V3 b) {
    float xx = a.x * b.x;
    float yy = a.y * b.y;
    float zz = a.z * b.z;
    return (xx + yy) + zz;
}
__device__ __forceinline__ float len3(V3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ V3 normalize3(V3 a) { return a / len3(a); }

// WGSL clamp(e, lo, hi) = min(max(e, lo), hi), with min/max defined as "e2 if
// e2 < e1 (resp. >), else e1; a NaN operand yields the other".  The hardware
// min/max (fminf/fmaxf) return the same value at every call site here: they
// also return the non-NaN operand, and they differ only for min(+0, -0) and
// max(-0, +0), argument orders that cannot occur with the bounds used below
// (+-65504, [-(r*R_AGENT), +0], +-edge with edge >= +0).
__device__ __forceinline__ float wclamp(float e, float lo, float hi) { return fminf(fmaxf(e, lo), hi); }
__device__ __forceinline__ float wsign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }

struct Agent {  // physics.wgsl:208-215
    V3 position;
    float scale;
    V3 velocity;
    float massv;
    V3 force;
};

__device__ __forceinline__ float h2f(uint32_t bits16) {
    return __half2float(__ushort_as_half((unsigned short)bits16));
}
__device__ __forceinline__ uint32_t f2h(float f) { return (uint32_t)__half_as_ushort(__float2half_rn(f)); }

// agent_new + unpack_vfme (physics.wgsl:217-233, 244-253)
__device__ __forceinline__ Agent unpack(float4 p, uint4 q) {
    Agent a;
    a.position = {p.x, p.y, p.z};
    a.scale = p.w;
    a.velocity = {h2f(q.x & 0xFFFFu), h2f(q.x >> 16), h2f(q.y & 0xFFFFu)};
    a.force = {h2f(q.y >> 16), h2f(q.z & 0xFFFFu), h2f(q.z >> 16)};
    a.massv = h2f(q.w & 0xFFFFu);
    return a;
}

// A neighbour as the spring response reads it (solve_sphere_constraint's
// spring branch, physics.wgsl:320-330, uses its position and scale only).
__device__ __forceinline__ Agent unpack_pos(float4 p) {
    Agent a;
    a.position = {p.x, p.y, p.z};
    a.scale = p.w;
    a.velocity = splat(0.0f);
    a.force = splat(0.0f);
    a.massv = 0.0f;
    return a;
}

// pack_vfme (physics.wgsl:235-242)
__device__ __forceinline__ uint4 pack(const Agent& a) {
    uint4 q;
    q.x = f2h(a.velocity.x) | (f2h(a.velocity.y) << 16);
    q.y = f2h(a.velocity.z) | (f2h(a.force.x) << 16);
    q.z = f2h(a.force.y) | (f2h(a.force.z) << 16);
    q.w = f2h(a.massv) | (f2h(0.0f) << 16);
    return q;
}

// n / d for the grid size d, exact for every u32 n (Granlund-Montgomery
// multiply-shift with a 33-bit magic, as set up by make_params).
__device__ __forceinline__ uint32_t div_grid(const PhysParams& P, uint32_t n) {
    uint32_t t = __umulhi(P.div_m, n);
    return (t + ((n - t) >> P.div_s1)) >> P.div_s2;
}

// get_collision_grid_id (physics.wgsl:107-109): saturating f32->u32, integer
// division by GRID_SIZE; clamped to the border cell for positions off the map.
__device__ __forceinline__ void cell_of(const PhysParams& P, float x, float z, uint32_t& cx,
                                        uint32_t& cz) {
    cx = div_grid(P, __float2uint_rz(x + P.half_map_size));
    cz = div_grid(P, __float2uint_rz(z + P.half_map_size));
    cx = min(cx, P.N - 1u);
    cz = min(cz, P.N - 1u);
}

// v / d.  When d is a power of two whose reciprocal is a normal float (unit
// masses, or equal masses in den = 2m), v * (1/d) is the same real number as
// v / d, so it rounds to the same float: three multiplies replace three IEEE
// divisions.  Otherwise IEEE division.  (A reciprocal with one checked
// correction step per numerator was exact too, but slower than IEEE division
// here: 74 vs 58 us per late 1M frame.)  mb_selftest_divide compares this with
// IEEE division on the GPU.
__device__ __forceinline__ V3 div_exact(V3 v, float d) {
    const uint32_t bits = __float_as_uint(d), e = (bits >> 23) & 0xFFu;
    if ((bits & 0x007FFFFFu) == 0u && e >= 1u && e <= 253u) {
        const float r = __uint_as_float((bits & 0x80000000u) | ((254u - e) << 23));
        return {v.x * r, v.y * r, v.z * r};
    }
    return v / d;
}

// length(v) > s (the jitter test, physics.wgsl:162-168).  sqrt is correctly
// rounded and monotone, so where dot(v, v) is below s^2 * (1 - 1e-5) or above
// s^2 * (1 + 1e-5) (products rounded once each, far inside the margin) the
// rounded length is certainly <= s, resp. > s; in between, and for s outside
// [2^-63, 2^63] or not positive, the length is computed.  The usual case, a
// sphere moved by less than its radius, needs no square root.
__device__ __forceinline__ bool longer_than(V3 v, float s) {
    const float d = dot3(v, v);  // the dot length() rounds
    const uint32_t es = (__float_as_uint(s) >> 23) & 0xFFu;
    if (s > 0.0f && es >= 64u && es <= 190u) {
        const float s2 = s * s;
        if (d < s2 * 0.99999f) return false;
        if (d > s2 * 1.00001f) return true;
    }
    return sqrtf(d) > s;
}

// Response model of a kernel instantiation: rigid, spring, or read from the
// parameters at run time (batches mix scenes of both).
enum : int { kRigid = 0, kSpring = 1, kSpringRuntime = 2 };
template <int kResp>
__device__ __forceinline__ bool spring_of(const PhysParams& P) {
    return kResp == kSpringRuntime ? P.spring != 0u : kResp == kSpring;
}

// solve_sphere_constraint (physics.wgsl:300-331)
template <int kResp>
__device__ __forceinline__ void sphere(const PhysParams& P, Agent& a, const Agent& b) {
    float edge = b.scale + a.scale;
    V3 tpos = a.position - b.position;
    float dist = len3(tpos);
    if (dist <= edge) {
        V3 norm = normalize3(tpos);
        if (!spring_of<kResp>(P)) {
            float m1 = a.massv, m2 = b.massv;
            V3 rvel = a.velocity - b.velocity;
            float rspd = dot3(rvel, norm);
            if (rspd < 0.0f) {
                V3 rvel_n = rspd * norm;
                float e_m2 = P.e_agent * m2;
                float num = m1 - e_m2;
                float den = m1 + m2;
                V3 rvel_c = div_exact(num * rvel_n, den);
                a.velocity = (b.velocity + (rvel - rvel_n)) + rvel_c;
            }
            float h = 0.5f * (edge - dist);
            a.position = a.position + h * norm;
        } else {
            float makeup = edge - dist;
            V3 kforce = (P.k_agent * makeup) * norm;
            V3 cforce = P.neg_c_over_dt * a.velocity;
            a.force = a.force + (kforce + cforce);
            float limit = makeup - P.r_agent * a.scale;
            if (limit > 0.0f) {
                a.position = a.position + limit * norm;
            }
        }
    }
}

// solve_cube_constraint (physics.wgsl:269-298)
template <int kResp>
__device__ __forceinline__ void cube(const PhysParams& P, Agent& a) {
    V3 edge = V3{P.half_map_size, P.half_map_height, P.half_map_size} - splat(a.scale);
    V3 cetr = {0.0f, P.half_map_height, 0.0f};
    V3 tpos = a.position - cetr;
    V3 makeup = {edge.x - fabsf(tpos.x), edge.y - fabsf(tpos.y), edge.z - fabsf(tpos.z)};
    bool tx = makeup.x < 0.0f, ty = makeup.y < 0.0f, tz = makeup.z < 0.0f;
    if (!(tx || ty || tz)) return;
    if (!spring_of<kResp>(P)) {
        a.position = V3{wclamp(tpos.x, -edge.x, edge.x), wclamp(tpos.y, -edge.y, edge.y),
                        wclamp(tpos.z, -edge.z, edge.z)} + cetr;
        float ne = -P.e_envir;
        V3 f = {tx ? ne : 1.0f, ty ? ne : 1.0f, tz ? ne : 1.0f};
        a.velocity = a.velocity * f;
    } else {
        float mm = -(a.scale * P.r_agent);
        V3 sgn = {wsign(tpos.x), wsign(tpos.y), wsign(tpos.z)};
        V3 kforce = (P.k_agent * sgn) *
                    V3{wclamp(makeup.x, mm, 0.0f), wclamp(makeup.y, mm, 0.0f), wclamp(makeup.z, mm, 0.0f)};
        V3 cforce = P.neg_c_over_dt * a.velocity;
        a.force = a.force + (kforce + cforce);
        bool ux = makeup.x < mm, uy = makeup.y < mm, uz = makeup.z < mm;
        if (ux || uy || uz) {
            V3 e2 = edge - splat(mm);
            a.position = V3{wclamp(tpos.x, -e2.x, e2.x), wclamp(tpos.y, -e2.y, e2.y),
                            wclamp(tpos.z, -e2.z, e2.z)} + cetr;
            V3 sel = {ux ? a.velocity.x : 0.0f, uy ? a.velocity.y : 0.0f, uz ? a.velocity.z : 0.0f};
            V3 dv = P.neg_1pe_over_dt * sel;
            V3 acc = dv / P.dt;
            a.force = a.force + a.massv * acc;
        }
    }
}

// Count of the emitted key's cell only: for keys in no particular order (INIT
// frames, re-keying), whose per-tile counts are summed from the cell counts
// afterwards (count_tile_counts) instead of thousands of lanes contending for a
// few tile counters.
__device__ __forceinline__ void emit_cell(uint32_t* hist, uint32_t key) {
    if (hist) atomicAdd(hist + key, 1u);
}

// Counts of the emitted key for the next frame's counting sort: the cell, and the
// 4096-cell scan tile (one atomic per run of equal tiles among the active lanes;
// the keys of a LOOP pass follow the sorted order, so a warp's keys share tiles).
__device__ __forceinline__ void emit_count(uint32_t* hist, uint32_t* coarse, uint32_t key) {
    if (!hist) return;
    atomicAdd(hist + key, 1u);
    const uint32_t t = key >> 12;  // kScanTile = 4096
    const uint32_t am = __activemask();
    const uint32_t peers = __match_any_sync(am, t);
    if ((threadIdx.x & 31u) == (uint32_t)(__ffs(peers) - 1)) atomicAdd(coarse + t, (uint32_t)__popc(peers));
}

// Rank placement's far-move list (worlds in MB_SORT_RANK): input slot i of the
// next frame moved more than one cell along x or z (`f`).  One atomic per warp;
// once the list has overflowed (the next frame claims and fixes instead) the
// count is no longer raised.
__device__ __forceinline__ void note_far(uint32_t* far, uint32_t i, bool f) {
    const uint32_t am = __activemask();
    const uint32_t b = __ballot_sync(am, f);
    if (!b) return;
    const uint32_t lane = threadIdx.x & 31u, leader = (uint32_t)(__ffs(b) - 1);
    uint32_t base = 0;
    if (lane == leader)
        base = *reinterpret_cast<volatile uint32_t*>(far) > kFarCap ? kFarCap : atomicAdd(far, (uint32_t)__popc(b));
    base = __shfl_sync(am, base, (int)leader);
    const uint32_t at = base + (uint32_t)__popc(b & ((1u << lane) - 1u));
    if (f && at < kFarCap) far[1u + at] = i;
}

// main, INIT pipeline (physics.wgsl:91-96): gather through perm, re-pack, emit key.
__global__ void __launch_bounds__(256)
    k_physics_init(PhysParams P, uint32_t n, const uint32_t* __restrict__ perm,
                   const float4* __restrict__ pos_in, const uint4* __restrict__ vfme_in,
                   float4* __restrict__ pos_out, uint4* __restrict__ vfme_out,
                   uint32_t* __restrict__ keys_out, uint32_t* __restrict__ hist,
                   uint32_t* __restrict__ coarse) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t old = min(perm[i], n - 1u);
    float4 p = pos_in[old];
    Agent a = unpack(p, vfme_in[old]);
    uint32_t cx, cz;
    cell_of(P, a.position.x, a.position.z, cx, cz);
    pos_out[i] = make_float4(a.position.x, a.position.y, a.position.z, a.scale);
    vfme_out[i] = pack(a);
    uint32_t key = cz * P.N + cx;
    keys_out[i] = key;
    emit_cell(hist, key);
}

// Neighbour row-bands of a tile of sorted slots.  Band b (row offset b-1 = -1, 0,
// +1) is the union of every tile sphere's candidate range in that row: since
// slots are sorted by cell, it is one contiguous slot range of the sorted state.
// Bands of at most kBandCap slots are copied to shared memory with TMA bulk
// copies (cp.async.bulk, completion on one mbarrier); wider bands (a tile
// spanning a row boundary) are read from global memory instead.
constexpr int kTileThreads = kPhysicsTile;  // slots per tile (batched and fused passes: always)
// Slots a staged band holds, for tiles of kTile slots (the world's collide_block:
// 64, 128 or 256).
template <uint32_t kTile>
__host__ __device__ constexpr uint32_t band_cap() {
    return kTile == 256u ? 384u : 2u * kTile;
}
constexpr uint32_t kBandCap = band_cap<kTileThreads>();
constexpr uint32_t kBandPad = 8;  // >= the widest look-ahead of the contact walk, minus one
constexpr uint32_t kWaitLimit = 1u << 22;  // bounded mbarrier wait (error flag on expiry)
constexpr uint32_t kGatherUnroll = 2;      // band entries a thread gathers per step (loads in flight)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
// The barrier is initialised through the generic proxy and completed by bulk
// copies through the async proxy: the proxy fence, and a CTA barrier before the
// first copy is issued, order the two (a copy issued straight after the init by
// the initialising thread is not ordered with it).
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0u;
}
// global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// handle_collisions' contact loop (physics.wgsl:122-160): the candidates of the
// three rows in the reference's order (own row without the sphere itself, row
// below, row above) as one flat sequence t in [0, T).  Row r holds t in
// [start_r, start_r + c_r) and candidate t sits at base[t + o_r] (o_r folds in
// the row's first slot, its band and start_r; unsigned wrap-around is intended).
//
// The walk tests up to kLook candidates of the current row at a time, at the
// sphere's current position (consecutive slots: their loads are independent and
// in flight together), and stops at the first that may touch: that one gets the
// exact solve, which moves the sphere, and the walk resumes right after it.
// Every candidate is therefore decided at the position the sphere has when the
// reference's sequential loop reaches it.  The test is a squared-distance bound
// with a 0.3% margin, d2 - (edge * sqrt(1.003))^2 > 0 in one fused step: sqrt is
// monotone and correctly rounded, so a pair it rejects can never pass
// `length(tpos) <= edge` in the solve (the fused d2 differs from the unfused one
// by a few ulps, far inside the margin); a NaN result counts as "may touch" and
// is left to the exact test.  Slots past the row's end inside a step are read
// but masked out: `bpos` must stay readable kLook - 1 slots past every row
// (the shared bands are padded; global reads are clamped).
//
// kIndirect (global reads only): `bpos`/`bvfme` hold the state in the previous
// frame's slot order and sorted slot j is read at perm[j] (clamped to nmax).
__device__ __forceinline__ uint32_t cand_slot(uint32_t t, const uint32_t (&o)[3], uint32_t c0, uint32_t c01) {
    return t + (t < c0 ? o[0] : (t < c01 ? o[1] : o[2]));
}

constexpr float kNearScale = 1.0014989f;  // about sqrt(1.003): squared, a 0.3% margin on edge^2

// Packed pairs of floats for the look-ahead bound (sm_100+ f32x2 arithmetic:
// two IEEE single-precision operations, each rounded to nearest, in one
// instruction).  A candidate's (x, y) and (z, radius) are adjacent in its
// float4, so they pair without moves.
__device__ __forceinline__ unsigned long long f2pack(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2unpack(unsigned long long v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2sub(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long f2mul(unsigned long long a, unsigned long long b) {
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long f2fma(unsigned long long a, unsigned long long b,
                                                    unsigned long long c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

template <bool kShared, uint32_t kLook, bool kIndirect, bool kCg, int kResp>
__device__ __forceinline__ void contact_walk(const PhysParams& P, Agent& a, const float4* __restrict__ bpos,
                                             const uint4* __restrict__ bvfme, const uint32_t (&o)[3],
                                             uint32_t c0, uint32_t c01, uint32_t T, uint32_t tself,
                                             const uint32_t* __restrict__ perm, uint32_t nmax) {
    const float sk = a.scale * kNearScale;
    const unsigned long long zr_k = f2pack(-1.0f, kNearScale);
    uint32_t t = 0;
    while (t < T) {
        const bool r0 = t < c0, r01 = t < c01;
        const uint32_t j0 = t + (r0 ? o[0] : (r01 ? o[1] : o[2]));
        const uint32_t rem = (r0 ? c0 : (r01 ? c01 : T)) - t;  // candidates left in this row, >= 1
        float4 bp[kLook];
#pragma unroll
        for (uint32_t q = 0; q < kLook; ++q) {
            if (kShared) {
                bp[q] = bpos[j0 + q];
            } else {
                const uint32_t j = j0 + min(q, rem - 1u);
                bp[q] = ld_in<kCg>(bpos + (kIndirect ? min(ld_in<kCg>(perm + j), nmax) : j));
            }
        }
        uint32_t m = 0;
        // (dx, dy) = own (x, y) - (x, y); (dz, e) = (z, r) * (-1, kNear) + (own z, sk);
        // d2 = (dx^2 + dy^2) + dz^2 rounded step by step: within a few ulps of the
        // exact square, far inside the margin
        const unsigned long long axy = f2pack(a.position.x, a.position.y), azs = f2pack(a.position.z, sk);
#pragma unroll
        for (uint32_t q = 0; q < kLook; ++q) {
            const unsigned long long dxy = f2sub(axy, f2pack(bp[q].x, bp[q].y));
            float dz, e, dx2, dy2;
            f2unpack(f2fma(f2pack(bp[q].z, bp[q].w), zr_k, azs), dz, e);
            f2unpack(f2mul(dxy, dxy), dx2, dy2);
            const float d2 = __fmaf_rn(dz, dz, __fadd_rn(dx2, dy2));
            m |= !(__fmaf_rn(-e, e, d2) > 0.0f) ? 1u << q : 0u;
        }
        if (rem < kLook) m &= (1u << rem) - 1u;
        if (tself - t < kLook) m &= ~(1u << (tself - t));
        if (m) {
            const uint32_t q = (uint32_t)(__ffs(m) - 1);
            t += q + 1u;
            const uint32_t j = j0 + q;
            if constexpr (kResp == kSpring) {  // the neighbour's packed state is not read
                if (kShared) {
                    sphere<kResp>(P, a, unpack_pos(bpos[j]));
                } else {
                    const uint32_t sj = kIndirect ? min(ld_in<kCg>(perm + j), nmax) : j;
                    sphere<kResp>(P, a, unpack_pos(ld_in<kCg>(bpos + sj)));
                }
            } else if (kShared) {
                sphere<kResp>(P, a, unpack(bpos[j], bvfme[j]));
            } else {
                const uint32_t sj = kIndirect ? min(ld_in<kCg>(perm + j), nmax) : j;
                sphere<kResp>(P, a, unpack(ld_in<kCg>(bpos + sj), ld_in<kCg>(bvfme + sj)));
            }
        } else {
            t += min(rem, kLook);
        }
    }
}

// Four candidates per step suit sparse neighbourhoods (about nine candidates);
// six hide more latency where cells are crowded.  The warp agrees on one width
// so its lanes run one loop.
constexpr uint32_t kCrowdedT = 48, kLookSparse = 4, kLookCrowded = 6;

template <bool kShared, bool kIndirect, bool kCg, int kResp>
__device__ __forceinline__ void contact_loop(const PhysParams& P, Agent& a, const float4* __restrict__ bpos,
                                             const uint4* __restrict__ bvfme, const uint32_t (&o)[3],
                                             uint32_t c0, uint32_t c01, uint32_t T, uint32_t tself,
                                             const uint32_t* __restrict__ perm, uint32_t nmax) {
    if (__any_sync(__activemask(), T >= kCrowdedT))
        contact_walk<kShared, kLookCrowded, kIndirect, kCg, kResp>(P, a, bpos, bvfme, o, c0, c01, T, tself, perm, nmax);
    else
        contact_walk<kShared, kLookSparse, kIndirect, kCg, kResp>(P, a, bpos, bvfme, o, c0, c01, T, tself, perm, nmax);
}

// Slot ranges of the three candidate rows of a sphere in cell (cx, cz), key =
// cz*N + cx (get_collision_grid_id's neighbourhood, physics.wgsl:122-160): own
// row [0], row below [1], row above [2]; rows off the map stay empty.
template <bool kCg>
__device__ __forceinline__ void row_bounds(uint32_t N, const uint32_t* __restrict__ of, uint32_t key, uint32_t cx,
                                           uint32_t cz, uint32_t (&lo)[3], uint32_t (&hi)[3]) {
    const uint32_t l = cx > 0u ? 1u : 0u, rr = cx < N - 1u ? 2u : 1u;
    lo[0] = ld_in<kCg>(of + key - l);
    hi[0] = ld_in<kCg>(of + key + rr);
    lo[1] = hi[1] = lo[2] = hi[2] = 0u;
    if (cz > 0u) {
        lo[1] = ld_in<kCg>(of + key - N - l);
        hi[1] = ld_in<kCg>(of + key - N + rr);
    }
    if (cz < N - 1u) {
        lo[2] = ld_in<kCg>(of + key + N - l);
        hi[2] = ld_in<kCg>(of + key + N + rr);
    }
}

// One sphere's LOOP step (physics.wgsl:57-90) at sorted slot i, state `a`
// unpacked from it: Verlet, contacts against its candidate rows, jitter, walls,
// clamp, pack, store, new key and its counts.  The bands of its tile are staged
// in b_pos/b_vfme ([3][kCap]: band 0 row below, 1 own row, 2 row above; band
// b holds slots [b_lo[b], b_lo[b] + b_cnt[b])); rows outside them are read from
// spos/svfme (through perm when kIndirect).  base_a / base_c: the scene's first
// slot and cell (0 for a world).
template <bool kIndirect, bool kCg, uint32_t kCap, int kResp>
__device__ __forceinline__ void step_sphere(const PhysParams& P, Agent a, uint32_t i, uint32_t n, uint32_t base_a,
                                            uint32_t base_c, const uint32_t (&lo)[3], const uint32_t (&hi)[3],
                                            const float4* b_pos, const uint4* b_vfme, const uint32_t* b_lo,
                                            const uint32_t* b_cnt, const float4* __restrict__ spos,
                                            const uint4* __restrict__ svfme, const uint32_t* __restrict__ perm,
                                            float4* __restrict__ pos_out,
                                            uint4* __restrict__ vfme_out, uint32_t* __restrict__ keys_out,
                                            uint32_t* __restrict__ hist, uint32_t* __restrict__ coarse,
                                            uint32_t* far = nullptr, uint32_t ocx = 0, uint32_t ocz = 0) {
    // candidate rows in the reference's order: own row (band 1), below (0), above (2)
    uint32_t c[3], o_s[3], o_g[3];
    bool shared = true;
    {
        const uint32_t band[3] = {1u, 0u, 2u};
        uint32_t start = 0;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const uint32_t b = band[r];
            const uint32_t h = min(hi[r], n);
            c[r] = h > lo[r] ? h - lo[r] : 0u;
            if (r == 0 && !(i >= lo[0] && i < lo[0] + c[0])) c[0] = 0u;  // inconsistent input: drop
            shared = shared && (c[r] == 0u || (lo[r] >= b_lo[b] && h <= b_lo[b] + b_cnt[b]));
            o_s[r] = b * kCap + lo[r] - b_lo[b] - start;
            o_g[r] = lo[r] - start;
            start += c[r];
        }
    }
    const uint32_t c01 = c[0] + c[1], T = c01 + c[2];
    const uint32_t tself = c[0] ? i - lo[0] : 0xFFFFFFFFu;

    // verlet_integration (physics.wgsl:262-266)
    {
        V3 acc = div_exact(a.force, a.massv);  // unit masses: three multiplies
        a.velocity = a.velocity + ((V3{P.gx, P.gy, P.gz} + acc) * P.dt) * P.dt;
        a.position = a.position + a.velocity;
    }
    a.force = splat(0.0f);

    // handle_collisions (physics.wgsl:119-169)
    V3 old_pos = a.position;
    if (shared)
        contact_loop<true, false, kCg, kResp>(P, a, b_pos, b_vfme, o_s, c[0], c01, T, tself, perm, n - 1u);
    else
        contact_loop<false, kIndirect, kCg, kResp>(P, a, spos, svfme, o_g, c[0], c01, T, tself, perm, n - 1u);
    V3 diff = a.position - old_pos;
    if (longer_than(diff, a.scale)) {
        // hash3f1u(new_agent_index) * 2 - 1 (physics.wgsl:166, 334-337); the
        // index is the slot inside the sphere's own scene
        const uint32_t li = i - base_a;
        uint32_t v = li * (li ^ (li >> 15));
        const float d = 4294967296.0f;
        V3 h = {__uint2float_rn(v * 0x1u) / d, __uint2float_rn(v * 0x1FFu) / d,
                __uint2float_rn(v * 0x3FFFFu) / d};
        V3 jitter = {h.x * 2.0f - 1.0f, h.y * 2.0f - 1.0f, h.z * 2.0f - 1.0f};
        a.position = a.position + normalize3(jitter);
    }

    cube<kResp>(P, a);

    const float lim = 65504.0f;  // CLAMP_F16
    a.velocity = {wclamp(a.velocity.x, -lim, lim), wclamp(a.velocity.y, -lim, lim),
                  wclamp(a.velocity.z, -lim, lim)};
    a.force = {wclamp(a.force.x, -lim, lim), wclamp(a.force.y, -lim, lim), wclamp(a.force.z, -lim, lim)};

    pos_out[i] = make_float4(a.position.x, a.position.y, a.position.z, a.scale);
    vfme_out[i] = pack(a);
    uint32_t nx, nz;
    cell_of(P, a.position.x, a.position.z, nx, nz);
    const uint32_t nk = base_c + nz * P.N + nx;
    keys_out[i] = nk;
    emit_count(hist, coarse, nk);
    if (far) note_far(far, i, nx - ocx + 1u > 2u || nz - ocz + 1u > 2u);  // (ocx, ocz): the cell it was sorted by
}

// Key of a position (physics.wgsl:115-117).
__device__ __forceinline__ uint32_t key_of(const PhysParams& P, float4 p) {
    uint32_t cx, cz;
    cell_of(P, p.x, p.z, cx, cz);
    return cz * P.N + cx;
}

// Scene of sorted slot i: start from the first scene of the tile.
__device__ __forceinline__ uint32_t scene_of(const SceneDev* __restrict__ scenes, uint32_t first, uint32_t i) {
    uint32_t s = first;
    while (i >= __ldg(&scenes[s].agent_end)) ++s;
    return s;
}

// Shared memory of one tile of kTile slots: bands (pos padded: the walk reads
// past rows) and the band bounds.  kPosOnly (a world of the spring model, whose
// contacts read the neighbours' positions only): the bands hold positions
// alone, twice as many slots in the same memory.  (The mbarrier of the band
// copies is kept apart, so that the fused frame kernel can reuse this memory for
// its other stages.)
template <uint32_t kTile, bool kPosOnly = false>
struct TileSmemT {
    static constexpr uint32_t kCap = kPosOnly ? 2u * band_cap<kTile>() : band_cap<kTile>();
    float4 pos[3 * kCap + kBandPad];
    uint4 vfme[kPosOnly ? 1u : 3 * kCap];
    uint32_t lo[3], cnt[3];
};
using TileSmem = TileSmemT<kTileThreads>;

// main (physics.wgsl:57-97) for one tile of kTile consecutive sorted
// slots, one thread per slot.  agent_new(agent_index_sorted[i]) of the reference
// is the state of sorted slot i:
//   kIndirect = false: spos/svfme hold the state in sorted order (the sort wrote
//     a copy), slot i is spos[i]; bands are copied with TMA bulk copies;
//   kIndirect = true: spos/svfme hold the state in the previous frame's slot
//     order and slot i is spos[perm[i]]; bands are gathered through perm by the
//     block's threads (the sort writes no state copy).
//
// kBatched = false: one scene, parameters P, LOOP pipeline.
// kBatched = true: many scenes in one flattened key space (scene s owns slots
// [agent_base, agent_end) and cells [cell_base, cell_base + N*N)); each slot runs
// its scene's mode: LOOP, INIT (re-pack, emit key) or HOLD (state carried over
// unchanged, key re-emitted).  Slot indices inside a scene (the jitter hash)
// are local, so every scene evolves exactly as it would alone.

// One tile of the physics pass, run by kTile threads (tid = 0 .. kTile-1 within
// the group; the block's __syncthreads must be reached by every thread of the
// block, so a block that runs two tiles side by side runs both halves through
// this function together).  s_bar must have been initialised (copy mode);
// bar_parity is the phase this tile's copies complete.  A tile at or past the
// end (tile * kTile >= n) does nothing but take part in the barriers.  The band
// table holds bounds per 128-slot tile: a 256-slot tile joins two entries, a
// 64-slot tile derives its own from its first and last cells.
template <bool kBatched, bool kIndirect, bool kCg = false, uint32_t kTile = kTileThreads,
          int kResp = kSpringRuntime>
__device__ __forceinline__ void physics_tile(
    uint32_t tile, uint32_t tid, uint32_t bar_parity, TileSmemT<kTile, kResp == kSpring>* sm, uint64_t* s_bar,
    const PhysParams& P1,
    const SceneDev* __restrict__ scenes, const uint32_t* __restrict__ tile_scene, uint32_t n,
    const uint32_t* __restrict__ offs, const uint4* __restrict__ bands, const float4* __restrict__ spos,
    const uint4* __restrict__ svfme, const uint32_t* __restrict__ perm, float4* __restrict__ pos_out0,
    float4* __restrict__ pos_out1, uint4* __restrict__ vfme_out0, uint4* __restrict__ vfme_out1,
    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ hist, uint32_t* __restrict__ coarse,
    uint32_t* __restrict__ err, uint32_t* __restrict__ far = nullptr) {
    static_assert(!(kBatched && kIndirect), "batches stage a sorted copy");
    static_assert(kTile == 64u || kTile == 128u || kTile == 256u, "tiles of 64, 128 or 256 slots");
    constexpr bool kPosOnly = kResp == kSpring;
    constexpr uint32_t kCap = TileSmemT<kTile, kPosOnly>::kCap;
    const uint4* __restrict__ btab = kTile == 64u ? nullptr : bands;
    float4* const s_pos = sm->pos;
    uint4* const s_vfme = sm->vfme;
    uint32_t* const s_lo = sm->lo;
    uint32_t* const s_cnt = sm->cnt;

    const uint32_t i0 = tile * kTile;
    const bool tile_ok = i0 < n;
    const uint32_t i = i0 + tid;
    const uint32_t ilast = tile_ok ? min(i0 + kTile, n) - 1u : 0u;
    const bool valid = tile_ok && i < n;

    // this slot's scene; its output buffer is the one its current state is not in
    uint32_t sc = 0, base_a = 0, base_c = 0, mode = kModeLoop;
    float4* __restrict__ pos_out = pos_out0;
    uint4* __restrict__ vfme_out = vfme_out0;
    if (kBatched && tile_ok) {
        const uint32_t first = __ldg(tile_scene + tile * kTile / kPhysicsTile);
        sc = scene_of(scenes, first, valid ? i : ilast);
        base_a = scenes[sc].agent_base;
        base_c = scenes[sc].cell_base;
        mode = scenes[sc].mode;
        if (scenes[sc].parity == 0u) {
            pos_out = pos_out1;
            vfme_out = vfme_out1;
        }
    }

    const PhysParams& P = kBatched ? scenes[sc].P : P1;  // read where it lives, not copied
    if (tid == 0 && !tile_ok) {
#pragma unroll
        for (int b = 0; b < 3; ++b) s_cnt[b] = 0u;  // nothing to stage
    }
    if (btab && tile_ok) {  // bounds from the band table: one load (a batch: tiles inside one LOOP scene)
        if (tid == 0) {
            bool stage = true;
            if (kBatched) {
                const uint32_t first = __ldg(tile_scene + tile * kTile / kPhysicsTile);
                const uint32_t sf = scene_of(scenes, first, i0), sl = scene_of(scenes, first, ilast);
                stage = sf == sl && __ldg(&scenes[sf].mode) == kModeLoop;
            }
            const uint4 z = make_uint4(0u, 0u, 0u, 0u);
            // read before the wait below: the scatter wrote the table and had
            // completed before the kernel this one follows could start (the
            // fixups in between reorder slots inside cells, never tile bounds);
            // read through L2
            constexpr uint32_t kPer = kTile / kPhysicsTile;  // 128-slot table tiles per tile
            const uint32_t tl = tile * kPer, th = min(tl + kPer - 1u, (n - 1u) / kPhysicsTile);
            const uint4 l = stage ? __ldcg(btab + 2u * tl) : z;
            const uint4 h = stage ? __ldcg(btab + 2u * th + 1u) : z;
            const uint32_t lo3[3] = {l.x, l.y, l.z}, hi3[3] = {h.x, h.y, h.z};
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const uint32_t hb = min(hi3[b], n);
                s_lo[b] = lo3[b];
                s_cnt[b] = (hb > lo3[b] && hb - lo3[b] <= kCap) ? hb - lo3[b] : 0u;
            }
        }
    }
    griddep_wait();  // the sort's outputs (order, state copy) are complete and visible
    if (!btab && tile_ok && tid < 3) {  // band b: keys of the tile's first and last sphere, then offsets
        uint32_t lo = 0, hi = 0;
        bool stage = true;
        PhysParams Q = P;
        uint32_t qc = base_c;
        if (kBatched) {  // stage only tiles inside one LOOP scene
            const uint32_t first = __ldg(tile_scene + tile * kTile / kPhysicsTile);
            const uint32_t sf = scene_of(scenes, first, i0), sl = scene_of(scenes, first, ilast);
            stage = sf == sl && scenes[sf].mode == kModeLoop;
            Q = scenes[sf].P;
            qc = scenes[sf].cell_base;
        }
        if (stage) {
            const uint32_t N = Q.N;
            const uint32_t sf0 = kIndirect ? min(ld_in<kCg>(perm + i0), n - 1u) : i0;
            const uint32_t sl0 = kIndirect ? min(ld_in<kCg>(perm + ilast), n - 1u) : ilast;
            const uint32_t kf = key_of(Q, ld_in<kCg>(spos + sf0)), kl = key_of(Q, ld_in<kCg>(spos + sl0));
            const uint32_t cxf = kf - (kf / N) * N, cxl = kl - (kl / N) * N;
            const uint32_t* of = offs + qc;
            if (tid == 1) {  // own row
                lo = ld_cur<kCg>(of + kf - (cxf > 0u ? 1u : 0u));
                hi = ld_cur<kCg>(of + kl + (cxl < N - 1u ? 2u : 1u));
            } else if (tid == 0) {  // row below, for tile spheres with cz > 0
                if (kl >= N) {
                    uint32_t f = max(kf, N);
                    uint32_t cf = f - (f / N) * N;
                    lo = ld_cur<kCg>(of + f - N - (cf > 0u ? 1u : 0u));
                    hi = ld_cur<kCg>(of + kl - N + (cxl < N - 1u ? 2u : 1u));
                }
            } else {  // row above, for tile spheres with cz < N-1
                const uint32_t top = N * (N - 1u);
                if (kf < top) {
                    uint32_t l = min(kl, top - 1u);
                    uint32_t cl = l - (l / N) * N;
                    lo = ld_cur<kCg>(of + kf + N - (cxf > 0u ? 1u : 0u));
                    hi = ld_cur<kCg>(of + l + N + (cl < N - 1u ? 2u : 1u));
                }
            }
        }
        hi = min(hi, n);
        s_lo[tid] = lo;
        s_cnt[tid] = (hi > lo && hi - lo <= kCap) ? hi - lo : 0u;
    }

    // own sphere: loads issued here overlap the band set-up
    float4 own_p = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint4 own_q = make_uint4(0u, 0u, 0u, 0u);
    if (valid) {
        const uint32_t o = kIndirect ? min(ld_in<kCg>(perm + i), n - 1u) : i;
        own_p = ld_in<kCg>(spos + o);
        own_q = ld_in<kCg>(svfme + o);
    }
    __syncthreads();  // band bounds published (and, copy mode, the mbarrier initialised)
    if (kIndirect) {
        // gather the bands through perm: every thread takes entries tid, tid + 128,
        // ... of the three bands laid end to end, kGatherUnroll at a time (loads
        // first, then stores)
        const uint32_t c0 = s_cnt[0], c01 = c0 + s_cnt[1], tot = c01 + s_cnt[2];
        for (uint32_t f0 = 0; f0 < tot; f0 += kGatherUnroll * kTile) {
            uint32_t dst[kGatherUnroll], src[kGatherUnroll];
#pragma unroll
            for (uint32_t u = 0; u < kGatherUnroll; ++u) {
                const uint32_t f = f0 + u * kTile + tid;
                const uint32_t b = f < c0 ? 0u : (f < c01 ? 1u : 2u);
                const uint32_t j = f - (b == 0u ? 0u : (b == 1u ? c0 : c01));
                dst[u] = b * kCap + j;
                src[u] = f < tot ? min(ld_in<kCg>(perm + s_lo[b] + j), n - 1u) : 0u;
            }
            float4 gp[kGatherUnroll];
            uint4 gq[kGatherUnroll];
#pragma unroll
            for (uint32_t u = 0; u < kGatherUnroll; ++u) {
                if (f0 + u * kTile + tid < tot) {
                    gp[u] = ld_in<kCg>(spos + src[u]);
                    if (!kPosOnly) gq[u] = ld_in<kCg>(svfme + src[u]);
                }
            }
#pragma unroll
            for (uint32_t u = 0; u < kGatherUnroll; ++u) {
                if (f0 + u * kTile + tid < tot) {
                    s_pos[dst[u]] = gp[u];
                    if (!kPosOnly) s_vfme[dst[u]] = gq[u];
                }
            }
        }
    } else if (tid == 0) {
        uint32_t bytes = 0;
#pragma unroll
        for (int b = 0; b < 3; ++b) bytes += s_cnt[b] * (kPosOnly ? 16u : 32u);
        mbar_arrive_expect_tx(s_bar, bytes);
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            if (s_cnt[b]) {
                bulk_g2s(s_pos + b * kCap, spos + s_lo[b], s_cnt[b] * 16u, s_bar);
                if (!kPosOnly) bulk_g2s(s_vfme + b * kCap, svfme + s_lo[b], s_cnt[b] * 16u, s_bar);
            }
        }
    }

    // candidate rows of the own sphere (overlaps the copies)
    const uint32_t N = P.N;
    Agent a;
    uint32_t cx = 0, cz = 0, key = 0;
    uint32_t lo[3] = {0u, 0u, 0u}, hi[3] = {0u, 0u, 0u};
    if (valid) {
        a = unpack(own_p, own_q);
        cell_of(P, a.position.x, a.position.z, cx, cz);
        key = cz * N + cx;
        if (mode == kModeLoop) row_bounds<kCg>(N, offs + base_c, key, cx, cz, lo, hi);
    }
    if (kIndirect) {
        __syncthreads();  // bands gathered
    } else {  // bounded wait for the bands (every thread, so all copies land before exit)
        uint32_t spins = 0;
        while (!mbar_try_wait(s_bar, bar_parity)) {
            if (++spins > kWaitLimit) {
                if (tid == 0) atomicOr(err, 4u);
                break;
            }
        }
    }
    if (!valid) return;

    if (kBatched && mode == kModeInit) {  // INIT (physics.wgsl:91-96): re-pack, emit key
        pos_out[i] = own_p;
        vfme_out[i] = pack(a);
        keys_out[i] = base_c + key;
        emit_cell(hist, base_c + key);  // tile counts of INIT scenes: count_tile_counts
        return;
    }
    if (kBatched && mode == kModeHold) return;  // keeps state, buffer, keys and counts

    step_sphere<kIndirect, kCg, kCap, kResp>(P, a, i, n, base_a, base_c, lo, hi, s_pos, s_vfme, s_lo, s_cnt, spos, svfme, perm,
                                pos_out, vfme_out, keys_out, hist, coarse, far, cx, cz);
}

template <bool kBatched, bool kIndirect, uint32_t kTile = kTileThreads, int kResp = kSpringRuntime>
__global__ void __launch_bounds__(kTile)
    k_physics_frame(const __grid_constant__ PhysParams P1, const SceneDev* __restrict__ scenes,
                    const uint32_t* __restrict__ tile_scene, uint32_t n, const uint32_t* __restrict__ offs,
                    const uint4* __restrict__ bands, const float4* __restrict__ spos,
                    const uint4* __restrict__ svfme, const uint32_t* __restrict__ perm, float4* __restrict__ pos_out0,
                    float4* __restrict__ pos_out1, uint4* __restrict__ vfme_out0, uint4* __restrict__ vfme_out1,
                    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ hist, uint32_t* __restrict__ coarse,
                    uint32_t* __restrict__ err, uint32_t* __restrict__ far) {
    __shared__ __align__(16) TileSmemT<kTile, kResp == kSpring> sm;
    __shared__ __align__(8) uint64_t s_bar;
    if (!kIndirect && threadIdx.x == 0) mbar_init(&s_bar, 1u);  // first copy after the tile's CTA barrier
    physics_tile<kBatched, kIndirect, false, kTile, kResp>(blockIdx.x, threadIdx.x, 0u, &sm, &s_bar, P1, scenes, tile_scene, n, offs,
                                      bands, spos, svfme, perm, pos_out0, pos_out1, vfme_out0, vfme_out1, keys_out,
                                      hist, coarse, err, far);
}

// ---------------------------------------------------------------- fused frame
// LOOP frames as one cooperative kernel: the stages of a frame (count scan,
// scatter, marked-cell fixup, cells above 256 slots if any, physics) run back to back in one launch,
// separated by grid barriers instead of kernel boundaries, for as many frames
// as the launch is given.  Every block is resident (cooperative launch), so a
// block may wait for the others; each wait is bounded.  The stages run the same
// device code as the per-stage kernels, reading data written earlier in the
// launch from L2 (kCg), so the results are identical.
constexpr uint32_t kFusedThreads = 256;
constexpr uint32_t kBarrierLimit = 1u << 24;  // polls of a grid barrier before it gives up (~2 s)

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// bar[0] counts arrivals, bar[1] is the generation.  The last block to arrive
// resets the count and advances the generation; the others wait for that.  A
// wait that runs out (or sees that another block's wait ran out) sets bit 8 of
// the error word and returns false: the caller then leaves the kernel.
__device__ __forceinline__ bool grid_barrier(uint32_t* bar, uint32_t* err, uint32_t* s_flag) {
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t ok = 1u;
        const uint32_t gen = ld_acquire_gpu(bar + 1);
        __threadfence();  // this block's writes before its arrival
        if (atomicAdd(bar, 1u) == gridDim.x - 1u) {
            __threadfence();  // every other block's writes (their arrivals are read above)
            atomicExch(bar, 0u);
            st_release_gpu(bar + 1, gen + 1u);
        } else {
            uint32_t spins = 0;
            while (ld_acquire_gpu(bar + 1) == gen) {
                ++spins;
                if (spins > kBarrierLimit || ((spins & 1023u) == 0u && (ld_acquire_gpu(err) & 8u))) {
                    atomicOr(err, 8u);
                    ok = 0u;
                    break;
                }
                if (spins > 32u) __nanosleep(64);
            }
        }
        __threadfence();
        *s_flag = ok;
    }
    __syncthreads();
    return *s_flag != 0u;
}

struct FusedArgs {
    PhysParams P;
    uint32_t n, cells, chunks, scan_tiles, phys_tiles, collect_blocks, frames, cur;
    uint32_t* keys;
    uint32_t* hist;
    uint32_t* coarse;
    uint32_t* offs;
    uint32_t* perm;
    uint4* bands;
    uint32_t* fix_bits;
    uint32_t* fix_tmp;
    FixLists lists;
    float4* pos[2];
    uint4* vfme[2];
    float4* spos;   // sorted copy (copy mode)
    uint4* svfme;
    uint32_t* bar;  // [2] grid barrier words (zero between launches)
    uint32_t* err;
};

union FusedSmem {
    struct {
        uint32_t warp[kScanThreads / 32], base[kScanThreads / 32];
    } scan;
    MarkedSmem marked;
    struct {
        uint32_t v[kBitmapWords];
        uint32_t red[kFixThreads / 32 + 1];
    } fix;
    TileSmem tile[2];  // the physics stage runs two 128-slot tiles per block side by side
};
static_assert(kScanThreads == kFusedThreads && kCollectThreads == kFusedThreads && kFixThreads == kFusedThreads &&
                  2u * kTileThreads == kFusedThreads,
              "the fused kernel runs every stage with its block shape");

template <bool kIndirect>
__global__ void __launch_bounds__(kFusedThreads, 4) k_frame_fused(const __grid_constant__ FusedArgs A) {
    extern __shared__ __align__(16) unsigned char fused_smem[];
    FusedSmem& S = *reinterpret_cast<FusedSmem*>(fused_smem);
    __shared__ __align__(8) uint64_t s_bar[2];
    __shared__ uint32_t s_flag;
    const uint32_t tid = threadIdx.x, half = tid / kTileThreads;
    if (!kIndirect && tid % kTileThreads == 0u) mbar_init(&s_bar[half], 1u);
    uint32_t parity = 0;
    for (uint32_t f = 0; f < A.frames; ++f) {
        const uint32_t cur = A.cur ^ (f & 1u), nxt = cur ^ 1u;
        // cell offsets from the counts the previous frame emitted
        for (uint32_t vb = blockIdx.x; vb < A.chunks; vb += gridDim.x) {
            scan_chunk<false, true>(vb, A.hist, A.coarse, A.cells, A.offs, A.lists.ctl, nullptr, nullptr, S.scan.warp,
                                    S.scan.base);
            __syncthreads();  // partial sums read before the next chunk writes them
        }
        if (!grid_barrier(A.bar, A.err, &s_flag)) return;
        scatter_range<true>(blockIdx.x, gridDim.x, A.keys, A.n, A.hist, A.perm, A.pos[cur], A.vfme[cur],
                            kIndirect ? nullptr : A.spos, kIndirect ? nullptr : A.svfme, A.offs, A.bands, A.P.N,
                            A.fix_bits);
        if (!grid_barrier(A.bar, A.err, &s_flag)) return;
        const OneBufferT<true> src{A.pos[cur], A.vfme[cur]};
        clear_counts(blockIdx.x, gridDim.x, src, A.hist, A.cells, A.coarse, A.scan_tiles);
        for (uint32_t vb = blockIdx.x; vb < A.collect_blocks; vb += gridDim.x) {
            fix_marked_block<OneBufferT<true>, true, false>(vb, A.collect_blocks, A.fix_bits, A.keys, A.n, A.offs,
                                                            A.perm, A.lists, A.fix_tmp, src,
                                                            kIndirect ? nullptr : A.spos,
                                                            kIndirect ? nullptr : A.svfme, S.marked);
            __syncthreads();  // the shared lists are done before the next block's counters reset
        }
        if (!grid_barrier(A.bar, A.err, &s_flag)) return;
        if (__ldcg(A.lists.ctl + kFixListHuge) != 0u) {  // cells above kFixWarp slots (the same count in every block)
            fix_huge<OneBufferT<true>, true, kBitmapWords>(blockIdx.x, gridDim.x, A.lists, A.offs, A.perm, A.fix_tmp,
                                                           src, kIndirect ? nullptr : A.spos,
                                                           kIndirect ? nullptr : A.svfme, S.fix.v, S.fix.red);
            if (!grid_barrier(A.bar, A.err, &s_flag)) return;
        }
        // the stages above wrote the sorted copy (global) and this block's shared
        // memory through the generic proxy; the bulk copies read and write them
        // through the async proxy
        asm volatile("fence.proxy.async;" ::: "memory");
        __syncthreads();
        for (uint32_t t2 = blockIdx.x; 2u * t2 < A.phys_tiles; t2 += gridDim.x) {
            physics_tile<false, kIndirect, true>(2u * t2 + half, tid % kTileThreads, parity, &S.tile[half],
                                                 &s_bar[half], A.P, nullptr, nullptr, A.n, A.offs, A.bands,
                                                 kIndirect ? A.pos[cur] : A.spos, kIndirect ? A.vfme[cur] : A.svfme,
                                                 kIndirect ? A.perm : nullptr, A.pos[nxt], nullptr, A.vfme[nxt],
                                                 nullptr, A.keys, A.hist, A.coarse, A.err);
            parity ^= 1u;
            __syncthreads();  // every thread is done with this tile's bands and bounds
            asm volatile("fence.proxy.async;" ::: "memory");
        }
        if (f + 1u < A.frames && !grid_barrier(A.bar, A.err, &s_flag)) return;
    }
}




// Self-test of div_exact against IEEE division over count generated cases:
// operands from all float bit patterns, normal-range operands, power-of-two
// divisors and exact multiples.  Mismatching bit patterns are counted;
// the first one is kept in bad[0..3] = a, d, div_exact, IEEE.
__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__global__ void k_selftest_divide(uint64_t seed, uint64_t count, unsigned long long* mismatches, uint32_t* bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride) {
        const uint64_t h = mix64(seed ^ mix64(k));
        uint32_t ua = (uint32_t)h, ud = (uint32_t)(h >> 32);
        switch (k & 3u) {
            case 0: break;  // any bit patterns
            case 1:  // any numerator, a power-of-two divisor of either sign
                ud &= 0xFF800000u;
                break;
            case 2: {  // a = d * m for a small integer or a power of two: exact and power-of-two quotients
                ud = (ud & 0x807FFFFFu) | ((100u + (ud >> 23) % 40u) << 23);
                const float m = (ua & 1u) ? (float)((ua >> 1) & 0xFFFu) : __uint_as_float((120u + ((ua >> 1) & 15u)) << 23);
                ua = __float_as_uint(__fmul_rn(__uint_as_float(ud), m));
                break;
            }
            default: {  // normalised vectors: |a| <= d, d near 1
                ud = 0x3F000000u + (ud & 0x00FFFFFFu);
                ua = (ua & 0x80000000u) | (__float_as_uint(__uint_as_float(ud) * ((ua & 0x7FFFFFu) * 0x1p-23f)));
                break;
            }
        }
        const float a = __uint_as_float(ua), d = __uint_as_float(ud);
        const V3 got = div_exact(V3{a, -a, __fmul_rn(a, 0.75f)}, d);
        const float want[3] = {__fdiv_rn(a, d), __fdiv_rn(-a, d), __fdiv_rn(__fmul_rn(a, 0.75f), d)};
        const float g[3] = {got.x, got.y, got.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (__float_as_uint(g[c]) != __float_as_uint(want[c])) {
                if (atomicAdd(mismatches, 1ull) == 0ull) {
                    bad[0] = ua;
                    bad[1] = ud;
                    bad[2] = __float_as_uint(g[c]);
                    bad[3] = __float_as_uint(want[c]);
                }
            }
        }
    }
}

__global__ void k_rekey(PhysParams P, uint32_t n, const float4* __restrict__ pos,
                        uint32_t* __restrict__ keys, uint32_t* __restrict__ hist,
                        uint32_t* __restrict__ coarse) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pos[i];
    uint32_t cx, cz;
    cell_of(P, p.x, p.z, cx, cz);
    keys[i] = cz * P.N + cx;
    emit_cell(hist, keys[i]);
}

}  // namespace

PhysParams make_params(const mb_consts& c) {
    PhysParams p;
    p.N = c.number_of_grids_one_dimension;
    p.grid_size = c.grid_size;
    p.half_map_size = c.half_map_size;
    p.half_map_height = c.half_map_height;
    p.gx = c.gravity[0];
    p.gy = c.gravity[1];
    p.gz = c.gravity[2];
    p.e_envir = c.e_envir;
    p.e_agent = c.e_agent;
    p.k_agent = c.k_agent;
    p.c_agent = c.c_agent;
    p.r_agent = c.r_agent;
    p.dt = c.time_delta;
    // const-folded in the shader (physics.wgsl:285, 292): one f32 division each
    volatile float nc = -c.c_agent;
    volatile float n1pe = -(1.0f + c.e_envir);
    p.neg_c_over_dt = nc / c.time_delta;
    p.neg_1pe_over_dt = n1pe / c.time_delta;
    p.spring = c.enable_spring;
    // magic numbers of n / grid_size (Hacker's Delight 10-8, 33-bit multiplier)
    uint32_t d = c.grid_size ? c.grid_size : 1u, lg = 0;
    while (lg < 32u && (1ull << lg) < d) ++lg;
    p.div_m = (uint32_t)(((1ull << 32) * ((1ull << lg) - d)) / d + 1ull);
    p.div_s1 = lg > 0u ? 1u : 0u;
    p.div_s2 = lg > 0u ? lg - 1u : 0u;
    return p;
}

cudaError_t launch_physics_init(const PhysParams& p, uint32_t n, const uint32_t* perm,
                                const float4* pos_in, const uint4* vfme_in, float4* pos_out,
                                uint4* vfme_out, uint32_t* keys_out, uint32_t* hist, uint32_t* coarse,
                                cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_physics_init<<<(n + 255u) / 256u, 256, 0, st>>>(p, n, perm, pos_in, vfme_in, pos_out, vfme_out,
                                                      keys_out, hist, coarse);
    return cudaGetLastError();
}

template <uint32_t kTile, int kResp>
cudaError_t launch_physics_resp(const PhysParams& p, uint32_t n, const uint32_t* offs, const uint4* bands,
                                const float4* spos, const uint4* svfme, const uint32_t* perm, float4* pos_out,
                                uint4* vfme_out, uint32_t* keys_out, uint32_t* hist, uint32_t* coarse,
                                uint32_t* err, cudaStream_t st, bool pdl, uint32_t* far) {
    const dim3 grid((n + kTile - 1u) / kTile), block(kTile);
    if (perm)
        return launch_pdl(pdl, k_physics_frame<false, true, kTile, kResp>, grid, block, 0, st, p, (const SceneDev*)nullptr,
                          (const uint32_t*)nullptr, n, offs, bands, spos, svfme, perm, pos_out, (float4*)nullptr,
                          vfme_out, (uint4*)nullptr, keys_out, hist, coarse, err, far);
    return launch_pdl(pdl, k_physics_frame<false, false, kTile, kResp>, grid, block, 0, st, p,
                      (const SceneDev*)nullptr, (const uint32_t*)nullptr, n, offs, bands, spos, svfme,
                      (const uint32_t*)nullptr, pos_out, (float4*)nullptr, vfme_out, (uint4*)nullptr, keys_out, hist,
                      coarse, err, far);
}

// One world's response model is known on the host: the kernel is compiled for it.
template <uint32_t kTile>
cudaError_t launch_physics_tiles(const PhysParams& p, uint32_t n, const uint32_t* offs, const uint4* bands,
                                 const float4* spos, const uint4* svfme, const uint32_t* perm, float4* pos_out,
                                 uint4* vfme_out, uint32_t* keys_out, uint32_t* hist, uint32_t* coarse,
                                 uint32_t* err, cudaStream_t st, bool pdl, uint32_t* far) {
    if (p.spring)
        return launch_physics_resp<kTile, kSpring>(p, n, offs, bands, spos, svfme, perm, pos_out, vfme_out,
                                                   keys_out, hist, coarse, err, st, pdl, far);
    return launch_physics_resp<kTile, kRigid>(p, n, offs, bands, spos, svfme, perm, pos_out, vfme_out, keys_out,
                                              hist, coarse, err, st, pdl, far);
}

cudaError_t launch_physics_loop(const PhysParams& p, uint32_t n, const uint32_t* offs, const uint4* bands,
                                const float4* spos, const uint4* svfme, const uint32_t* perm, float4* pos_out,
                                uint4* vfme_out, uint32_t* keys_out, uint32_t* hist, uint32_t* coarse, uint32_t* err,
                                cudaStream_t st, bool pdl, uint32_t tile, uint32_t* far) {
    if (!n) return cudaSuccess;
    if (tile == 64u)
        return launch_physics_tiles<64u>(p, n, offs, bands, spos, svfme, perm, pos_out, vfme_out, keys_out, hist,
                                         coarse, err, st, pdl, far);
    if (tile == 256u)
        return launch_physics_tiles<256u>(p, n, offs, bands, spos, svfme, perm, pos_out, vfme_out, keys_out, hist,
                                          coarse, err, st, pdl, far);
    return launch_physics_tiles<128u>(p, n, offs, bands, spos, svfme, perm, pos_out, vfme_out, keys_out, hist,
                                      coarse, err, st, pdl, far);
}

int fused_blocks_per_sm() {
    static int per_sm = -1;  // same for every device of one architecture
    if (per_sm < 0) {
        int b = 0;
        const size_t smem = sizeof(FusedSmem);
        cudaError_t e = cudaFuncSetAttribute(k_frame_fused<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (!e) e = cudaFuncSetAttribute(k_frame_fused<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (!e) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_frame_fused<false>, kFusedThreads, smem);
        int b2 = 0;
        if (!e) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_frame_fused<true>, kFusedThreads, smem);
        per_sm = e ? 0 : std::min(b, b2);
    }
    return per_sm;
}

cudaError_t launch_frame_fused(const FusedFrame& f, cudaStream_t st) {
    if (!f.frames || !f.n) return cudaSuccess;
    const int per_sm = fused_blocks_per_sm();
    if (per_sm <= 0) return cudaErrorCooperativeLaunchTooLarge;
    FusedArgs A;
    A.P = f.P;
    A.n = f.n;
    A.cells = f.cells;
    A.chunks = (f.cells + kScanChunk - 1u) / kScanChunk;
    A.scan_tiles = (f.cells + kScanTile - 1u) / kScanTile;
    A.phys_tiles = (f.n + kTileThreads - 1u) / kTileThreads;
    A.collect_blocks = ((f.n + 31u) / 32u + kCollectWords - 1u) / kCollectWords;
    A.frames = f.frames;
    A.cur = f.cur;
    A.keys = f.keys;
    A.hist = f.cnt->hist;
    A.coarse = f.cnt->coarse;
    A.offs = f.offs;
    A.perm = f.perm;
    A.bands = f.bands;
    A.fix_bits = f.cnt->fix_bits;
    A.fix_tmp = f.cnt->fix_tmp;
    A.lists = FixLists{f.cnt->fix_ctl, {f.cnt->fix[0], f.cnt->fix[1], f.cnt->fix[2]},
                       {f.cnt->fix_cap[0], f.cnt->fix_cap[1], f.cnt->fix_cap[2]}};
    for (int b = 0; b < 2; ++b) {
        A.pos[b] = f.pos[b];
        A.vfme[b] = f.vfme[b];
    }
    A.spos = f.spos;
    A.svfme = f.svfme;
    A.bar = f.bar;
    A.err = f.err;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((uint32_t)(per_sm * device_sm_count()));
    cfg.blockDim = dim3(kFusedThreads);
    cfg.dynamicSmemBytes = sizeof(FusedSmem);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return f.indirect ? cudaLaunchKernelEx(&cfg, k_frame_fused<true>, A) : cudaLaunchKernelEx(&cfg, k_frame_fused<false>, A);
}

template <uint32_t kTile>
cudaError_t launch_batch_tiles(const SceneDev* scenes, const uint32_t* tile_scene, uint32_t n, const uint32_t* offs,
                               const uint4* bands, const float4* spos, const uint4* svfme, float4* pos_buf0,
                               float4* pos_buf1, uint4* vfme_buf0, uint4* vfme_buf1, uint32_t* keys, uint32_t* hist,
                               uint32_t* coarse, uint32_t* err, cudaStream_t st, uint32_t* far) {
    PhysParams unused{};
    k_physics_frame<true, false, kTile><<<(n + kTile - 1u) / kTile, kTile, 0, st>>>(
        unused, scenes, tile_scene, n, offs, bands, spos, svfme, nullptr, pos_buf0, pos_buf1, vfme_buf0, vfme_buf1,
        keys, hist, coarse, err, far);
    return cudaGetLastError();
}

cudaError_t launch_physics_batch(const SceneDev* scenes, const uint32_t* tile_scene, uint32_t n,
                                 const uint32_t* offs, const uint4* bands, const float4* spos, const uint4* svfme,
                                 float4* pos_buf0, float4* pos_buf1, uint4* vfme_buf0, uint4* vfme_buf1,
                                 uint32_t* keys, uint32_t* hist, uint32_t* coarse, uint32_t* err, cudaStream_t st,
                                 uint32_t tile, uint32_t* far) {
    if (!n) return cudaSuccess;
    if (tile == 64u)
        return launch_batch_tiles<64u>(scenes, tile_scene, n, offs, bands, spos, svfme, pos_buf0, pos_buf1, vfme_buf0,
                                       vfme_buf1, keys, hist, coarse, err, st, far);
    if (tile == 256u)
        return launch_batch_tiles<256u>(scenes, tile_scene, n, offs, bands, spos, svfme, pos_buf0, pos_buf1,
                                        vfme_buf0, vfme_buf1, keys, hist, coarse, err, st, far);
    return launch_batch_tiles<128u>(scenes, tile_scene, n, offs, bands, spos, svfme, pos_buf0, pos_buf1, vfme_buf0,
                                    vfme_buf1, keys, hist, coarse, err, st, far);
}

cudaError_t launch_rekey(const PhysParams& p, uint32_t n, const float4* pos, uint32_t* keys,
                         uint32_t* hist, uint32_t* coarse, cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_rekey<<<(n + 255u) / 256u, 256, 0, st>>>(p, n, pos, keys, hist, coarse);
    return cudaGetLastError();
}

cudaError_t selftest_divide(uint64_t seed, uint64_t count, uint64_t* mismatches, uint32_t* bad4) {
    unsigned long long* d_mis = nullptr;
    uint32_t* d_bad = nullptr;
    cudaError_t e = cudaMalloc(&d_mis, sizeof(unsigned long long));
    if (!e) e = cudaMalloc(&d_bad, 4 * sizeof(uint32_t));
    if (!e) e = cudaMemset(d_mis, 0, sizeof(unsigned long long));
    if (!e) e = cudaMemset(d_bad, 0, 4 * sizeof(uint32_t));
    if (!e) {
        k_selftest_divide<<<(uint32_t)device_sm_count() * 8u, 256>>>(seed, count, d_mis, d_bad);
        e = cudaGetLastError();
    }
    unsigned long long mis = 0;
    if (!e) e = cudaMemcpy(&mis, d_mis, sizeof(mis), cudaMemcpyDeviceToHost);
    if (!e && bad4) e = cudaMemcpy(bad4, d_bad, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaFree(d_mis);
    cudaFree(d_bad);
    if (!e && mismatches) *mismatches = (uint64_t)mis;
    return e;
}

}  // namespace mb
