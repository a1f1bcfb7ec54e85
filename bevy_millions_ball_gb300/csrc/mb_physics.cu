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

// WGSL min/max: "e2 if e2 < e1 (resp. >), else e1; a NaN operand yields the other".
__device__ __forceinline__ float wmin(float a, float b) {
    if (isnan(a)) return b;
    if (isnan(b)) return a;
    return b < a ? b : a;
}
__device__ __forceinline__ float wmax(float a, float b) {
    if (isnan(a)) return b;
    if (isnan(b)) return a;
    return b > a ? b : a;
}
__device__ __forceinline__ float wclamp(float e, float lo, float hi) { return wmin(wmax(e, lo), hi); }
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

// pack_vfme (physics.wgsl:235-242)
__device__ __forceinline__ uint4 pack(const Agent& a) {
    uint4 q;
    q.x = f2h(a.velocity.x) | (f2h(a.velocity.y) << 16);
    q.y = f2h(a.velocity.z) | (f2h(a.force.x) << 16);
    q.z = f2h(a.force.y) | (f2h(a.force.z) << 16);
    q.w = f2h(a.massv) | (f2h(0.0f) << 16);
    return q;
}

// get_collision_grid_id (physics.wgsl:107-109): saturating f32->u32, integer
// division by GRID_SIZE; clamped to the border cell for positions off the map.
__device__ __forceinline__ void cell_of(const PhysParams& P, float x, float z, uint32_t& cx,
                                        uint32_t& cz) {
    cx = __float2uint_rz(x + P.half_map_size) / P.grid_size;
    cz = __float2uint_rz(z + P.half_map_size) / P.grid_size;
    cx = min(cx, P.N - 1u);
    cz = min(cz, P.N - 1u);
}

// solve_sphere_constraint (physics.wgsl:300-331).  Returns the length factor of
// the position change it applied (0 if none): |dp| <= returned value * |norm|.
__device__ __forceinline__ float sphere(const PhysParams& P, Agent& a, const Agent& b) {
    float edge = b.scale + a.scale;
    V3 tpos = a.position - b.position;
    float dist = len3(tpos);
    float moved = 0.0f;
    if (dist <= edge) {
        V3 norm = normalize3(tpos);
        if (!P.spring) {
            float m1 = a.massv, m2 = b.massv;
            V3 rvel = a.velocity - b.velocity;
            float rspd = dot3(rvel, norm);
            if (rspd < 0.0f) {
                V3 rvel_n = rspd * norm;
                float e_m2 = P.e_agent * m2;
                float num = m1 - e_m2;
                float den = m1 + m2;
                V3 rvel_c = (num * rvel_n) / den;
                a.velocity = (b.velocity + (rvel - rvel_n)) + rvel_c;
            }
            float h = 0.5f * (edge - dist);
            a.position = a.position + h * norm;
            moved = h;
        } else {
            float makeup = edge - dist;
            V3 kforce = (P.k_agent * makeup) * norm;
            V3 cforce = P.neg_c_over_dt * a.velocity;
            a.force = a.force + (kforce + cforce);
            float limit = makeup - P.r_agent * a.scale;
            if (limit > 0.0f) {
                a.position = a.position + limit * norm;
                moved = limit;
            }
        }
    }
    return moved;
}

// solve_cube_constraint (physics.wgsl:269-298)
__device__ __forceinline__ void cube(const PhysParams& P, Agent& a) {
    V3 edge = V3{P.half_map_size, P.half_map_height, P.half_map_size} - splat(a.scale);
    V3 cetr = {0.0f, P.half_map_height, 0.0f};
    V3 tpos = a.position - cetr;
    V3 makeup = {edge.x - fabsf(tpos.x), edge.y - fabsf(tpos.y), edge.z - fabsf(tpos.z)};
    bool tx = makeup.x < 0.0f, ty = makeup.y < 0.0f, tz = makeup.z < 0.0f;
    if (!(tx || ty || tz)) return;
    if (!P.spring) {
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

// solve_sphere_constraint against a packed neighbour (raw float4 + uint4).  The
// distance test first rejects pairs whose squared distance exceeds the squared
// edge by a 0.3% margin: sqrt is monotone and correctly rounded, so such pairs
// can never pass `length(tpos) <= edge`, and all others take the exact path.
__device__ __forceinline__ float sphere_raw(const PhysParams& P, Agent& a, float4 bp, uint4 bq) {
    float edge = bp.w + a.scale;
    V3 tpos = a.position - V3{bp.x, bp.y, bp.z};
    float d2 = dot3(tpos, tpos);
    if (d2 > (edge * edge) * 1.003f) return 0.0f;
    return sphere(P, a, unpack(bp, bq));
}

// main, INIT pipeline (physics.wgsl:91-96): gather through perm, re-pack, emit key.
__global__ void __launch_bounds__(256)
    k_physics_init(PhysParams P, uint32_t n, const uint32_t* __restrict__ perm,
                   const float4* __restrict__ pos_in, const uint4* __restrict__ vfme_in,
                   float4* __restrict__ pos_out, uint4* __restrict__ vfme_out,
                   uint32_t* __restrict__ keys_out, uint32_t* __restrict__ hist) {
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
    if (hist) atomicAdd(hist + key, 1u);
}

// Neighbour row-bands of a tile of sorted slots.  Band b (row offset b-1 = -1, 0,
// +1) is the union of every tile sphere's candidate range in that row: since
// slots are sorted by cell, it is one contiguous slot range.  Bands of at most
// kBandCap slots are staged in shared memory through perm (all loads of a band
// in flight at once); wider bands (a tile spanning a row boundary) are read from
// global memory instead.
constexpr int kTileThreads = 128;
constexpr uint32_t kBandCap = 2 * kTileThreads;

// The candidates of one sphere, in the reference's order (physics.wgsl:119-160):
// own row without itself, row below, row above.  Ordinal o maps to a slot j and
// the shared-memory band holding it (if that band was staged).
struct Cands {
    uint32_t m_lo, n_mid, b_lo, n_bot, t_lo, n_top, self;
    __device__ __forceinline__ uint32_t total() const { return n_mid + n_bot + n_top; }
    __device__ __forceinline__ uint32_t slot(uint32_t o, int& band) const {
        if (o < n_mid) {
            band = 1;
            uint32_t j = m_lo + o;
            return j >= self ? j + 1u : j;
        }
        o -= n_mid;
        if (o < n_bot) {
            band = 0;
            return b_lo + o;
        }
        band = 2;
        return t_lo + (o - n_bot);
    }
};

struct Bands {
    const float4 (*pos)[kBandCap];
    const uint4 (*vfme)[kBandCap];
    const uint32_t* lo;
    const uint32_t* cnt;
};

__device__ __forceinline__ float4 cand_pos(const Bands& B, int band, uint32_t j, uint32_t n,
                                           const uint32_t* __restrict__ perm,
                                           const float4* __restrict__ pos_in) {
    uint32_t r = j - B.lo[band];
    if (r < B.cnt[band]) return B.pos[band][r];
    return __ldg(pos_in + min(__ldg(perm + j), n - 1u));
}
__device__ __forceinline__ uint4 cand_vfme(const Bands& B, int band, uint32_t j, uint32_t n,
                                          const uint32_t* __restrict__ perm,
                                          const uint4* __restrict__ vfme_in) {
    uint32_t r = j - B.lo[band];
    if (r < B.cnt[band]) return B.vfme[band][r];
    return __ldg(vfme_in + min(__ldg(perm + j), n - 1u));
}

// handle_collisions' contact loop (physics.wgsl:122-160), in two phases that give
// the same result as the plain sequential loop:
//  1. the first 64 candidates are classified against the position p0 at loop
//     entry: "near" if within edge + margin (squared test with slack);
//  2. contacts run in candidate order over the near ones only, while a bound on
//     |p - p0| (sum of applied shifts, with rounding slack) stays below the
//     margin: then every skipped candidate is farther than edge from p and
//     would have been a no-op.  If the bound is exceeded, or beyond ordinal 63,
//     the remaining candidates run through the exact loop.
__device__ __forceinline__ void collide_all(const PhysParams& P, Agent& a, const Cands& C,
                                            const Bands& B, uint32_t n,
                                            const uint32_t* __restrict__ perm,
                                            const float4* __restrict__ pos_in,
                                            const uint4* __restrict__ vfme_in) {
    const uint32_t total = C.total();
    uint32_t start = 0;  // ordinals from here on take the exact loop
    // the rounding slack below assumes |coordinate| <= 8192 (ulp <= 2^-10)
    const bool small = fabsf(a.position.x) <= 8192.0f && fabsf(a.position.y) <= 8192.0f &&
                       fabsf(a.position.z) <= 8192.0f;
    if (P.filter_margin > 0.0f && small) {
        uint64_t near = 0;
        const uint32_t nf = min(total, 64u);
        for (uint32_t o = 0; o < nf; ++o) {
            int band;
            uint32_t j = C.slot(o, band);
            float4 bp = cand_pos(B, band, j, n, perm, pos_in);
            float em = (bp.w + a.scale) + P.filter_margin;
            V3 tpos = a.position - V3{bp.x, bp.y, bp.z};
            float d2 = dot3(tpos, tpos);
            if (!(d2 > (em * em) * 1.0001f)) near |= 1ull << o;
        }
        float disp = 0.0f;
        const float limit = P.filter_margin - 0.02f;
        start = nf;
        while (near) {
            uint32_t o = (uint32_t)(__ffsll((long long)near) - 1);
            near &= near - 1ull;
            int band;
            uint32_t j = C.slot(o, band);
            float mv = sphere_raw(P, a, cand_pos(B, band, j, n, perm, pos_in),
                                  cand_vfme(B, band, j, n, perm, vfme_in));
            if (mv != 0.0f) {
                disp = disp + (mv * 1.001f + P.pos_slack);
                if (!(disp <= limit)) {  // moved too far: later skips would not be safe
                    start = o + 1u;
                    break;
                }
            }
        }
    }
    for (uint32_t o = start; o < total; ++o) {
        int band;
        uint32_t j = C.slot(o, band);
        sphere_raw(P, a, cand_pos(B, band, j, n, perm, pos_in), cand_vfme(B, band, j, n, perm, vfme_in));
    }
}

// main, LOOP pipeline (physics.wgsl:57-89): one thread per sorted slot, one
// block per tile of kTileThreads consecutive slots.
__global__ void __launch_bounds__(kTileThreads)
    k_physics_loop(PhysParams P, uint32_t n, const uint32_t* __restrict__ perm,
                   const uint32_t* __restrict__ offs, const float4* __restrict__ pos_in,
                   const uint4* __restrict__ vfme_in, float4* __restrict__ pos_out,
                   uint4* __restrict__ vfme_out, uint32_t* __restrict__ keys_out,
                   uint32_t* __restrict__ hist) {
    __shared__ float4 s_pos[3][kBandCap];
    __shared__ uint4 s_vfme[3][kBandCap];
    __shared__ uint32_t s_lo[3], s_cnt[3], s_kf, s_kl;

    const uint32_t tid = threadIdx.x;
    const uint32_t i0 = blockIdx.x * kTileThreads;
    const uint32_t i = i0 + tid;
    const uint32_t ilast = min(i0 + kTileThreads, n) - 1u;
    const bool valid = i < n;
    const uint32_t N = P.N;

    Agent a;
    uint32_t cx = 0, cz = 0, key = 0;
    if (valid) {
        uint32_t old = min(__ldg(perm + i), n - 1u);
        a = unpack(__ldg(pos_in + old), __ldg(vfme_in + old));
        cell_of(P, a.position.x, a.position.z, cx, cz);
        key = cz * N + cx;
        if (i == i0) s_kf = key;
        if (i == ilast) s_kl = key;
    }
    __syncthreads();
    if (tid < 3) {
        const uint32_t kf = s_kf, kl = s_kl;
        uint32_t lo = 0, hi = 0;
        if (tid == 1) {  // own row
            lo = offs[kf - (kf % N > 0u ? 1u : 0u)];
            hi = offs[kl + (kl % N < N - 1u ? 2u : 1u)];
        } else if (tid == 0) {  // row below, for tile spheres with cz > 0
            if (kl >= N) {
                uint32_t f = max(kf, N);
                lo = offs[f - N - (f % N > 0u ? 1u : 0u)];
                hi = offs[kl - N + (kl % N < N - 1u ? 2u : 1u)];
            }
        } else {  // row above, for tile spheres with cz < N-1
            const uint32_t top = N * (N - 1u);
            if (kf < top) {
                uint32_t l = min(kl, top - 1u);
                lo = offs[kf + N - (kf % N > 0u ? 1u : 0u)];
                hi = offs[l + N + (l % N < N - 1u ? 2u : 1u)];
            }
        }
        hi = min(hi, n);
        s_lo[tid] = lo;
        s_cnt[tid] = (hi > lo && hi - lo <= kBandCap) ? hi - lo : 0u;
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        const uint32_t lo = s_lo[b], cnt = s_cnt[b];
        for (uint32_t r = tid; r < cnt; r += kTileThreads) {
            uint32_t o = min(__ldg(perm + lo + r), n - 1u);
            s_pos[b][r] = __ldg(pos_in + o);
            s_vfme[b][r] = __ldg(vfme_in + o);
        }
    }
    __syncthreads();
    if (!valid) return;

    const uint32_t l = cx > 0u ? 1u : 0u, rr = cx < N - 1u ? 2u : 1u;
    Cands C;
    C.self = i;
    C.m_lo = __ldg(offs + key - l);
    {
        uint32_t hi = min(__ldg(offs + key + rr), n);
        C.n_mid = (hi > C.m_lo && i >= C.m_lo && i < hi) ? hi - C.m_lo - 1u : 0u;  // own cell holds i
    }
    C.b_lo = C.t_lo = 0;
    C.n_bot = C.n_top = 0;
    if (cz > 0u) {
        C.b_lo = __ldg(offs + key - N - l);
        uint32_t hi = min(__ldg(offs + key - N + rr), n);
        C.n_bot = hi > C.b_lo ? hi - C.b_lo : 0u;
    }
    if (cz < N - 1u) {
        C.t_lo = __ldg(offs + key + N - l);
        uint32_t hi = min(__ldg(offs + key + N + rr), n);
        C.n_top = hi > C.t_lo ? hi - C.t_lo : 0u;
    }
    Bands B{s_pos, s_vfme, s_lo, s_cnt};

    // verlet_integration (physics.wgsl:262-266)
    {
        V3 acc = a.force / a.massv;
        a.velocity = a.velocity + ((V3{P.gx, P.gy, P.gz} + acc) * P.dt) * P.dt;
        a.position = a.position + a.velocity;
    }
    a.force = splat(0.0f);

    // handle_collisions (physics.wgsl:119-169): own row, row below, row above
    V3 old_pos = a.position;
    collide_all(P, a, C, B, n, perm, pos_in, vfme_in);
    V3 diff = a.position - old_pos;
    if (len3(diff) > a.scale) {
        // hash3f1u(new_agent_index) * 2 - 1 (physics.wgsl:166, 334-337)
        uint32_t v = i * (i ^ (i >> 15));
        const float d = 4294967296.0f;
        V3 h = {__uint2float_rn(v * 0x1u) / d, __uint2float_rn(v * 0x1FFu) / d,
                __uint2float_rn(v * 0x3FFFFu) / d};
        V3 jitter = {h.x * 2.0f - 1.0f, h.y * 2.0f - 1.0f, h.z * 2.0f - 1.0f};
        a.position = a.position + normalize3(jitter);
    }

    cube(P, a);

    const float lim = 65504.0f;  // CLAMP_F16
    a.velocity = {wclamp(a.velocity.x, -lim, lim), wclamp(a.velocity.y, -lim, lim),
                  wclamp(a.velocity.z, -lim, lim)};
    a.force = {wclamp(a.force.x, -lim, lim), wclamp(a.force.y, -lim, lim), wclamp(a.force.z, -lim, lim)};

    pos_out[i] = make_float4(a.position.x, a.position.y, a.position.z, a.scale);
    vfme_out[i] = pack(a);
    uint32_t nx, nz;
    cell_of(P, a.position.x, a.position.z, nx, nz);
    const uint32_t nk = nz * N + nx;
    keys_out[i] = nk;
    if (hist) atomicAdd(hist + nk, 1u);
}

__global__ void k_rekey(PhysParams P, uint32_t n, const float4* __restrict__ pos,
                        uint32_t* __restrict__ keys, uint32_t* __restrict__ hist) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 p = pos[i];
    uint32_t cx, cz;
    cell_of(P, p.x, p.z, cx, cz);
    keys[i] = cz * P.N + cx;
    if (hist) atomicAdd(hist + keys[i], 1u);
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
    // contact-loop filter margin (collide_all): disabled on maps so large that
    // f32 rounding of positions approaches the margin
    p.filter_margin = c.half_map_size <= 4096.0f ? 0.25f : 0.0f;
    p.pos_slack = 1e-3f;
    return p;
}

cudaError_t launch_physics_init(const PhysParams& p, uint32_t n, const uint32_t* perm,
                                const float4* pos_in, const uint4* vfme_in, float4* pos_out,
                                uint4* vfme_out, uint32_t* keys_out, uint32_t* hist, cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_physics_init<<<(n + 255u) / 256u, 256, 0, st>>>(p, n, perm, pos_in, vfme_in, pos_out, vfme_out,
                                                      keys_out, hist);
    return cudaGetLastError();
}

cudaError_t launch_physics_loop(const PhysParams& p, uint32_t n, const uint32_t* perm,
                                const uint32_t* offs, const float4* pos_in, const uint4* vfme_in,
                                float4* pos_out, uint4* vfme_out, uint32_t* keys_out, uint32_t* hist,
                                cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_physics_loop<<<(n + kTileThreads - 1u) / kTileThreads, kTileThreads, 0, st>>>(
        p, n, perm, offs, pos_in, vfme_in, pos_out, vfme_out, keys_out, hist);
    return cudaGetLastError();
}

cudaError_t launch_rekey(const PhysParams& p, uint32_t n, const float4* pos, uint32_t* keys,
                         uint32_t* hist, cudaStream_t st) {
    if (!n) return cudaSuccess;
    k_rekey<<<(n + 255u) / 256u, 256, 0, st>>>(p, n, pos, keys, hist);
    return cudaGetLastError();
}

}  // namespace mb
