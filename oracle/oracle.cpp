// oracle.cpp — CPU restatement of the reference's per-frame passes.
//
// TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); the product
// library never links it.  Build: oracle/build_oracle.py (-O2 -ffp-contract=off).
// Every function cites the reference line it restates; paths are relative to the
// reference project (bevy_millions_ball).

#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

constexpr uint32_t kInvalid = 0xFFFFFFFFu;  // physics.wgsl:18, spatial_hashing.wgsl:42

// ---------------------------------------------------------------- threading
int resolve_threads(int threads) {
    if (threads > 0) return threads;
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

template <class F>
void parallel_for(uint32_t n, int threads, F&& body) {
    threads = resolve_threads(threads);
    if (threads <= 1 || n < 4096) {
        body(0u, n, 0);
        return;
    }
    std::vector<std::thread> pool;
    uint32_t chunk = (n + (uint32_t)threads - 1) / (uint32_t)threads;
    for (int t = 0; t < threads; ++t) {
        uint32_t b = (uint32_t)t * chunk, e = std::min<uint32_t>(n, b + chunk);
        if (b >= e) break;
        pool.emplace_back([&, b, e, t] { body(b, e, t); });
    }
    for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------- f32 helpers
inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// WGSL min(e1, e2): e2 if e2 < e1, else e1; a NaN operand yields the other.
// max likewise with >.  clamp(e, lo, hi) = min(max(e, lo), hi).
inline float wmin(float a, float b) {
    if (std::isnan(a)) return b;
    if (std::isnan(b)) return a;
    return b < a ? b : a;
}
inline float wmax(float a, float b) {
    if (std::isnan(a)) return b;
    if (std::isnan(b)) return a;
    return b > a ? b : a;
}
inline float wclamp(float e, float lo, float hi) { return wmin(wmax(e, lo), hi); }
// WGSL sign(): 1, -1 or 0.
inline float wsign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }

// f32 -> u32 conversion of WGSL: truncate toward zero, saturate, NaN -> 0.
inline uint32_t f32_to_u32_sat(float v) {
    if (!(v > 0.0f)) return 0u;
    if (v >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)v;
}

struct V3 {
    float x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
inline V3 splat(float s) { return {s, s, s}; }
// dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z, no contraction
inline float dot(V3 a, V3 b) {
    float xx = a.x * b.x;
    float yy = a.y * b.y;
    float zz = a.z * b.z;
    float s = xx + yy;
    return s + zz;
}
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) { return a / length(a); }

// ---------------------------------------------------------------- quantisation
// ShaderDefVal::Int(".." , (x * 1000.) as i32) — Rust float->int casts truncate
// and saturate, NaN -> 0 (mod.rs:473-481).
int32_t q_i32(float x) {
    float v = x * 1000.0f;
    if (std::isnan(v)) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v <= -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}
uint32_t q_u32(float x) { return f32_to_u32_sat(x * 1000.0f); }

}  // namespace

// ================================================================ f16 (IEEE RNE)
// pack2x16float / Rust `as f16` (mod.rs:215-217): binary32 -> binary16 with
// round-to-nearest-even, from the IEEE-754 definition.
extern "C" uint16_t mbo_f32_to_f16(float f) {
    uint32_t x = f2u(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t a = x & 0x7FFFFFFFu;
    if (a > 0x7F800000u) return (uint16_t)(sign | 0x7E00u | ((a >> 13) & 0x3FFu));  // NaN
    if (a >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u);  // >= 65520 -> inf
    if (a >= 0x38800000u) {                                   // normal binary16
        uint32_t base = (a - (112u << 23)) >> 13;
        uint32_t rem = a & 0x1FFFu;
        if (rem > 0x1000u || (rem == 0x1000u && (base & 1u))) ++base;
        return (uint16_t)(sign | base);
    }
    uint32_t e = a >> 23;
    if (e == 0) return (uint16_t)sign;  // zero or binary32 subnormal
    uint32_t m = (a & 0x7FFFFFu) | 0x800000u;
    uint32_t shift = 126u - e;  // value / 2^-24 = m >> shift
    if (shift > 24u) return (uint16_t)sign;
    uint32_t q = m >> shift;
    uint32_t rem = m & ((1u << shift) - 1u);
    uint32_t half = 1u << (shift - 1u);
    if (rem > half || (rem == half && (q & 1u))) ++q;
    return (uint16_t)(sign | q);
}

extern "C" float mbo_f16_to_f32(uint16_t h) {
    uint32_t sign = ((uint32_t)h & 0x8000u) << 16;
    uint32_t e = ((uint32_t)h >> 10) & 0x1Fu;
    uint32_t m = (uint32_t)h & 0x3FFu;
    if (e == 0x1Fu) return u2f(sign | 0x7F800000u | (m << 13));
    if (e == 0) {
        if (m == 0) return u2f(sign);
        // subnormal: m * 2^-24, exact in binary32
        float v = (float)m * 5.9604644775390625e-08f;
        return sign ? -v : v;
    }
    return u2f(sign | ((e + 112u) << 23) | (m << 13));
}

// ================================================================ constants
// CompiledConsts::shader_defs (mod.rs:459-485) and the const declarations of
// physics.wgsl:2-16: every real constant is f32(int) / 1000 evaluated in f32.
extern "C" int mbo_quantize(const mb_settings* s, mb_consts* c) {
    if (!s || !c) return 1;
    std::memset(c, 0, sizeof(*c));
    c->number_of_grids_one_dimension = s->number_of_grids_one_dimension;
    c->grid_size = s->grid_size;
    c->half_map_height = (float)s->half_map_height;
    // half_map_size_u = map_size_u / 2 (mod.rs:393-399)
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
        for (int i = 0; i < 3; ++i) c->gravity[i] = (float)q_i32(s->gravity[i]) / 1000.0f;
        c->e_envir = (float)q_u32(s->e_envir) / 1000.0f;
        c->e_agent = (float)q_u32(s->e_agent) / 1000.0f;
        c->k_agent = (float)q_u32(s->k_agent) / 1000.0f;
        c->c_agent = (float)q_u32(s->c_agent) / 1000.0f;
        c->r_agent = (float)q_u32(s->r_agent) / 1000.0f;
        c->time_delta = (float)q_u32(s->time_delta) / 1000.0f;
    }
    c->enable_spring = s->enable_spring ? 1u : 0u;
    return 0;
}

// ================================================================ cell key
// get_collision_grid_id / get_collision_grid_index (physics.wgsl:107-117):
// cell = vec2u(pos.xz + HALF_MAP_SIZE) / GRID_SIZE; key = cz * N + cx.
// Positions outside the map are clamped to the border cell (the reference
// would index past its tables there; its wall constraint keeps agents inside).
extern "C" uint32_t mbo_cell_key(const mb_consts* c, float x, float z) {
    uint32_t N = c->number_of_grids_one_dimension;
    uint32_t cx = f32_to_u32_sat(x + c->half_map_size) / c->grid_size;
    uint32_t cz = f32_to_u32_sat(z + c->half_map_size) / c->grid_size;
    if (cx > N - 1u) cx = N - 1u;
    if (cz > N - 1u) cz = N - 1u;
    return cz * N + cx;
}

// hash3f1u (physics.wgsl:334-337)
extern "C" void mbo_hash3f1u(uint32_t n, float out[3]) {
    uint32_t v = n * (n ^ (n >> 15));
    const float d = 4294967296.0f;  // f32(0xFFFFFFFFu) rounds to 2^32
    out[0] = (float)(v * 0x1u) / d;
    out[1] = (float)(v * 0x1FFu) / d;
    out[2] = (float)(v * 0x3FFFFu) / d;
}

// ================================================================ radix sort
// bevy_radix_sort::run(.., 0..passes, vals_are_iota, ..) as called at
// mod.rs:880-890: stable LSD sort by 8-bit digits.  Parallel version: per-thread
// digit histograms over contiguous chunks, digit-major/thread-minor offsets,
// order-preserving scatter — the result equals a sequential stable sort.
extern "C" void mbo_radix_sort(const uint32_t* keys, const uint32_t* vals, uint32_t n,
                               uint32_t passes, uint32_t* keys_out, uint32_t* vals_out,
                               int threads) {
    std::vector<uint32_t> ka(keys, keys + n), va(n), kb(n), vb(n);
    if (vals) std::memcpy(va.data(), vals, sizeof(uint32_t) * n);
    else for (uint32_t i = 0; i < n; ++i) va[i] = i;
    int T = resolve_threads(threads);
    if (n < 65536) T = 1;
    uint32_t chunk = n ? (n + (uint32_t)T - 1) / (uint32_t)T : 0;
    std::vector<uint32_t> hist((size_t)T * 256);
    for (uint32_t p = 0; p < passes; ++p) {
        uint32_t shift = 8u * p;
        std::fill(hist.begin(), hist.end(), 0u);
        auto count = [&](int t) {
            uint32_t b = (uint32_t)t * chunk, e = std::min(n, b + chunk);
            uint32_t* h = &hist[(size_t)t * 256];
            for (uint32_t i = b; i < e; ++i) h[(ka[i] >> shift) & 0xFFu]++;
        };
        auto scatter = [&](int t, std::vector<uint32_t>& offs) {
            uint32_t b = (uint32_t)t * chunk, e = std::min(n, b + chunk);
            uint32_t* o = &offs[(size_t)t * 256];
            for (uint32_t i = b; i < e; ++i) {
                uint32_t d = (ka[i] >> shift) & 0xFFu;
                uint32_t dst = o[d]++;
                kb[dst] = ka[i];
                vb[dst] = va[i];
            }
        };
        std::vector<uint32_t> offs((size_t)T * 256);
        if (T == 1) {
            count(0);
        } else {
            std::vector<std::thread> pool;
            for (int t = 0; t < T; ++t) pool.emplace_back(count, t);
            for (auto& th : pool) th.join();
        }
        uint32_t run = 0;
        for (uint32_t d = 0; d < 256; ++d)
            for (int t = 0; t < T; ++t) {
                offs[(size_t)t * 256 + d] = run;
                run += hist[(size_t)t * 256 + d];
            }
        if (T == 1) {
            scatter(0, offs);
        } else {
            std::vector<std::thread> pool;
            for (int t = 0; t < T; ++t) pool.emplace_back(scatter, t, std::ref(offs));
            for (auto& th : pool) th.join();
        }
        ka.swap(kb);
        va.swap(vb);
    }
    std::memcpy(keys_out, ka.data(), sizeof(uint32_t) * n);
    std::memcpy(vals_out, va.data(), sizeof(uint32_t) * n);
}

// ================================================================ cell ranges
// ZEROING (spatial_hashing.wgsl:29-44) over all cells — the reference clears
// only n entries and so relies on n >= N*N (mod.rs:351-362); clearing every
// cell is the intended meaning.  HASHING (spatial_hashing.wgsl:46-70): a sorted
// slot whose key differs from its predecessor starts its cell, one that differs
// from its successor closes it (close is inclusive).  The ends compare with the
// sentinel 0xFFFFFFFF - key, which always differs.
extern "C" void mbo_spatial_hash(const uint32_t* sk, uint32_t n, uint32_t cells, uint32_t* start,
                                 uint32_t* close) {
    for (uint32_t c = 0; c < cells; ++c) {
        start[c] = kInvalid;
        if (close) close[c] = kInvalid;
    }
    for (uint32_t t = 0; t < n; ++t) {
        uint32_t k = sk[t];
        uint32_t prv = kInvalid - k, nxt = kInvalid - k;
        if (t > 0u) prv = sk[t - 1u];
        if (t < n - 1u) nxt = sk[t + 1u];
        if (k >= cells) continue;  // out-of-table keys are dropped (robust access)
        if (k != prv) start[k] = t;
        if (k != nxt && close) close[k] = t;
    }
}

// ================================================================ physics
namespace {

struct Agent {  // physics.wgsl:208-215
    V3 position;
    float scale;
    V3 velocity;  // displacement per step
    float massv;
    V3 force;
};

// unpack_vfme (physics.wgsl:244-253) and agent_new (217-233)
inline Agent agent_load(const float* pos, const uint32_t* vfme, uint32_t idx) {
    Agent a;
    const float* p = pos + 4ull * idx;
    const uint32_t* q = vfme + 4ull * idx;
    a.position = {p[0], p[1], p[2]};
    a.scale = p[3];
    a.velocity = {mbo_f16_to_f32((uint16_t)(q[0] & 0xFFFFu)), mbo_f16_to_f32((uint16_t)(q[0] >> 16)),
                  mbo_f16_to_f32((uint16_t)(q[1] & 0xFFFFu))};
    a.force = {mbo_f16_to_f32((uint16_t)(q[1] >> 16)), mbo_f16_to_f32((uint16_t)(q[2] & 0xFFFFu)),
               mbo_f16_to_f32((uint16_t)(q[2] >> 16))};
    a.massv = mbo_f16_to_f32((uint16_t)(q[3] & 0xFFFFu));
    return a;
}

inline uint32_t pack2(float a, float b) {
    return (uint32_t)mbo_f32_to_f16(a) | ((uint32_t)mbo_f32_to_f16(b) << 16);
}

// pack_vfme (physics.wgsl:235-242)
inline void agent_store(const Agent& a, float* pos, uint32_t* vfme, uint32_t idx) {
    float* p = pos + 4ull * idx;
    uint32_t* q = vfme + 4ull * idx;
    p[0] = a.position.x;
    p[1] = a.position.y;
    p[2] = a.position.z;
    p[3] = a.scale;
    q[0] = pack2(a.velocity.x, a.velocity.y);
    q[1] = pack2(a.velocity.z, a.force.x);
    q[2] = pack2(a.force.y, a.force.z);
    q[3] = pack2(a.massv, 0.0f);
}

struct Ctx {
    const mb_consts* c;
    uint32_t N;
    float neg_c_over_dt;       // -C_AGENT / T_DELTA          (physics.wgsl:285, 324)
    float neg_1pe_over_dt;     // -(1. + E_ENVIR) / T_DELTA   (physics.wgsl:292)
    V3 gravity;
    const uint32_t* perm;
    const uint32_t* start;
    const uint32_t* close;
    const float* pos_in;
    const uint32_t* vfme_in;
};

// verlet_integration (physics.wgsl:262-266)
inline void verlet(const Ctx& x, Agent& a) {
    float dt = x.c->time_delta;
    V3 acc = a.force / a.massv;
    a.velocity = a.velocity + ((x.gravity + acc) * dt) * dt;
    a.position = a.position + a.velocity;
}

// solve_sphere_constraint (physics.wgsl:300-331)
inline void sphere(const Ctx& x, Agent& a, const Agent& b) {
    float edge = b.scale + a.scale;
    V3 tpos = a.position - b.position;
    float dist = length(tpos);
    if (dist <= edge) {
        V3 norm = normalize(tpos);
        if (!x.c->enable_spring) {
            float m1 = a.massv, m2 = b.massv;
            V3 rvel = a.velocity - b.velocity;
            float rspd = dot(rvel, norm);
            if (rspd < 0.0f) {
                V3 rvel_n = rspd * norm;
                float e_m2 = x.c->e_agent * m2;
                float num = m1 - e_m2;
                float den = m1 + m2;
                V3 rvel_c = (num * rvel_n) / den;
                a.velocity = (b.velocity + (rvel - rvel_n)) + rvel_c;
            }
            float h = 0.5f * (edge - dist);
            a.position = a.position + h * norm;
        } else {
            float makeup = edge - dist;
            V3 kforce = (x.c->k_agent * makeup) * norm;
            V3 cforce = x.neg_c_over_dt * a.velocity;
            a.force = a.force + (kforce + cforce);
            float limit = makeup - x.c->r_agent * a.scale;
            if (limit > 0.0f) a.position = a.position + limit * norm;
        }
    }
}

// handle_collision (physics.wgsl:171-206): a row of three cells, each empty cell
// skipped, merged into one contiguous slot range.
inline void row(const Ctx& x, Agent& a, uint32_t cx, uint32_t base) {
    uint32_t s = kInvalid, e = 0u;
    if (cx > 0u) {
        uint32_t si = x.start[base - 1u];
        if (si != kInvalid) {
            s = si;
            e = x.close[base - 1u];
        }
    }
    {
        uint32_t si = x.start[base];
        if (si != kInvalid) {
            if (s == kInvalid) s = si;
            e = x.close[base];
        }
    }
    if (cx < x.N - 1u) {
        uint32_t si = x.start[base + 1u];
        if (si != kInvalid) {
            if (s == kInvalid) s = si;
            e = x.close[base + 1u];
        }
    }
    if (s == kInvalid) return;  // for (i = INVALID; i <= 0; ..) runs zero times
    for (uint32_t j = s; j <= e; ++j) {
        Agent b = agent_load(x.pos_in, x.vfme_in, x.perm[j]);
        sphere(x, a, b);
    }
}

// handle_collisions (physics.wgsl:119-169)
inline void collisions(const Ctx& x, Agent& a, uint32_t slot, uint32_t cx, uint32_t cz,
                       uint32_t key) {
    V3 old = a.position;
    {  // middle row: own cell (never empty), left and right neighbours
        uint32_t s = x.start[key];
        uint32_t e = x.close[key];
        if (cx > 0u) {
            uint32_t si = x.start[key - 1u];
            if (si != kInvalid) s = si;
        }
        if (cx < x.N - 1u) {
            uint32_t si = x.start[key + 1u];
            if (si != kInvalid) e = x.close[key + 1u];
        }
        for (uint32_t j = s; j <= e; ++j) {
            if (j == slot) continue;
            Agent b = agent_load(x.pos_in, x.vfme_in, x.perm[j]);
            sphere(x, a, b);
        }
    }
    if (cz > 0u) row(x, a, cx, key - x.N);         // bottom
    if (cz < x.N - 1u) row(x, a, cx, key + x.N);   // top
    V3 diff = a.position - old;
    if (length(diff) > a.scale) {
        float h[3];
        mbo_hash3f1u(slot, h);
        V3 jitter = {h[0] * 2.0f - 1.0f, h[1] * 2.0f - 1.0f, h[2] * 2.0f - 1.0f};
        a.position = a.position + normalize(jitter);
    }
}

// solve_cube_constraint (physics.wgsl:269-298)
inline void cube(const Ctx& x, Agent& a) {
    const mb_consts* c = x.c;
    V3 edge = V3{c->half_map_size, c->half_map_height, c->half_map_size} - splat(a.scale);
    V3 cetr = {0.0f, c->half_map_height, 0.0f};
    V3 tpos = a.position - cetr;
    V3 makeup = {edge.x - std::fabs(tpos.x), edge.y - std::fabs(tpos.y), edge.z - std::fabs(tpos.z)};
    bool tx = makeup.x < 0.0f, ty = makeup.y < 0.0f, tz = makeup.z < 0.0f;
    if (!(tx || ty || tz)) return;
    if (!c->enable_spring) {
        a.position = V3{wclamp(tpos.x, -edge.x, edge.x), wclamp(tpos.y, -edge.y, edge.y),
                        wclamp(tpos.z, -edge.z, edge.z)} + cetr;
        float ne = -c->e_envir;
        V3 f = {tx ? ne : 1.0f, ty ? ne : 1.0f, tz ? ne : 1.0f};
        a.velocity = a.velocity * f;
    } else {
        float mm = -(a.scale * c->r_agent);
        V3 min_makeup = splat(mm);
        V3 sgn = {wsign(tpos.x), wsign(tpos.y), wsign(tpos.z)};
        V3 kforce = (c->k_agent * sgn) * V3{wclamp(makeup.x, mm, 0.0f), wclamp(makeup.y, mm, 0.0f),
                                            wclamp(makeup.z, mm, 0.0f)};
        V3 cforce = x.neg_c_over_dt * a.velocity;
        a.force = a.force + (kforce + cforce);
        bool ux = makeup.x < min_makeup.x, uy = makeup.y < min_makeup.y, uz = makeup.z < min_makeup.z;
        if (ux || uy || uz) {
            V3 e2 = edge - min_makeup;
            a.position = V3{wclamp(tpos.x, -e2.x, e2.x), wclamp(tpos.y, -e2.y, e2.y),
                            wclamp(tpos.z, -e2.z, e2.z)} + cetr;
            V3 sel = {ux ? a.velocity.x : 0.0f, uy ? a.velocity.y : 0.0f, uz ? a.velocity.z : 0.0f};
            V3 dv = x.neg_1pe_over_dt * sel;
            V3 acc = dv / c->time_delta;
            a.force = a.force + a.massv * acc;
        }
    }
}

}  // namespace

// main (physics.wgsl:57-97), one call per sorted slot
extern "C" void mbo_physics(const mb_consts* c, int init, uint32_t n, const uint32_t* perm,
                            const uint32_t* start, const uint32_t* close, const float* pos_in,
                            const uint32_t* vfme_in, float* pos_out, uint32_t* vfme_out,
                            uint32_t* keys_out, int threads) {
    Ctx x;
    x.c = c;
    x.N = c->number_of_grids_one_dimension;
    x.neg_c_over_dt = -c->c_agent / c->time_delta;
    x.neg_1pe_over_dt = -(1.0f + c->e_envir) / c->time_delta;
    x.gravity = {c->gravity[0], c->gravity[1], c->gravity[2]};
    x.perm = perm;
    x.start = start;
    x.close = close;
    x.pos_in = pos_in;
    x.vfme_in = vfme_in;
    const float lim = 65504.0f;  // CLAMP_F16 (physics.wgsl:19)
    parallel_for(n, threads, [&](uint32_t b, uint32_t e, int) {
        for (uint32_t i = b; i < e; ++i) {
            Agent a = agent_load(pos_in, vfme_in, perm[i]);
            uint32_t key = mbo_cell_key(c, a.position.x, a.position.z);
            if (init) {
                agent_store(a, pos_out, vfme_out, i);
                keys_out[i] = key;
                continue;
            }
            uint32_t cx = key % x.N, cz = key / x.N;
            verlet(x, a);
            a.force = splat(0.0f);
            collisions(x, a, i, cx, cz, key);
            cube(x, a);
            a.velocity = {wclamp(a.velocity.x, -lim, lim), wclamp(a.velocity.y, -lim, lim),
                          wclamp(a.velocity.z, -lim, lim)};
            a.force = {wclamp(a.force.x, -lim, lim), wclamp(a.force.y, -lim, lim),
                       wclamp(a.force.z, -lim, lim)};
            agent_store(a, pos_out, vfme_out, i);
            keys_out[i] = mbo_cell_key(c, a.position.x, a.position.z);
        }
    });
}

// ================================================================ world
struct mbo_world {
    mb_settings s;
    mb_consts c;
    uint32_t n = 0, cells = 0;
    int64_t time = -1;
    bool has_state = false;
    std::vector<float> pos[2];
    std::vector<uint32_t> vfme[2];
    std::vector<uint32_t> keys, sorted_keys, perm, start, close;
    int cur = 0;
};

namespace {
bool settings_ok(const mb_settings* s) {
    if (!s) return false;
    if (s->max_number_of_agents == 0 || s->number_of_grids_one_dimension == 0 || s->grid_size == 0)
        return false;
    uint64_t cells = (uint64_t)s->number_of_grids_one_dimension * s->number_of_grids_one_dimension;
    return cells <= (1ull << 30);
}
}  // namespace

extern "C" mbo_world* mbo_create(const mb_settings* s) {
    if (!settings_ok(s)) return nullptr;
    mbo_world* w = new mbo_world();
    w->s = *s;
    mbo_quantize(s, &w->c);
    w->n = s->max_number_of_agents;
    w->cells = s->number_of_grids_one_dimension * s->number_of_grids_one_dimension;
    for (int i = 0; i < 2; ++i) {
        w->pos[i].assign(4ull * w->n, 0.0f);
        w->vfme[i].assign(4ull * w->n, 0u);
    }
    w->keys.assign(w->n, 0u);
    w->sorted_keys.assign(w->n, 0u);
    w->perm.assign(w->n, 0u);
    w->start.assign(w->cells, kInvalid);
    w->close.assign(w->cells, kInvalid);
    return w;
}

extern "C" void mbo_destroy(mbo_world* w) { delete w; }

extern "C" int mbo_set_settings(mbo_world* w, const mb_settings* s) {
    if (!w || !settings_ok(s) || s->max_number_of_agents != w->n) return 1;
    uint32_t oldN = w->s.number_of_grids_one_dimension, oldg = w->s.grid_size;
    w->s = *s;
    mbo_quantize(s, &w->c);
    if (s->number_of_grids_one_dimension != oldN || s->grid_size != oldg) {
        w->cells = s->number_of_grids_one_dimension * s->number_of_grids_one_dimension;
        w->start.assign(w->cells, kInvalid);
        w->close.assign(w->cells, kInvalid);
        // keys emitted with the old grid are re-derived with the new one; before
        // the first frame they are still the all-zero keys of a fresh upload
        if (w->time > 0) {
            const float* p = w->pos[w->cur].data();
            for (uint32_t i = 0; i < w->n; ++i)
                w->keys[i] = mbo_cell_key(&w->c, p[4ull * i], p[4ull * i + 2]);
        }
    }
    return 0;
}

extern "C" int mbo_set_state(mbo_world* w, const float* pos, const uint32_t* vfme) {
    if (!w || !pos || !vfme) return 1;
    std::memcpy(w->pos[0].data(), pos, sizeof(float) * 4ull * w->n);
    std::memcpy(w->vfme[0].data(), vfme, sizeof(uint32_t) * 4ull * w->n);
    w->cur = 0;
    // fresh sort buffers hold zeros: frame 0 sorts all-zero keys (identity perm)
    std::fill(w->keys.begin(), w->keys.end(), 0u);
    w->time = 0;
    w->has_state = true;
    return 0;
}

extern "C" int mbo_get_state(const mbo_world* w, float* pos, uint32_t* vfme) {
    if (!w || !w->has_state) return 1;
    if (pos) std::memcpy(pos, w->pos[w->cur].data(), sizeof(float) * 4ull * w->n);
    if (vfme) std::memcpy(vfme, w->vfme[w->cur].data(), sizeof(uint32_t) * 4ull * w->n);
    return 0;
}

// One frame of PhysicsNode::run (mod.rs:846-912): sort -> hash -> physics.
extern "C" int mbo_step(mbo_world* w, uint32_t k, int threads) {
    if (!w || !w->has_state) return 1;
    if (!w->s.enable_simulation) return 0;
    uint32_t bits = 1;
    while (bits < 32 && (1ull << bits) < w->cells) ++bits;
    uint32_t passes = (bits + 7u) / 8u;
    for (uint32_t f = 0; f < k; ++f) {
        mbo_radix_sort(w->keys.data(), nullptr, w->n, passes, w->sorted_keys.data(), w->perm.data(),
                       threads);
        mbo_spatial_hash(w->sorted_keys.data(), w->n, w->cells, w->start.data(), w->close.data());
        int nxt = w->cur ^ 1;
        mbo_physics(&w->c, w->time == 0, w->n, w->perm.data(), w->start.data(), w->close.data(),
                    w->pos[w->cur].data(), w->vfme[w->cur].data(), w->pos[nxt].data(),
                    w->vfme[nxt].data(), w->keys.data(), threads);
        w->cur = nxt;
        w->time += 1;
    }
    return 0;
}

extern "C" int mbo_get_debug(const mbo_world* w, uint32_t* keys, uint32_t* perm, uint32_t* start,
                             uint32_t* close) {
    if (!w) return 1;
    if (keys) std::memcpy(keys, w->keys.data(), sizeof(uint32_t) * w->n);
    if (perm) std::memcpy(perm, w->perm.data(), sizeof(uint32_t) * w->n);
    if (start) std::memcpy(start, w->start.data(), sizeof(uint32_t) * w->cells);
    if (close) std::memcpy(close, w->close.data(), sizeof(uint32_t) * w->cells);
    return 0;
}

extern "C" int64_t mbo_time(const mbo_world* w) { return w ? w->time : -1; }

extern "C" int mbo_hardware_threads(void) { return resolve_threads(0); }

// ---------------------------------------------------------------- impostor render
// Test infrastructure: CPU restatement of the headless top-down impostor render
// (the per-fragment arithmetic of src/custom_materials/physics_ball/
// deferred_physics_ball.wgsl:26-107 and src/custom_materials/sdf.wgsl:11-27,
// 93-109 for an orthographic view straight down), in the same operation order
// as the library's renderer so that results agree up to exp2/log2 rounding.
namespace {
struct RSphere {
    float x, y, z, r;
};
RSphere grown(const float* p) {  // temporary_solution (deferred_physics_ball.wgsl:28-33)
    float x = std::fmin(std::fmax(p[1] / p[3], 0.0f), 1.0f);
    float y = 0.26f * (x - 1.0f) * (x - 1.0f) + 1.0f;
    return {p[0], p[1], p[2], p[3] * y};
}
float len3r(float x, float y, float z) { return std::sqrt(x * x + y * y + z * z); }
float smooth_max_r(float a, float b, float k) {
    const float ki = 1.0f / k;
    return k * std::log2(std::exp2(a * ki) + std::exp2(b * ki));
}
}  // namespace

extern "C" void mbo_render_topdown(const float* pos4, uint32_t n, uint32_t w, uint32_t h, float x0, float z0,
                                   float x1, float z1, uint32_t* rgba, float* height, uint32_t* winner) {
    const float sx = (x1 - x0) / (float)w, sz = (z1 - z0) / (float)h;
    std::vector<uint64_t> zb((size_t)w * h, 0ull);
    for (uint32_t i = 0; i < n; ++i) {
        const RSphere s = grown(pos4 + 4 * (size_t)i);
        if (!(s.r > 0.0f)) continue;
        const float u0 = std::ceil((s.x - s.r - x0) / sx - 0.5f), u1 = std::floor((s.x + s.r - x0) / sx - 0.5f);
        const float v0 = std::ceil((s.z - s.r - z0) / sz - 0.5f), v1 = std::floor((s.z + s.r - z0) / sz - 0.5f);
        if (!(u1 >= 0.0f && v1 >= 0.0f && u0 < (float)w && v0 < (float)h)) continue;
        const int ua = (int)std::fmax(u0, 0.0f), ub = (int)std::fmin(u1, (float)w - 1.0f);
        const int va = (int)std::fmax(v0, 0.0f), vb = (int)std::fmin(v1, (float)h - 1.0f);
        const float r2 = s.r * s.r;
        for (int v = va; v <= vb; ++v) {
            const float dz = z0 + ((float)v + 0.5f) * sz - s.z;
            for (int u = ua; u <= ub; ++u) {
                const float dx = x0 + ((float)u + 0.5f) * sx - s.x;
                const float c2 = r2 - (dx * dx + dz * dz);
                if (c2 < 0.0f) continue;
                float top = s.y + std::sqrt(c2);
                top = top > 0.0f ? top : 0.0f;
                uint32_t bits;
                std::memcpy(&bits, &top, 4);
                const uint64_t key = ((uint64_t)bits << 32) | (uint64_t)(i + 1u);
                uint64_t& z = zb[(size_t)v * w + u];
                if (key > z) z = key;
            }
        }
    }
    const float K = 0.08f;
    for (size_t p = 0; p < (size_t)w * h; ++p) {
        const uint32_t u = (uint32_t)(p % w), v = (uint32_t)(p / w);
        const uint64_t key = zb[p];
        const uint32_t floor_rgba = 0xFF4D4D4Du;
        if (winner) winner[p] = (uint32_t)(key & 0xFFFFFFFFull);  // sphere index + 1, 0 = none
        if (key == 0ull) {
            rgba[p] = floor_rgba;
            height[p] = 0.0f;
            continue;
        }
        const RSphere s = grown(pos4 + 4 * (size_t)((uint32_t)(key & 0xFFFFFFFFull) - 1u));
        float hx = x0 + ((float)u + 0.5f) * sx, hz = z0 + ((float)v + 0.5f) * sz;
        const uint32_t hb = (uint32_t)(key >> 32);
        float hy;
        std::memcpy(&hy, &hb, 4);
        float nx = hx - s.x, ny = hy - s.y, nz = hz - s.z;
        const float nl = len3r(nx, ny, nz);
        nx /= nl;
        ny /= nl;
        nz /= nl;
        float sd_sphere = 0.0f, sd_plane = -hy;
        bool hit = false;
        for (int it = 0; it < 16; ++it) {
            const float d = smooth_max_r(sd_sphere, sd_plane, K);
            hy -= d;
            if (d < 0.001f) {
                hit = true;
                break;
            }
            sd_sphere = len3r(hx - s.x, hy - s.y, hz - s.z) - s.r;
            sd_plane = -hy;
        }
        if (!hit) {
            rgba[p] = floor_rgba;
            height[p] = 0.0f;
            continue;
        }
        const float hh = (sd_plane - sd_sphere) / K;
        const float pa = 1.0f / (1.0f + std::exp2(hh)), pb = 1.0f / (1.0f + std::exp2(-hh));
        float gx = pa * nx, gy = pa * ny - pb, gz = pa * nz;
        const float gl = len3r(gx, gy, gz);
        if (gl > 0.0f) {
            gx /= gl;
            gy /= gl;
            gz /= gl;
        }
        const float lx = 0.3713907f, ly = 0.9284767f, lz = 0.0f;
        const float lit = 0.25f + 0.75f * std::fmax(gx * lx + gy * ly + gz * lz, 0.0f);
        const uint32_t r = (uint32_t)std::fmin(255.0f * lit + 0.5f, 255.0f);
        const uint32_t g = (uint32_t)std::fmin(191.0f * lit + 0.5f, 255.0f);
        rgba[p] = 0xFF000000u | r | (g << 8);
        height[p] = hy;
    }
}

// CPU restatement of the perspective view (mb_render_view), in the library's
// operation order: camera basis, pixel rays, nearest sphere per pixel (ties to
// the lower index), the shader's march and normal along the pixel's ray, GGX +
// Lambert + ambient lighting, sRGB encoding, the box interior behind.
namespace {
struct RCam {
    float ex, ey, ez, gx, gy, gz, th, ta, lx, ly, lz, hs, top;
    uint32_t w, h;
    float fx, fy, fz, rx, ry, rz, ux, uy, uz;
};
void rbasis(RCam& C) {
    float fx = C.gx - C.ex, fy = C.gy - C.ey, fz = C.gz - C.ez;
    float l = len3r(fx, fy, fz);
    C.fx = fx / l;
    C.fy = fy / l;
    C.fz = fz / l;
    float rx = -C.fz, rz = C.fx;
    l = std::sqrt(rx * rx + rz * rz);
    C.rx = rx / l;
    C.ry = 0.0f;
    C.rz = rz / l;
    C.ux = C.ry * C.fz - C.rz * C.fy;
    C.uy = C.rz * C.fx - C.rx * C.fz;
    C.uz = C.rx * C.fy - C.ry * C.fx;
}
void rray(const RCam& C, uint32_t u, uint32_t v, float& dx, float& dy, float& dz) {
    const float sx = (2.0f * ((float)u + 0.5f) / (float)C.w - 1.0f) * C.ta;
    const float sy = (1.0f - 2.0f * ((float)v + 0.5f) / (float)C.h) * C.th;
    const float x = C.fx + sx * C.rx + sy * C.ux, y = C.fy + sx * C.ry + sy * C.uy, z = C.fz + sx * C.rz + sy * C.uz;
    const float l = len3r(x, y, z);
    dx = x / l;
    dy = y / l;
    dz = z / l;
}
float rsphere(const RCam& C, float dx, float dy, float dz, const RSphere& s) {
    const float ox = C.ex - s.x, oy = C.ey - s.y, oz = C.ez - s.z;
    const float b = ox * dx + oy * dy + oz * dz;
    const float c = (ox * ox + oy * oy + oz * oz) - s.r * s.r;
    const float disc = b * b - c;
    if (!(disc >= 0.0f)) return -1.0f;
    return -b - std::sqrt(disc);
}
float rsrgb8(float x) {
    x = std::fmin(std::fmax(x, 0.0f), 1.0f);
    const float e = x <= 0.0031308f ? 12.92f * x : 1.055f * std::pow(x, 1.0f / 2.4f) - 0.055f;
    return std::fmin(255.0f * e + 0.5f, 255.0f);
}
uint32_t rrgba8(float r, float g, float b) {
    return 0xFF000000u | (uint32_t)rsrgb8(r) | ((uint32_t)rsrgb8(g) << 8) | ((uint32_t)rsrgb8(b) << 16);
}
}  // namespace

extern "C" void mbo_reference_view(float* eye, float* target, float* fov_degrees, float* to_light) {
    eye[0] = 0.0f;
    eye[1] = 64.0f;
    eye[2] = 64.0f;
    target[0] = target[1] = target[2] = 0.0f;
    *fov_degrees = 45.0f;
    const double pi = 3.14159265358979323846, b = -0.15 * pi, c = -0.15 * pi;
    const double x = -std::cos(c) * std::sin(b), y = std::sin(c), z = -std::cos(c) * std::cos(b);
    to_light[0] = (float)-x;
    to_light[1] = (float)-y;
    to_light[2] = (float)-z;
}

extern "C" void mbo_render_view(const float* pos4, uint32_t n, uint32_t w, uint32_t h, const float* eye,
                                const float* target, float fov_degrees, const float* to_light, float half_map_size,
                                float map_top, uint32_t* rgba, float* depth, uint32_t* winner) {
    RCam C{};
    C.ex = eye[0];
    C.ey = eye[1];
    C.ez = eye[2];
    C.gx = target[0];
    C.gy = target[1];
    C.gz = target[2];
    C.th = (float)std::tan((double)fov_degrees * 3.14159265358979323846 / 360.0);
    C.ta = C.th * ((float)w / (float)h);
    C.lx = to_light[0];
    C.ly = to_light[1];
    C.lz = to_light[2];
    C.hs = half_map_size;
    C.top = map_top;
    C.w = w;
    C.h = h;
    rbasis(C);
    std::vector<uint64_t> zb((size_t)w * h, ~0ull);
    for (uint32_t i = 0; i < n; ++i) {
        const RSphere s = grown(pos4 + 4 * (size_t)i);
        if (!(s.r > 0.0f)) continue;
        const float px = s.x - C.ex, py = s.y - C.ey, pz = s.z - C.ez;
        const float cx = px * C.rx + py * C.ry + pz * C.rz, cy = px * C.ux + py * C.uy + pz * C.uz,
                    cz = px * C.fx + py * C.fy + pz * C.fz;
        if (!(cz - s.r > 1e-3f)) continue;
        const float zn = cz - s.r, zf = cz + s.r;
        const float xl = cx - s.r, xh = cx + s.r, yl = cy - s.r, yh = cy + s.r;
        const float sxl = xl / (xl >= 0.0f ? zf : zn), sxh = xh / (xh >= 0.0f ? zn : zf);
        const float syl = yl / (yl >= 0.0f ? zf : zn), syh = yh / (yh >= 0.0f ? zn : zf);
        const float ua = (sxl / C.ta + 1.0f) * 0.5f * (float)w - 1.5f, ub = (sxh / C.ta + 1.0f) * 0.5f * (float)w + 0.5f;
        const float va = (1.0f - syh / C.th) * 0.5f * (float)h - 1.5f, vb = (1.0f - syl / C.th) * 0.5f * (float)h + 0.5f;
        if (!(ub >= 0.0f && vb >= 0.0f && ua < (float)w && va < (float)h)) continue;
        const int u0 = (int)std::fmax(std::ceil(ua), 0.0f), u1 = (int)std::fmin(std::floor(ub), (float)w - 1.0f);
        const int v0 = (int)std::fmax(std::ceil(va), 0.0f), v1 = (int)std::fmin(std::floor(vb), (float)h - 1.0f);
        for (int v = v0; v <= v1; ++v) {
            for (int u = u0; u <= u1; ++u) {
                float dx, dy, dz;
                rray(C, (uint32_t)u, (uint32_t)v, dx, dy, dz);
                const float t = rsphere(C, dx, dy, dz, s);
                if (!(t > 0.0f)) continue;
                uint32_t bits;
                std::memcpy(&bits, &t, 4);
                const uint64_t key = ((uint64_t)bits << 32) | (uint64_t)(i + 1u);
                uint64_t& z = zb[(size_t)v * w + u];
                if (key < z) z = key;
            }
        }
    }
    const float K = 0.08f, kAmbient = 0.2f, kAlpha = 0.435f * 0.435f, kF0 = 0.04f, kPi = 3.14159265f;
    for (size_t p = 0; p < (size_t)w * h; ++p) {
        const uint32_t u = (uint32_t)(p % w), v = (uint32_t)(p / w);
        float dx, dy, dz;
        rray(C, u, v, dx, dy, dz);
        const uint64_t key = zb[p];
        if (winner) winner[p] = key == ~0ull ? 0u : (uint32_t)(key & 0xFFFFFFFFull);
        if (key != ~0ull) {
            const RSphere s = grown(pos4 + 4 * (size_t)((uint32_t)(key & 0xFFFFFFFFull) - 1u));
            const uint32_t tb = (uint32_t)(key >> 32);
            float t;
            std::memcpy(&t, &tb, 4);
            float hx = C.ex + t * dx, hy = C.ey + t * dy, hz = C.ez + t * dz;
            float nx = hx - s.x, ny = hy - s.y, nz = hz - s.z;
            const float nl = len3r(nx, ny, nz);
            nx /= nl;
            ny /= nl;
            nz /= nl;
            float sd_sphere = 0.0f, sd_plane = -hy, walked = 0.0f;
            bool hit = false;
            for (int it = 0; it < 16; ++it) {
                const float d = smooth_max_r(sd_sphere, sd_plane, K);
                hx += d * dx;
                hy += d * dy;
                hz += d * dz;
                walked += d;
                if (d < 0.001f) {
                    hit = true;
                    break;
                }
                sd_sphere = len3r(hx - s.x, hy - s.y, hz - s.z) - s.r;
                sd_plane = -hy;
            }
            if (hit) {
                const float hh = (sd_plane - sd_sphere) / K;
                const float pa = 1.0f / (1.0f + std::exp2(hh)), pb = 1.0f / (1.0f + std::exp2(-hh));
                float gx = pa * nx, gy = pa * ny - pb, gz = pa * nz;
                const float gl = len3r(gx, gy, gz);
                if (gl > 0.0f) {
                    gx /= gl;
                    gy /= gl;
                    gz /= gl;
                }
                const float vx = -dx, vy = -dy, vz = -dz;
                const float nl_ = std::fmax(gx * C.lx + gy * C.ly + gz * C.lz, 0.0f);
                const float nv = std::fmax(gx * vx + gy * vy + gz * vz, 1e-4f);
                float ax = vx + C.lx, ay = vy + C.ly, az = vz + C.lz;
                const float al = len3r(ax, ay, az);
                float spec = 0.0f;
                if (al > 0.0f && nl_ > 0.0f) {
                    ax /= al;
                    ay /= al;
                    az /= al;
                    const float nh = std::fmax(gx * ax + gy * ay + gz * az, 0.0f),
                                vh = std::fmax(vx * ax + vy * ay + vz * az, 0.0f);
                    const float a2 = kAlpha * kAlpha, dd = nh * nh * (a2 - 1.0f) + 1.0f;
                    const float D = a2 / (kPi * dd * dd);
                    const float vis =
                        0.5f / (nl_ * std::sqrt(nv * nv * (1.0f - a2) + a2) + nv * std::sqrt(nl_ * nl_ * (1.0f - a2) + a2));
                    const float m = 1.0f - vh, m2 = m * m;
                    const float F = kF0 + (1.0f - kF0) * (m2 * m2 * m);
                    spec = D * vis * F * nl_;
                }
                const float lit = kAmbient + nl_;
                rgba[p] = rrgba8(1.0f * lit + spec, (191.0f / 255.0f) * lit + spec, spec);
                if (depth) depth[p] = t + walked;
                continue;
            }
        }
        float tn = 0.0f, tf = 3.0e38f;
        int axis = -1;
        const float lo[3] = {-C.hs, 0.0f, -C.hs}, hi[3] = {C.hs, C.top, C.hs}, e[3] = {C.ex, C.ey, C.ez},
                    d[3] = {dx, dy, dz};
        for (int k = 0; k < 3; ++k) {
            if (d[k] != 0.0f) {
                float t0 = (lo[k] - e[k]) / d[k], t1 = (hi[k] - e[k]) / d[k];
                if (t0 > t1) std::swap(t0, t1);
                tn = std::fmax(tn, t0);
                if (t1 < tf) {
                    tf = t1;
                    axis = k;
                }
            } else if (e[k] < lo[k] || e[k] > hi[k]) {
                tn = 3.0e38f;
            }
        }
        if (axis >= 0 && tf > tn) {
            const float bx = axis == 0 ? (dx > 0.0f ? -1.0f : 1.0f) : 0.0f;
            const float by = axis == 1 ? (dy > 0.0f ? -1.0f : 1.0f) : 0.0f;
            const float bz = axis == 2 ? (dz > 0.0f ? -1.0f : 1.0f) : 0.0f;
            const float lit = kAmbient + std::fmax(bx * C.lx + by * C.ly + bz * C.lz, 0.0f);
            rgba[p] = rrgba8(0.8f * lit, 0.7f * lit, 0.6f * lit);
            if (depth) depth[p] = tf;
            continue;
        }
        rgba[p] = 0xFF000000u | 248u | (151u << 8) | (184u << 16);
        if (depth) depth[p] = 0.0f;
    }
}
