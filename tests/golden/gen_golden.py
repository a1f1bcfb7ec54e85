"""Generate the golden fixtures under tests/golden/ (run: python tests/golden/gen_golden.py).

Two kinds of fixtures:

1. hashing_kat.npz — the reference's own known-answer test for sort + cell ranges
   (src/physics/spatial_hashing.rs:536-632): keys k_v = v mod 256 for v in [0, n),
   vals 0..n-1, sorted, then ZEROING + HASHING; expected
   start[c] = sum_{c' < c} cnt(c'), close[c] = start[c] + cnt(c) - 1 with
   cnt(c) = n // 256 + (n % 256 > c), for c < min(n, 256), n in {1, 100, 256, 16777216}.
   The expectations are the test's closed form, evaluated here.

2. physics_*.npz — small dense scenes stepped by a second, independent restatement
   of src/physics/physics.wgsl written in plain Python on numpy float32 scalars
   (every operation rounds to binary32; f16 via numpy's RNE conversion), with the
   reference's frame routing (src/physics/mod.rs:846-956): stable sort of the keys,
   ZEROING + HASHING (spatial_hashing.wgsl:29-70), INIT on frame 0, LOOP afterwards.
   It is deliberately a different code path from oracle/oracle.cpp (start/close
   tables, WGSL-level expressions) so that the C++ oracle is checked against it.

Pure-Python loops: only for scenes of a few hundred spheres.
"""

from __future__ import annotations

import math
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
F = np.float32
INVALID = 0xFFFFFFFF


# ------------------------------------------------------------------ hashing KAT
def hashing_kat():
    out = {}
    for n in (1, 100, 256, 16_777_216):
        m = min(n, 256)
        cnt = np.array([n // 256 + (1 if n % 256 > c else 0) for c in range(m)], np.int64)
        start = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.uint32)
        close = (start.astype(np.int64) + cnt - 1).astype(np.uint32)
        out[f"start_{n}"] = start
        out[f"close_{n}"] = close
    np.savez_compressed(HERE / "hashing_kat.npz", **out)


# ------------------------------------------------------------------ WGSL pieces
def q_u32(x: float) -> int:  # (x * 1000.) as u32
    v = F(x) * F(1000.0)
    if not (v > 0):
        return 0
    return min(int(v), 0xFFFFFFFF)


def q_i32(x: float) -> int:  # (x * 1000.) as i32
    v = F(x) * F(1000.0)
    if math.isnan(v):
        return 0
    return max(-(2**31), min(2**31 - 1, int(v)))


def consts(cfg: dict) -> dict:
    N, g = cfg["N"], cfg["grid_size"]
    return {
        "N": N,
        "G": g,
        "HMH": F(cfg["half_map_height"]),
        "HMS": F((N * g) // 2),
        "GRAV": [F(F(q_i32(v)) / F(1000.0)) for v in cfg["gravity"]],
        "E_ENVIR": F(F(q_u32(cfg["e_envir"])) / F(1000.0)),
        "E_AGENT": F(F(q_u32(cfg["e_agent"])) / F(1000.0)),
        "K_AGENT": F(F(q_u32(cfg["k_agent"])) / F(1000.0)),
        "C_AGENT": F(F(q_u32(cfg["c_agent"])) / F(1000.0)),
        "R_AGENT": F(F(q_u32(cfg["r_agent"])) / F(1000.0)),
        "T": F(F(q_u32(cfg["time_delta"])) / F(1000.0)),
        "SPRING": bool(cfg["enable_spring"]),
    }


def u32_of(v: np.float32) -> int:  # WGSL u32(f32): truncate, saturate, NaN -> 0
    if not (v > 0):
        return 0
    if v >= F(4294967296.0):
        return 0xFFFFFFFF
    return int(v)


def grid_id(K, x, z):
    cx = u32_of(F(x + K["HMS"])) // K["G"]
    cz = u32_of(F(z + K["HMS"])) // K["G"]
    return min(cx, K["N"] - 1), min(cz, K["N"] - 1)


def vmin(a, b):  # WGSL min
    if math.isnan(a):
        return b
    if math.isnan(b):
        return a
    return b if b < a else a


def vmax(a, b):
    if math.isnan(a):
        return b
    if math.isnan(b):
        return a
    return b if b > a else a


def vclamp(e, lo, hi):
    return vmin(vmax(e, lo), hi)


def vsign(x):
    return F(1.0) if x > 0 else (F(-1.0) if x < 0 else F(0.0))


def add(a, b):
    return [F(a[i] + b[i]) for i in range(3)]


def sub(a, b):
    return [F(a[i] - b[i]) for i in range(3)]


def mul(a, b):
    return [F(a[i] * b[i]) for i in range(3)]


def smul(s, a):
    return [F(s * a[i]) for i in range(3)]


def sdiv(a, s):
    return [F(a[i] / s) for i in range(3)]


def dot(a, b):
    return F(F(F(a[0] * b[0]) + F(a[1] * b[1])) + F(a[2] * b[2]))


def length(a):
    return F(np.sqrt(dot(a, a)))


def normalize(a):
    return sdiv(a, length(a))


def f16(x) -> int:
    return int(np.array([x], np.float32).astype(np.float16).view(np.uint16)[0])


def unf16(b: int) -> np.float32:
    return F(np.array([b], np.uint16).view(np.float16)[0])


def agent_new(pos, vfme, idx):
    p = pos[idx]
    q = [int(x) for x in vfme[idx]]
    return {
        "position": [F(p[0]), F(p[1]), F(p[2])],
        "scale": F(p[3]),
        "velocity": [unf16(q[0] & 0xFFFF), unf16(q[0] >> 16), unf16(q[1] & 0xFFFF)],
        "force": [unf16(q[1] >> 16), unf16(q[2] & 0xFFFF), unf16(q[2] >> 16)],
        "massv": unf16(q[3] & 0xFFFF),
    }


def pack(a):
    v, f = a["velocity"], a["force"]
    return [f16(v[0]) | (f16(v[1]) << 16), f16(v[2]) | (f16(f[0]) << 16), f16(f[1]) | (f16(f[2]) << 16),
            f16(a["massv"]) | (f16(F(0.0)) << 16)]


def hash3f1u(n: int):
    v = (n * (n ^ (n >> 15))) & 0xFFFFFFFF
    d = F(4294967296.0)
    return [F(F((v * m) & 0xFFFFFFFF) / d) for m in (1, 0x1FF, 0x3FFFF)]


def sphere(K, a, b):
    edge = F(b["scale"] + a["scale"])
    tpos = sub(a["position"], b["position"])
    dist = length(tpos)
    if dist <= edge:
        norm = normalize(tpos)
        if not K["SPRING"]:
            m1, m2 = a["massv"], b["massv"]
            rvel = sub(a["velocity"], b["velocity"])
            rspd = dot(rvel, norm)
            if rspd < 0:
                rvel_n = smul(rspd, norm)
                rvel_c = sdiv(smul(F(m1 - F(K["E_AGENT"] * m2)), rvel_n), F(m1 + m2))
                a["velocity"] = add(add(b["velocity"], sub(rvel, rvel_n)), rvel_c)
            a["position"] = add(a["position"], smul(F(F(0.5) * F(edge - dist)), norm))
        else:
            makeup = F(edge - dist)
            kforce = smul(F(K["K_AGENT"] * makeup), norm)
            cforce = smul(F(F(-K["C_AGENT"]) / K["T"]), a["velocity"])
            a["force"] = add(a["force"], add(kforce, cforce))
            limit = F(makeup - F(K["R_AGENT"] * a["scale"]))
            if limit > 0:
                a["position"] = add(a["position"], smul(limit, norm))


def cube(K, a):
    edge = sub([K["HMS"], K["HMH"], K["HMS"]], [a["scale"]] * 3)
    cetr = [F(0.0), K["HMH"], F(0.0)]
    tpos = sub(a["position"], cetr)
    makeup = [F(edge[i] - F(abs(tpos[i]))) for i in range(3)]
    itouch = [m < 0 for m in makeup]
    if not any(itouch):
        return
    if not K["SPRING"]:
        a["position"] = add([vclamp(tpos[i], F(-edge[i]), edge[i]) for i in range(3)], cetr)
        a["velocity"] = mul(a["velocity"], [F(-K["E_ENVIR"]) if t else F(1.0) for t in itouch])
    else:
        mm = F(-F(a["scale"] * K["R_AGENT"]))
        kforce = mul(smul(K["K_AGENT"], [vsign(t) for t in tpos]), [vclamp(m, mm, F(0.0)) for m in makeup])
        cforce = smul(F(F(-K["C_AGENT"]) / K["T"]), a["velocity"])
        a["force"] = add(a["force"], add(kforce, cforce))
        it2 = [m < mm for m in makeup]
        if any(it2):
            e2 = sub(edge, [mm] * 3)
            a["position"] = add([vclamp(tpos[i], F(-e2[i]), e2[i]) for i in range(3)], cetr)
            dv = smul(F(F(-F(F(1.0) + K["E_ENVIR"])) / K["T"]), [a["velocity"][i] if it2[i] else F(0.0) for i in range(3)])
            acc = sdiv(dv, K["T"])
            a["force"] = add(a["force"], smul(a["massv"], acc))


def collide_row(K, a, cid, base, start, close, perm, pos, vfme):
    s, e = INVALID, 0
    if cid[0] > 0 and start[base - 1] != INVALID:
        s, e = start[base - 1], close[base - 1]
    if start[base] != INVALID:
        if s == INVALID:
            s = start[base]
        e = close[base]
    if cid[0] < K["N"] - 1 and start[base + 1] != INVALID:
        if s == INVALID:
            s = start[base + 1]
        e = close[base + 1]
    if s == INVALID:
        return
    for j in range(s, e + 1):
        sphere(K, a, agent_new(pos, vfme, perm[j]))


def physics(K, init, perm, start, close, pos, vfme):
    n = len(perm)
    pos_o = np.zeros_like(pos)
    vfme_o = np.zeros_like(vfme)
    keys_o = np.zeros(n, np.uint32)
    N = K["N"]
    for i in range(n):
        a = agent_new(pos, vfme, int(perm[i]))
        cid = grid_id(K, a["position"][0], a["position"][2])
        idx = cid[1] * N + cid[0]
        if not init:
            acc = sdiv(a["force"], a["massv"])
            a["velocity"] = add(a["velocity"], smul(K["T"], smul(K["T"], add(K["GRAV"], acc))))
            a["position"] = add(a["position"], a["velocity"])
            a["force"] = [F(0.0)] * 3
            old = list(a["position"])
            s, e = int(start[idx]), int(close[idx])
            if cid[0] > 0 and start[idx - 1] != INVALID:
                s = int(start[idx - 1])
            if cid[0] < N - 1 and start[idx + 1] != INVALID:
                e = int(close[idx + 1])
            for j in range(s, e + 1):
                if j == i:
                    continue
                sphere(K, a, agent_new(pos, vfme, int(perm[j])))
            if cid[1] > 0:
                collide_row(K, a, cid, idx - N, start, close, perm, pos, vfme)
            if cid[1] < N - 1:
                collide_row(K, a, cid, idx + N, start, close, perm, pos, vfme)
            if length(sub(a["position"], old)) > a["scale"]:
                jitter = [F(F(h * F(2.0)) - F(1.0)) for h in hash3f1u(i)]
                a["position"] = add(a["position"], normalize(jitter))
            cube(K, a)
            lim = F(65504.0)
            a["velocity"] = [vclamp(v, F(-lim), lim) for v in a["velocity"]]
            a["force"] = [vclamp(v, F(-lim), lim) for v in a["force"]]
        pos_o[i] = [*a["position"], a["scale"]]
        vfme_o[i] = pack(a)
        if init:
            keys_o[i] = idx
        else:
            c2 = grid_id(K, a["position"][0], a["position"][2])
            keys_o[i] = c2[1] * N + c2[0]
    return pos_o, vfme_o, keys_o


def run_frames(cfg, pos, vfme, frames):
    """Reference frame routing: keys start as zeros; frame 0 is INIT."""
    K = consts(cfg)
    C = K["N"] * K["N"]
    n = pos.shape[0]
    keys = np.zeros(n, np.uint32)
    snaps = []
    for f in range(frames):
        perm = np.argsort(keys, kind="stable").astype(np.uint32)
        sk = keys[perm]
        start = np.full(C, INVALID, np.uint32)
        close = np.full(C, INVALID, np.uint32)
        for t in range(n):
            k = int(sk[t])
            if t == 0 or sk[t - 1] != k:
                start[k] = t
            if t == n - 1 or sk[t + 1] != k:
                close[k] = t
        pos, vfme, keys = physics(K, f == 0, perm, start, close, pos, vfme)
        snaps.append({"pos": pos.copy(), "vfme": vfme.copy(), "keys": keys.copy(), "perm": perm,
                      "start": start, "close": close})
    return snaps


def scene(n, N, seed, spring, H=2, radius=0.5, grid_size=1):
    """Dense little scene: ~n/(N*N) spheres per cell, many contacts and wall hits."""
    rng = np.random.default_rng(seed)
    hs = (N * grid_size) // 2
    x = rng.uniform(-hs, hs, n).astype(np.float32)
    z = rng.uniform(-hs, hs, n).astype(np.float32)
    y = rng.uniform(0, 2 * H, n).astype(np.float32)
    top = np.nextafter(np.float32(hs), np.float32(-np.inf))
    x, z = np.minimum(x, top), np.minimum(z, top)
    r = rng.uniform(radius * 0.6, radius * 1.2, n).astype(np.float32)
    cfg = {"N": N, "grid_size": grid_size, "half_map_height": H, "gravity": (0.0, -9.81, 0.0),
           "e_envir": 0.8, "e_agent": 0.8, "k_agent": 1000.0 if spring else 25.0,
           "c_agent": 5.0 if spring else 0.1, "r_agent": 0.9, "time_delta": 1.0 / 60.0,
           "enable_spring": spring}
    dt = F(F(q_u32(cfg["time_delta"])) / F(1000.0))
    v = (rng.standard_normal((n, 3)).astype(np.float32) * F(3.0) * dt).astype(np.float32)
    h = np.zeros((n, 8), np.float16)
    h[:, 0:3] = v.astype(np.float16)
    h[:, 6] = rng.uniform(0.5, 2.0, n).astype(np.float16)
    vfme = h.view(np.uint32).reshape(n, 4).copy()
    pos = np.stack([x, y, z, r], 1).astype(np.float32)
    return cfg, pos, vfme


def physics_fixtures():
    cases = {
        "rigid": dict(n=192, N=8, seed=1, spring=False),
        "spring": dict(n=160, N=8, seed=2, spring=True),
        "rigid_sparse": dict(n=64, N=16, seed=3, spring=False, H=4),
    }
    frames = 6
    for name, kw in cases.items():
        cfg, pos, vfme = scene(**kw)
        snaps = run_frames(cfg, pos.copy(), vfme.copy(), frames)
        out = {"pos0": pos, "vfme0": vfme, "frames": np.int64(frames)}
        for k, v in cfg.items():
            out["cfg_" + k] = np.asarray(v)
        for f, s in enumerate(snaps):
            for k, v in s.items():
                out[f"f{f}_{k}"] = v
        np.savez_compressed(HERE / f"physics_{name}.npz", **out)


if __name__ == "__main__":
    hashing_kat()
    physics_fixtures()
    print("fixtures written to", HERE)
