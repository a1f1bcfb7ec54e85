"""Seeded synthetic scenes for the benchmark workloads (numpy PCG64).

The reference's own start-up scene (src/physics/mod.rs:172-212) is rebuilt by
``reference_default`` with the reference's random stream (ChaCha8 seeded from
0, rand 0.8's f32 ``gen_range``; see ``chacha``).  The benchmark workloads are
seeded numpy PCG64 scenes:

* ``plain_uniform``  — uniform positions, N(0, 1) m/s velocities (65,536 / 1,048,576 spheres)
* ``plain_clustered`` — 16 Gaussian clusters, spring response (4,194,304 spheres)
* ``batch``          — many independent scenes of log-uniform size

Frame of reference: the reference's box is x, z in [-H_s, H_s) and y in [0, 2H]
(physics.wgsl:268-275).  A workload stated as "y in [-8, 8]" is shifted by +H
into that box.  Velocity is stored as displacement per step: f16(v0 * dt_q), with
dt_q the quantised step the shader uses.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import PhysicsPlugin, pack_vfme


def quantized_dt(dt: float) -> float:
    """f32(trunc(f32(dt) * 1000)) / 1000 in f32 (src/physics/mod.rs:481)."""
    v = np.float32(dt) * np.float32(1000.0)
    return float(np.float32(np.float32(int(v)) / np.float32(1000.0)))


@dataclass
class Scene:
    plugin: PhysicsPlugin
    pos_scale: np.ndarray  # (n, 4) float32
    vfme: np.ndarray       # (n, 4) uint32
    name: str = ""

    @property
    def n(self) -> int:
        return self.pos_scale.shape[0]


def _below(x: np.ndarray, hi: float) -> np.ndarray:
    """Clamp float32 values that rounded up to `hi` back to the largest float below it."""
    top = np.nextafter(np.float32(hi), np.float32(-np.inf))
    return np.minimum(x, top).astype(np.float32)


def _state(pos_xyz: np.ndarray, radius: float, vel: np.ndarray, plugin: PhysicsPlugin):
    n = pos_xyz.shape[0]
    pos = np.empty((n, 4), np.float32)
    pos[:, :3] = pos_xyz
    pos[:, 3] = np.float32(radius)
    dt = np.float32(quantized_dt(plugin.time_delta))
    disp = (vel.astype(np.float32) * dt).astype(np.float32)
    vfme = pack_vfme(disp, np.zeros_like(disp), 1.0)
    return pos, vfme


def plain_uniform(n: int, grids: int, *, grid_size: int = 1, half_map_height: int = 8, radius: float = 0.5,
                  seed: int = 0, spring: bool = False, e: float = 0.8, k: float = 25.0, c: float = 0.1,
                  dt: float = 1.0 / 60.0, gravity=(0.0, -9.81, 0.0)) -> Scene:
    """Uniform positions in the box, N(0, 1 m/s) per-axis velocities, unit mass."""
    plugin = PhysicsPlugin(
        max_number_of_agents=n, number_of_grids_one_dimension=grids, grid_size=grid_size,
        half_map_height=half_map_height, gravity=tuple(gravity), e_envir=e, e_agent=e,
        k_agent=k, c_agent=c, enable_spring=spring, time_delta=dt,
    )
    rng = np.random.default_rng(seed)
    hs = (grids * grid_size) // 2
    x = _below(rng.uniform(-hs, hs, n).astype(np.float32), hs)
    z = _below(rng.uniform(-hs, hs, n).astype(np.float32), hs)
    y = _below(rng.uniform(0.0, 2 * half_map_height, n).astype(np.float32), 2 * half_map_height)
    v0 = rng.standard_normal((n, 3)).astype(np.float32)
    pos, vfme = _state(np.stack([x, y, z], 1), radius, v0, plugin)
    return Scene(plugin, pos, vfme, f"uniform n={n} N={grids}")


def plain_clustered(n: int, grids: int, *, clusters: int = 16, sigma_xz: float = 32.0, sigma_y: float = 2.0,
                    grid_size: int = 1, half_map_height: int = 8, radius: float = 0.5, seed: int = 0,
                    k: float = 1000.0, c: float = 5.0, e: float = 0.8, dt: float = 1.0 / 60.0,
                    gravity=(0.0, -9.81, 0.0)) -> Scene:
    """Gaussian clusters (sigma in cells), centres uniform in the box, truncated to
    the box, spring response."""
    plugin = PhysicsPlugin(
        max_number_of_agents=n, number_of_grids_one_dimension=grids, grid_size=grid_size,
        half_map_height=half_map_height, gravity=tuple(gravity), e_envir=e, e_agent=e,
        k_agent=k, c_agent=c, enable_spring=True, time_delta=dt,
    )
    rng = np.random.default_rng(seed)
    hs = (grids * grid_size) // 2
    h2 = 2 * half_map_height
    cx = rng.uniform(-hs, hs, clusters)
    cz = rng.uniform(-hs, hs, clusters)
    cy = rng.uniform(0.0, h2, clusters)
    which = rng.integers(0, clusters, n)
    # Gaussian clusters truncated to the domain: samples that fall outside are
    # drawn again (clipping them would pile them onto the border cells)
    x = np.empty(n)
    y = np.empty(n)
    z = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        w = which[todo]
        x[todo] = cx[w] + rng.standard_normal(todo.size) * sigma_xz * grid_size
        z[todo] = cz[w] + rng.standard_normal(todo.size) * sigma_xz * grid_size
        y[todo] = cy[w] + rng.standard_normal(todo.size) * sigma_y * grid_size
        out = (x[todo] < -hs) | (x[todo] >= hs) | (z[todo] < -hs) | (z[todo] >= hs) | (y[todo] < 0.0) | (y[todo] > h2)
        todo = todo[out]
    x = _below(x.astype(np.float32), hs)
    z = _below(z.astype(np.float32), hs)
    y = _below(y.astype(np.float32), h2)
    v0 = rng.standard_normal((n, 3)).astype(np.float32)
    pos, vfme = _state(np.stack([x, y, z], 1), radius, v0, plugin)
    return Scene(plugin, pos, vfme, f"clustered n={n} N={grids} k={clusters}")


def reference_default(plugin: PhysicsPlugin | None = None, seed: int = 0) -> Scene:
    """The reference plugin's own start-up scene (src/physics/mod.rs:172-212) for
    its default settings (16,384 spheres, N = 128, grid_size 8): a lattice of
    2^(L//2) x 2^(L - L//2) spheres (L = log2 n), x-major, 4 units apart, centred
    on the origin, at height 4, radius 1, mass 1, horizontal velocities (stored
    as displacement per step, as the reference packs them) from
    ``ChaCha8Rng::seed_from_u64(seed)`` through rand 0.8's ``gen_range(-0.8..0.8)``
    (x then z per sphere, mod.rs:198-205), vertical 0.  The stream restates the
    crates' published algorithms (``chacha``); it is unpinned against a run of the
    reference itself, which needs a Rust toolchain."""
    plugin = plugin or PhysicsPlugin()
    n = int(plugin.max_number_of_agents)
    if n <= 0 or n & (n - 1):
        raise ValueError("the reference lattice needs a power-of-two sphere count")
    L = n.bit_length() - 1
    cx, cz = 1 << (L // 2), 1 << (L - L // 2)
    xs = (np.arange(cx, dtype=np.float32) - np.float32(0.5) * np.float32(cx - 1)) * np.float32(4.0)
    zs = (np.arange(cz, dtype=np.float32) - np.float32(0.5) * np.float32(cz - 1)) * np.float32(4.0)
    pos = np.empty((n, 4), np.float32)
    pos[:, 0] = np.repeat(xs, cz)
    pos[:, 1] = 4.0
    pos[:, 2] = np.tile(zs, cx)
    pos[:, 3] = 1.0
    from .chacha import reference_start_velocities

    v = reference_start_velocities(n, seed)
    vfme = pack_vfme(v, np.zeros_like(v), 1.0)
    return Scene(plugin, pos, vfme, f"reference default lattice n={n}")


def next_pow2(x: int) -> int:
    return 1 << max(0, (int(x) - 1).bit_length())


def batch(count: int = 512, *, n_min: int = 1024, n_max: int = 262144, seed: int = 0,
          radius: float = 0.5, dt: float = 1.0 / 60.0) -> list[Scene]:
    """Independent scenes: n log-uniform in [n_min, n_max], N = next_pow2(ceil(sqrt(n))),
    H in {4, 8, 16}, e_agent / e_envir uniform in [0.5, 0.95], half of them spring."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        grids = next_pow2(math.isqrt(n - 1) + 1)
        h = int(rng.choice([4, 8, 16]))
        e_a, e_e = float(rng.uniform(0.5, 0.95)), float(rng.uniform(0.5, 0.95))
        spring = bool(rng.integers(0, 2))
        sc = plain_uniform(n, grids, half_map_height=h, radius=radius, seed=int(rng.integers(0, 2**31)),
                           spring=spring, e=e_a, dt=dt)
        sc.plugin = sc.plugin.replace(e_envir=e_e, e_agent=e_a)
        sc.name = f"batch[{s}] n={n} N={grids}"
        out.append(sc)
    return out


WORKLOADS = {
    # name: (generator, kwargs, steps)
    "P-small": (plain_uniform, {"n": 65536, "grids": 256}, 100),
    "P-1M": (plain_uniform, {"n": 1048576, "grids": 1024}, 1000),
    "P-4M": (plain_clustered, {"n": 4194304, "grids": 2048}, 500),
}


def workload(name: str, seed: int = 0) -> Scene:
    gen, kw, _ = WORKLOADS[name]
    return gen(seed=seed, **kw)
