"""Contact and energy statistics of a scene state (host-side analysis).

Long runs of the contact dynamics are chaotic: the reference resolves each
sphere's contacts one after another (src/physics/physics.wgsl:119-169) and
nudges spheres that moved further than their radius in a hashed direction
(physics.wgsl:162-168), so a one-ulp difference anywhere grows until the two
runs differ sphere by sphere.  Runs that are not bit-identical are compared
through statistics of the state instead:

* penetration depth ``max(0, r1 + r2 - |p1 - p2|)`` over every pair of spheres
  closer than ``r1 + r2`` (count, mean, 99th percentile, maximum);
* kinetic energy ``sum(0.5 * m * |v|^2)`` with ``v`` the stored displacement per
  step divided by the step length (m/s).

:data:`BOUNDS` states how far two such runs may drift apart and still count as
the same physics; :func:`compare` applies them.  The bounds were set from two
oracle runs of the 65,536-sphere workload whose start differs in one ulp of one
coordinate: by frame 1,000 about 9,000 spheres differ, while the kinetic energy
agrees within 1.1 %, the mean and 99th-percentile depth within 2 %, the contact
count within 0.2 % and the maximum depth exactly.
"""

from __future__ import annotations

import numpy as np

from . import unpack_vfme

# relative differences allowed between two runs of the same scene that diverged
BOUNDS = {
    "contacts": 0.05,     # number of overlapping pairs
    "mean_depth": 0.10,
    "p99_depth": 0.10,
    "max_depth": 0.50,    # an extreme value: one pair decides it
    "kinetic_energy": 0.05,
}
# absolute floor under each relative bound (depths in length units, energy in mass (m/s)^2)
FLOORS = {"contacts": 8.0, "mean_depth": 1e-4, "p99_depth": 1e-4, "max_depth": 1e-3, "kinetic_energy": 1e-3}


def contact_stats(pos_scale: np.ndarray, vfme: np.ndarray, dt: float) -> dict:
    """Penetration-depth and kinetic-energy statistics of one state.

    pos_scale: (n, 4) float32 (x, y, z, radius); vfme: (n, 4) uint32 packed
    velocity-as-displacement / force / mass; dt: the step length the kernels use
    (the quantised one)."""
    try:
        from scipy.spatial import cKDTree
    except ImportError as e:  # pragma: no cover - scipy is part of the supported environment
        raise ImportError("contact_stats needs scipy (scipy.spatial.cKDTree)") from e
    p = np.ascontiguousarray(pos_scale, np.float32).reshape(-1, 4)
    pts = p[:, :3].astype(np.float64)
    r = p[:, 3].astype(np.float64)
    if p.shape[0] > 1:
        pairs = cKDTree(pts).query_pairs(2.0 * float(r.max()), output_type="ndarray")
    else:
        pairs = np.zeros((0, 2), np.int64)
    d = np.linalg.norm(pts[pairs[:, 0]] - pts[pairs[:, 1]], axis=1)
    depth = r[pairs[:, 0]] + r[pairs[:, 1]] - d
    pen = depth[depth > 0.0]
    v, _, m = unpack_vfme(vfme)
    speed2 = np.sum((v.astype(np.float64) / float(dt)) ** 2, axis=1)
    return {
        "contacts": int(pen.size),
        "mean_depth": float(pen.mean()) if pen.size else 0.0,
        "p99_depth": float(np.percentile(pen, 99)) if pen.size else 0.0,
        "max_depth": float(pen.max()) if pen.size else 0.0,
        "kinetic_energy": float(0.5 * np.sum(m.astype(np.float64) * speed2)),
    }


def compare(a: dict, b: dict) -> dict:
    """For each statistic: (|a - b|, allowed, ok) under BOUNDS and FLOORS."""
    out = {}
    for k, rel in BOUNDS.items():
        diff = abs(float(a[k]) - float(b[k]))
        allowed = max(rel * max(abs(float(a[k])), abs(float(b[k]))), FLOORS[k])
        out[k] = (diff, allowed, diff <= allowed)
    return out


def within_bounds(a: dict, b: dict) -> bool:
    return all(ok for _, _, ok in compare(a, b).values())


def candidate_tests(start: np.ndarray, close: np.ndarray, grids: int) -> int:
    """Candidate pairs one physics pass tests, from a frame's cell ranges.

    The reference tests every sphere against every other sphere in the 3 x 3
    cells around its own (physics.wgsl:122-160, the three row ranges of
    handle_collisions).  With m[c] spheres in cell c and M[c] the sum of m over
    c's 3 x 3 neighbourhood, a frame tests sum(m[c] * (M[c] - 1)) pairs.  start
    and close are the frame's tables (0xFFFFFFFF for empty cells, close
    inclusive)."""
    st = np.asarray(start, np.int64).reshape(grids, grids)
    cl = np.asarray(close, np.int64).reshape(grids, grids)
    m = np.where(st == 0xFFFFFFFF, 0, cl - st + 1)
    pad = np.pad(m, 1)
    nb = sum(pad[1 + dz:1 + dz + grids, 1 + dx:1 + dx + grids] for dz in (-1, 0, 1) for dx in (-1, 0, 1))
    return int(np.sum(m * (nb - 1)))
