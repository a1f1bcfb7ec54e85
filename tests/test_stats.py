"""Contact / kinetic-energy statistics (bevy_millions_ball_gb300.stats) and the
bounds that compare two runs whose contact dynamics diverged.

The bounds (stats.BOUNDS, relative, with absolute floors stats.FLOORS): contact
count 5 %, mean and 99th-percentile penetration depth 10 %, maximum depth 50 %,
kinetic energy 5 %.  The chaos test shows why statistics are needed at all: a
one-ulp change of one coordinate makes thousands of spheres differ within a few
hundred frames, while the statistics stay inside those bounds."""

import numpy as np
import pytest

pytest.importorskip("scipy")

import oracle
from bevy_millions_ball_gb300 import pack_vfme, scenes, stats


def test_stats_of_a_known_pair():
    pos = np.array([[0.0, 1.0, 0.0, 0.5], [0.9, 1.0, 0.0, 0.5], [5.0, 1.0, 5.0, 0.5]], np.float32)
    v = np.array([[0.016, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, -0.032, 0.0]], np.float32)
    q = pack_vfme(v, np.zeros_like(v), np.array([1.0, 1.0, 2.0], np.float32))
    s = stats.contact_stats(pos, q, 0.016)
    assert s["contacts"] == 1
    assert s["max_depth"] == pytest.approx(0.1, abs=1e-6)
    assert s["mean_depth"] == pytest.approx(0.1, abs=1e-6)
    vv = np.float16(0.016).astype(np.float64) / 0.016
    vy = np.float16(-0.032).astype(np.float64) / 0.016
    assert s["kinetic_energy"] == pytest.approx(0.5 * vv * vv + 0.5 * 2.0 * vy * vy, rel=1e-12)
    assert stats.within_bounds(s, s)
    worse = dict(s, kinetic_energy=s["kinetic_energy"] * 1.2)
    assert not stats.within_bounds(s, worse)


def test_diverged_runs_keep_their_statistics():
    """Two oracle runs of the 65,536-sphere workload, one with a single x
    coordinate moved by one ulp: after 300 frames many spheres differ, the
    statistics agree within the stated bounds."""
    sc = scenes.workload("P-small")
    dt = scenes.quantized_dt(sc.plugin.time_delta)
    pert = sc.pos_scale.copy()
    pert[12345, 0] = np.nextafter(pert[12345, 0], np.float32(np.inf))
    runs = []
    for start in (sc.pos_scale, pert):
        ow = oracle.OracleWorld(sc.plugin.to_c())
        ow.set_state(start, sc.vfme)
        ow.step(300)
        runs.append(ow.get_state())
        ow.close()
    (p0, q0), (p1, q1) = runs
    differ = int(np.sum(np.any(p0.view(np.uint32) != p1.view(np.uint32), axis=1)))
    assert differ > 100, "the perturbation should have spread (chaotic contacts)"
    a, b = stats.contact_stats(p0, q0, dt), stats.contact_stats(p1, q1, dt)
    assert a["contacts"] > 10_000
    cmp = stats.compare(a, b)
    assert all(ok for _, _, ok in cmp.values()), cmp


def test_candidate_tests_counts_the_reference_neighbourhood():
    """Brute-force count of (sphere, candidate) pairs in the 3 x 3 cells around
    each sphere's cell against the closed form."""
    rng = np.random.default_rng(7)
    N = 9
    cells = rng.integers(0, N * N, 300)
    keys = np.sort(cells)
    start = np.full(N * N, 0xFFFFFFFF, np.uint32)
    close = np.full(N * N, 0xFFFFFFFF, np.uint32)
    for c in np.unique(keys):
        idx = np.flatnonzero(keys == c)
        start[c], close[c] = idx[0], idx[-1]
    want = 0
    for c in keys:
        cz, cx = divmod(int(c), N)
        for d in keys:
            dz, dx = divmod(int(d), N)
            want += abs(dz - cz) <= 1 and abs(dx - cx) <= 1
        want -= 1
    assert stats.candidate_tests(start, close, N) == want
