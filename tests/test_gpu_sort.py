"""GPU parity of the sort + cell-range stage (mb_sort_and_hash) against the oracle
and the reference's known-answer test.  Bit-exact: integer/index work."""

import math

import numpy as np
import pytest

import oracle
from bevy_millions_ball_gb300 import SortPlan
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu
INV = 0xFFFFFFFF


def run_stage(torch, plan, keys: np.ndarray, cells: int, vals: np.ndarray | None = None):
    n = keys.size
    dk = torch.from_numpy(keys.astype(np.int64).astype(np.uint32).view(np.int32)).cuda()
    dv = None if vals is None else torch.from_numpy(vals.view(np.int32)).cuda()
    sk = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    sv = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
    st = torch.empty(cells, dtype=torch.int32, device="cuda")
    cl = torch.empty(cells, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    plan.run(dk.data_ptr(), None if dv is None else dv.data_ptr(), n, cells, sk.data_ptr(), sv.data_ptr(),
             st.data_ptr(), cl.data_ptr(), stream)
    torch.cuda.synchronize()
    u = lambda t: t.cpu().numpy().view(np.uint32)
    return u(sk)[:n], u(sv)[:n], u(st), u(cl)


@pytest.fixture(scope="module")
def plan(built_lib, cuda):
    p = SortPlan(max_keys=1 << 24, max_cells=(1 << 24) + 64)
    yield p
    p.close()


@pytest.mark.parametrize("n", [1, 100, 256, 16_777_216])
def test_hashing_kat_gpu(cuda, plan, n):
    """src/physics/spatial_hashing.rs:536-632 restated: keys v mod 256, vals iota."""
    kat = np.load(GOLDEN / "hashing_kat.npz")
    keys = (np.arange(n, dtype=np.uint64) % 256).astype(np.uint32)
    sk, sv, start, close = run_stage(cuda, plan, keys, 256, np.arange(n, dtype=np.uint32))
    m = min(n, 256)
    np.testing.assert_array_equal(start[:m], kat[f"start_{n}"])
    np.testing.assert_array_equal(close[:m], kat[f"close_{n}"])
    assert np.all(np.diff(sk.astype(np.int64)) >= 0)


CASES = [
    (1, 1), (2, 1), (5, 3), (1000, 7), (4095, 256), (4096, 256), (4097, 257), (100_003, 4096),
    (65_536, 65_536), (1 << 20, 1 << 20), (300_001, 1 << 22), (3_000_001, 1 << 20), (2_000_000, 1000),
    (50_000, (1 << 24) + 5),
]


@pytest.mark.parametrize("n,cells", CASES)
def test_sort_matches_oracle(cuda, plan, n, cells):
    rng = np.random.default_rng(n * 31 + cells)
    keys = rng.integers(0, cells, n, dtype=np.uint64).astype(np.uint32)
    sk, perm, start, close = run_stage(cuda, plan, keys, cells)
    passes = max(1, math.ceil(max(1, (cells - 1).bit_length()) / 8))
    rk, rperm = oracle.radix_sort(keys, None, passes=passes)
    np.testing.assert_array_equal(perm, rperm)
    np.testing.assert_array_equal(sk, rk)
    rs, rc = oracle.spatial_hash(rk, cells)
    np.testing.assert_array_equal(start, rs)
    np.testing.assert_array_equal(close, rc)  # both report 0xFFFFFFFF for empty cells


@pytest.mark.parametrize("pattern", ["equal", "sorted", "descending", "top", "clustered", "nearly_sorted"])
def test_sort_patterns(cuda, plan, pattern):
    n, cells = 1 << 20, 1 << 22
    rng = np.random.default_rng(5)
    if pattern == "equal":
        keys = np.full(n, 12345, np.uint32)
    elif pattern == "sorted":
        keys = np.sort(rng.integers(0, cells, n)).astype(np.uint32)
    elif pattern == "descending":
        keys = np.sort(rng.integers(0, cells, n))[::-1].astype(np.uint32).copy()
    elif pattern == "top":
        keys = np.full(n, cells - 1, np.uint32)
        keys[::7] = 0
    elif pattern == "clustered":
        c = rng.integers(0, cells, 16)
        keys = np.clip(c[rng.integers(0, 16, n)] + rng.integers(-300, 300, n), 0, cells - 1).astype(np.uint32)
    else:
        keys = np.sort(rng.integers(0, cells, n)).astype(np.uint32)
        idx = rng.integers(0, n, n // 50)
        keys[idx] = np.clip(keys[idx].astype(np.int64) + rng.integers(-2048, 2048, idx.size), 0, cells - 1)
    sk, perm, start, close = run_stage(cuda, plan, keys, cells)
    ref = np.argsort(keys, kind="stable").astype(np.uint32)
    np.testing.assert_array_equal(perm, ref)
    np.testing.assert_array_equal(sk, keys[ref])
    rs, rc = oracle.spatial_hash(keys[ref], cells)
    np.testing.assert_array_equal(start, rs)
    np.testing.assert_array_equal(close, rc)


def test_sort_repeated_calls_and_sizes(cuda, plan):
    """Look-back words are reused across calls (epoch tags): alternate sizes and repeat."""
    rng = np.random.default_rng(11)
    for n in [70_000, 10, 1 << 20, 70_000, 70_000, 70_000, 5000, 1 << 20, 1 << 20, 1 << 20, 1 << 20]:
        cells = 1 << 18
        keys = rng.integers(0, cells, n, dtype=np.uint64).astype(np.uint32)
        sk, perm, start, close = run_stage(cuda, plan, keys, cells)
        np.testing.assert_array_equal(perm, np.argsort(keys, kind="stable").astype(np.uint32))


def test_sort_digit_split_changes_at_same_tile_count(cuda, plan):
    """Same key count (same tile count) under cell counts whose digit schedules
    differ (2^18 cells: 5 + 5 + 8 bits; 2^17: 5 + 4 + 8): a changed digit width
    re-lays the look-back table, so words left by an older sort must not be read
    as published ones."""
    rng = np.random.default_rng(12)
    n = 200_000
    for cells in [1 << 18, 1 << 17, 1 << 17, 1 << 18, 1 << 17, 1 << 18, 1 << 18, 1 << 17, 1 << 18]:
        keys = rng.integers(0, cells, n, dtype=np.uint64).astype(np.uint32)
        sk, perm, start, close = run_stage(cuda, plan, keys, cells)
        ref = np.argsort(keys, kind="stable").astype(np.uint32)
        np.testing.assert_array_equal(perm, ref, err_msg=f"cells {cells}")
        np.testing.assert_array_equal(sk, keys[ref])
        rs, rc = oracle.spatial_hash(keys[ref], cells)
        np.testing.assert_array_equal(start, rs)
        np.testing.assert_array_equal(close, rc)
    plan.status(cuda.cuda.current_stream().cuda_stream)  # no wait gave up


def test_lookback_wait_runs_out_and_reports_timeout(cuda, plan, built_lib):
    """A bounded look-back wait that runs out (a lone block whose predecessor tile
    never publishes, 1000 polls) sets the plan's error word, which
    mb_sort_plan_status reports as MB_ERR_TIMEOUT once; the plan keeps working."""
    from bevy_millions_ball_gb300 import MbError

    lib = built_lib
    stream = cuda.cuda.current_stream().cuda_stream
    plan.status(stream)
    assert lib.mb_sort_plan_selftest_stall(plan._h, 1000, stream) == 0, lib.mb_last_error(None)
    with pytest.raises(MbError) as e:
        plan.status(stream)
    assert e.value.status == 4 and "look-back" in str(e.value)
    plan.status(stream)  # read once, then clear
    rng = np.random.default_rng(13)
    for n, cells in [(300_000, 1 << 20), (300_000, 1 << 20), (5000, 77)]:
        keys = rng.integers(0, cells, n, dtype=np.uint64).astype(np.uint32)
        sk, perm, start, close = run_stage(cuda, plan, keys, cells)
        np.testing.assert_array_equal(perm, np.argsort(keys, kind="stable").astype(np.uint32))
    plan.status(stream)


def test_sort_with_values(cuda, plan):
    rng = np.random.default_rng(2)
    n, cells = 123_457, 5000
    keys = rng.integers(0, cells, n, dtype=np.uint64).astype(np.uint32)
    vals = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    sk, sv, _, _ = run_stage(cuda, plan, keys, cells, vals)
    ref = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(sv, vals[ref])


def test_stage_rejects_oversize(cuda, plan):
    from bevy_millions_ball_gb300 import MbError

    with pytest.raises(MbError):
        plan.run(0, None, (1 << 24) + 1, 16, 0, 0, None, None)


def test_empty_input_leaves_every_cell_empty(cuda, plan):
    """n = 0: no keys, so start and close are 0xFFFFFFFF everywhere (also after a
    call that filled them)."""
    rng = np.random.default_rng(3)
    cells = 100_000
    run_stage(cuda, plan, rng.integers(0, cells, 5000, dtype=np.uint64).astype(np.uint32), cells)
    _, _, start, close = run_stage(cuda, plan, np.zeros(0, np.uint32), cells)
    assert np.all(start == INV) and np.all(close == INV)


def test_sparse_keys_long_empty_runs(cuda, plan):
    """Few keys over many cells: long runs of empty cells between them (and before
    the first, after the last) are filled by the gap pass."""
    rng = np.random.default_rng(4)
    cells = 1 << 22
    keys = np.sort(rng.choice(cells, 300, replace=False)).astype(np.uint32)
    keys = np.repeat(keys, rng.integers(1, 4, keys.size))[::-1].copy()
    sk, perm, start, close = run_stage(cuda, plan, keys, cells)
    ref = np.argsort(keys, kind="stable").astype(np.uint32)
    np.testing.assert_array_equal(perm, ref)
    rs, rc = oracle.spatial_hash(keys[ref], cells)
    np.testing.assert_array_equal(start, rs)
    np.testing.assert_array_equal(close, rc)
