"""mb_sort_and_hash_static: the sort + cell-range stage for callers that may not
allocate device memory where they issue work (a frame loop that forbids
allocation after start-up, or code recording into a CUDA stream capture).

Its scratch is a fixed array inside the library, shared by all calls on a
device, so the test runs two different calls back to back through the C ABI
and checks each against mb_sort_and_hash (which works from a cudaMalloc'd
plan).  The results are integers: they must be identical.  This file is
collected last on purpose (tests/test_zz_*), and also passes run on its own.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(torch, lib, fn, keys, cells, vals, plan=None):
    n = keys.size
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dv = None if vals is None else torch.from_numpy(vals.view(np.int32)).cuda()
    sk = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    sv = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    st = torch.full((cells,), -1, dtype=torch.int32, device="cuda")
    cl = torch.full((cells,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    args = [dk.data_ptr(), None if dv is None else dv.data_ptr(), n, cells, sk.data_ptr(), sv.data_ptr(),
            st.data_ptr(), cl.data_ptr(), stream]
    status = fn(*args) if plan is None else fn(plan, *args)
    assert status == 0, lib.mb_last_error(None)
    torch.cuda.synchronize()
    u = lambda t: t.cpu().numpy().view(np.uint32)
    return u(sk)[:n], u(sv)[:n], u(st), u(cl)


def test_static_scratch_matches_planned_entry_point(built_lib, cuda):
    torch, lib = cuda, built_lib
    plan = C.c_void_p()
    assert lib.mb_sort_plan_create(1 << 18, 1 << 18, C.byref(plan)) == 0
    rng = np.random.default_rng(2024)
    cases = [
        # two calls in a row with different sizes / digit schedules
        (rng.integers(0, 250_000, 200_000, dtype=np.uint64).astype(np.uint32), 250_000, None),
        (rng.integers(0, 4096, 262_144, dtype=np.uint64).astype(np.uint32), 4096,
         rng.integers(0, 2**32, 262_144, dtype=np.uint64).astype(np.uint32)),
        (np.sort(rng.integers(0, 70_000, 100_000)).astype(np.uint32), 70_000, None),
    ]
    try:
        for keys, cells, vals in cases:
            got = _run(torch, lib, lib.mb_sort_and_hash_static, keys, cells, vals)
            ref = _run(torch, lib, lib.mb_sort_and_hash, keys, cells, vals, plan=plan)
            for g, r, what in zip(got, ref, ["sorted keys", "sorted values", "start", "close"]):
                np.testing.assert_array_equal(g, r, err_msg=what)
            order = np.argsort(keys, kind="stable")
            np.testing.assert_array_equal(got[0], keys[order])
    finally:
        lib.mb_sort_plan_destroy(plan)


def test_static_scratch_digit_split_changes(built_lib, cuda):
    """The same key count under cell counts with different digit schedules
    (2^18 cells: 5 + 5 + 8 bits; 2^17: 5 + 4 + 8), alternating: every call clears
    the look-back words it uses, so none of an older call is misread."""
    torch, lib = cuda, built_lib
    plan = C.c_void_p()
    assert lib.mb_sort_plan_create(1 << 18, 1 << 18, C.byref(plan)) == 0
    rng = np.random.default_rng(77)
    try:
        for cells in [1 << 18, 1 << 17, 1 << 17, 1 << 18, 1 << 17, 1 << 18]:
            keys = rng.integers(0, cells, 200_000, dtype=np.uint64).astype(np.uint32)
            got = _run(torch, lib, lib.mb_sort_and_hash_static, keys, cells, None)
            ref = _run(torch, lib, lib.mb_sort_and_hash, keys, cells, None, plan=plan)
            for g, r, what in zip(got, ref, ["sorted keys", "sorted values", "start", "close"]):
                np.testing.assert_array_equal(g, r, err_msg=f"{what}, cells {cells}")
            np.testing.assert_array_equal(got[1], np.argsort(keys, kind="stable").astype(np.uint32))
        assert lib.mb_sort_static_status(torch.cuda.current_stream().cuda_stream) == 0
    finally:
        lib.mb_sort_plan_destroy(plan)


def test_static_scratch_rejects_sizes_beyond_its_limit(built_lib, cuda):
    lib = built_lib
    assert lib.mb_sort_and_hash_static(None, None, 262_145, 16, None, None, None, None, None) == 1
    assert b"MB_STATIC_MAX_KEYS" in lib.mb_last_error(None)
    assert lib.mb_sort_and_hash_static(None, None, 0, 262_145, None, None, None, None, None) == 1
    assert b"MB_STATIC_MAX_CELLS" in lib.mb_last_error(None)
