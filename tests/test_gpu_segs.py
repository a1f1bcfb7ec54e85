"""GPU parity of the compacted segment table (mb_assemble_segments) against the
reference's known-answer tests (src/physics/assemble_segs.rs:559-776, restated:
keys v mod M, sorted, then one segment per run) and a numpy restatement on random
sorted keys.  Bit-exact: integer/index work."""

import numpy as np
import pytest

from bevy_millions_ball_gb300 import SortPlan

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def plan(built_lib, cuda):
    p = SortPlan(max_keys=1 << 24, max_cells=(1 << 20) + 64)
    yield p
    p.close()


def assemble(torch, plan, sorted_keys: np.ndarray, map_size: int):
    n = sorted_keys.size
    dk = torch.from_numpy(sorted_keys.astype(np.uint32).view(np.int32)).cuda() if n else \
        torch.empty(1, dtype=torch.int32, device="cuda")
    segs = torch.full((max(n, 1),), -1, dtype=torch.int32, device="cuda")
    kmap = torch.full((map_size,), -1, dtype=torch.int32, device="cuda")
    num = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    plan.assemble_segments(dk.data_ptr(), n, segs.data_ptr(), kmap.data_ptr(), num.data_ptr(),
                           torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    u = lambda t: t.cpu().numpy().view(np.uint32)
    return u(segs), u(kmap), int(u(num)[0])


def sort_keys(torch, plan, keys: np.ndarray, cells: int) -> np.ndarray:
    n = keys.size
    dk = torch.from_numpy(keys.astype(np.uint32).view(np.int32)).cuda()
    sk = torch.empty(n, dtype=torch.int32, device="cuda")
    sv = torch.empty(n, dtype=torch.int32, device="cuda")
    plan.run(dk.data_ptr(), None, n, cells, sk.data_ptr(), sv.data_ptr(), None, None,
             torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return sk.cpu().numpy().view(np.uint32)


KAT = [(0, 127), (0, 256), (1, 127), (1, 256), (100, 127), (100, 256), (256, 127), (256, 256), (1000, 127),
       (1000, 256), (16 * 256, 127), (16 * 256, 256), (16_000_000, 127), (16_000_000, 1048576),
       (16_777_216, 127), (16_777_216, 1048576)]


@pytest.mark.parametrize("n,m", KAT)
def test_segments_kat(cuda, plan, n, m):
    torch = cuda
    keys = (np.arange(n, dtype=np.uint64) % m).astype(np.uint32)
    sk = sort_keys(torch, plan, keys, m) if n else keys
    segs, kmap, total = assemble(torch, plan, sk, m)
    assert total == min(n, m)
    counts = np.array([n // m + (n % m > s) for s in range(total)], dtype=np.int64)
    answer = np.concatenate([[0], np.cumsum(counts)[:-1]]) if total else np.zeros(0, np.int64)
    np.testing.assert_array_equal(segs[:total], answer.astype(np.uint32))
    np.testing.assert_array_equal(kmap[:total], np.arange(total, dtype=np.uint32))


@pytest.mark.parametrize("n,span", [(5, 3), (4097, 50), (300_000, 1 << 20), (1_000_000, 2000), (2_000_001, 1 << 20)])
def test_segments_random(cuda, plan, n, span):
    torch = cuda
    rng = np.random.default_rng(n + span)
    sk = np.sort(rng.integers(0, span, n)).astype(np.uint32)
    segs, kmap, total = assemble(torch, plan, sk, span)
    starts = np.flatnonzero(np.concatenate([[True], sk[1:] != sk[:-1]]))
    assert total == starts.size
    np.testing.assert_array_equal(segs[:total], starts.astype(np.uint32))
    present = sk[starts]
    np.testing.assert_array_equal(kmap[present], np.arange(total, dtype=np.uint32))
    absent = np.setdiff1d(np.arange(span), present)
    assert np.all(kmap[absent] == 0xFFFFFFFF)  # left as they were


def test_segments_reject_oversize(cuda, plan):
    from bevy_millions_ball_gb300 import MbError
    with pytest.raises(MbError):
        plan.assemble_segments(0, (1 << 24) + 1, 0, 0, 0)
