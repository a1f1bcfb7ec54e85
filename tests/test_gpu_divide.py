"""The physics pass divides by power-of-two divisors (unit masses) with an exact
reciprocal multiply and by anything else with IEEE division; its results must be
the IEEE round-to-nearest quotients bit for bit (the oracle divides with IEEE
division).  The library's self-test compares the two on the GPU over generated
operands: arbitrary bit patterns, power-of-two divisors of either sign (incl.
ones whose reciprocal is subnormal or infinite), exact and power-of-two
quotients, and components of normalised vectors."""

import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_division_is_ieee_round_to_nearest(built_lib, cuda, seed):
    mismatches = C.c_uint64(0)
    bad = (C.c_uint32 * 4)()
    status = built_lib.mb_selftest_divide(seed, 1 << 28, C.byref(mismatches), bad)
    assert status == 0
    assert mismatches.value == 0, "a=%08x d=%08x got=%08x ieee=%08x" % tuple(bad)


def test_selftest_rejects_null_output(built_lib, cuda):
    assert built_lib.mb_selftest_divide(1, 16, None, None) != 0
