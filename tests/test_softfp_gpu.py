"""The integer-pipe FP64 operations of the fused pass (armon-kokkos_gb300/csrc/softfp.cuh) against
the FP64 instructions they replace, bit for bit, on generated operands."""
import ctypes as C

import pytest

import armon_gb300 as A

pytestmark = pytest.mark.gpu

MODES = {0: "random normal operands", 1: "random bit patterns (zeros, subnormals, inf, NaN)",
         2: "quotients near a rounding midpoint", 3: "exact quotients", 4: "power-of-two divisors",
         5: "zero dividends, extreme exponents", 6: "solver-like magnitudes", 100: "lt / gt0 / neg_if / lt_pos",
         101: "scale / half / twice", 102: "sqrt / absval", 103: "mul",
         104: "division quotient estimate within one", 105: "add"}


def selftest(mode, n, seed):
    L = A.lib()
    L.armon_selftest_softfp.argtypes = [C.c_uint64, C.c_int64, C.c_int32, C.POINTER(C.c_uint64)]
    out = (C.c_uint64 * 4)()
    rc = L.armon_selftest_softfp(seed, n, mode, out)
    assert rc == 0
    return list(out)


@pytest.mark.parametrize("mode", sorted(MODES), ids=lambda m: MODES[m])
def test_soft_fp64_matches_hardware(mode):
    n = 1 << 30
    for seed in (0x9E3779B97F4A7C15, 0xDEADBEEF):
        mism, fast, a, b = selftest(mode, n, seed)
        assert mism == 0, f"{MODES[mode]}: {mism} mismatches, first a=0x{a:016x} b=0x{b:016x}"
        if mode in (0, 2, 3, 4, 6):
            assert fast == n     # these operands all take the integer fast path
