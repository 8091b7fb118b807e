"""CPU check of the constant-divisor division the stencils use for x / 3 and
x / 5 (`ddiv_small_rn` in csrc/fp64_emu.cuh): one multiply by RN(1/D), an
exact remainder, one fused correction.  The three steps are reproduced here
with exact rational arithmetic (each FMA is one rounding of an exact value)
and must give IEEE x / D bit for bit; the GPU test checks the CUDA code
against the device's own division."""
from fractions import Fraction

import numpy as np
import pytest


def _rn(q):
    # round an exact rational to the nearest double, ties to even
    return float(q)


def _method(x, d):
    z = 1.0 / d                          # RN(1/D)
    q0 = x * z                           # RN(x * z)
    if not np.isfinite(q0):
        return q0
    r = Fraction(x) - d * Fraction(q0)   # the FMA's exact value ...
    r = _rn(r)                           # ... rounded once (exact: asserted below)
    assert Fraction(r) == Fraction(x) - d * Fraction(q0)
    if r == 0.0:
        return q0
    return _rn(Fraction(q0) + Fraction(r) * Fraction(z))


def _doubles(rng, n):
    e = rng.integers(0, 2047, n).astype(np.uint64)
    m = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    x = ((e << np.uint64(52)) | m).view(np.float64)
    x[::2] = -x[::2]
    return x


@pytest.mark.parametrize("d", [3, 5])
def test_constant_division_matches_ieee(d):
    rng = np.random.default_rng(7 + d)
    xs = list(_doubles(rng, 4000))
    xs += [0.0, -0.0, 5e-324, -5e-324, 1e-323, np.finfo(np.float64).tiny, np.finfo(np.float64).max,
           -np.finfo(np.float64).max, 1.0, 3.0, 5.0, 15.0, 0.1, 2.0 ** 1023]
    xs += [float(k * d) for k in range(1, 200)] + [float(k * d + 1) for k in range(1, 200)]
    xs += [k * d * 5e-324 for k in range(1, 50)]
    for x in xs:
        got, want = _method(float(x), d), float(x) / d
        assert np.float64(got).view(np.uint64) == np.float64(want).view(np.uint64), (x, got, want)
