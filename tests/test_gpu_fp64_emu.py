"""The integer-pipe binary64 addition used by the stencil variants of levels
1-2 (csrc/fp64_emu.cuh) must equal IEEE-754 round-to-nearest-even addition
bit for bit: against the FP64 unit on the same device and against numpy."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _bits(t):
    return t.cpu().numpy().view(np.uint64)


def _check(hc, x, y, dev):
    xt, yt = torch.from_numpy(x).to(dev), torch.from_numpy(y).to(dev)
    emu, hw = hc.selftest_dadd(xt, yt)
    assert np.array_equal(_bits(emu), _bits(hw))
    with np.errstate(over="ignore"):
        ref = x + y
    fin = np.isfinite(ref) | np.isinf(ref)
    assert np.array_equal(_bits(hw)[fin], ref.view(np.uint64)[fin])


def _from_parts(rng, n, exp_lo, exp_hi):
    e = rng.integers(exp_lo, exp_hi + 1, n).astype(np.uint64)
    m = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    return ((e << np.uint64(52)) | m).view(np.float64)


def test_random_positive_normals_every_exponent_gap(hc, dev):
    rng = np.random.default_rng(31)
    n = 1 << 20
    x = _from_parts(rng, n, 1, 2046)
    gap = rng.integers(0, 70, n)
    ex = (x.view(np.uint64) >> np.uint64(52)).astype(np.int64)
    ey = np.clip(ex - gap, 1, 2046).astype(np.uint64)
    y = ((ey << np.uint64(52)) | rng.integers(0, 1 << 52, n, dtype=np.uint64)).view(np.float64)
    _check(hc, x, y, dev)
    _check(hc, y, x, dev)  # operand order


def test_ties_carries_and_overflow(hc, dev):
    one = 1.0
    ulp = np.spacing(1.0)
    big = np.finfo(np.float64).max
    half_ulp_big = 2.0 ** 970  # half an ulp of the largest double
    xs = [one, one + ulp, one + 2 * ulp, 2.0 - ulp, 1.5, big,
          big, 1e308, 0.5, 3.0, 2.0 ** 1023, 1.0]
    ys = [ulp / 2, ulp / 2, ulp / 2, ulp / 2, 1.5, big,
          half_ulp_big, 1e308, 0.5 - ulp / 4, ulp, 2.0 ** 1023, 2.0 ** -1022]
    x, y = np.array(xs), np.array(ys)
    _check(hc, x, y, dev)
    # exhaustive low-bit patterns around ties: x = 1 + k ulp, y = j * 2^-56
    k = np.arange(64, dtype=np.float64)
    j = np.arange(64, dtype=np.float64)
    K, J = np.meshgrid(k, j)
    _check(hc, (1.0 + K * ulp).ravel(), (J * 2.0 ** -56).ravel() + 2.0 ** -60, dev)


def test_other_operand_classes_fall_back(hc, dev):
    vals = np.array([0.0, -0.0, 5e-324, 2.2250738585072009e-308, 2.2250738585072014e-308, -1.0, 1.0,
                     np.inf, -np.inf, np.nan, 1e-300, -1e-300, 1.7e308], dtype=np.float64)
    X, Y = np.meshgrid(vals, vals)
    x, y = X.ravel().copy(), Y.ravel().copy()
    xt, yt = torch.from_numpy(x).to(dev), torch.from_numpy(y).to(dev)
    emu, hw = hc.selftest_dadd(xt, yt)
    assert np.array_equal(_bits(emu), _bits(hw))  # NaN payloads included: same FP64 unit


@pytest.mark.parametrize("divisor", [3, 5])
def test_small_division_correctly_rounded(hc, dev, divisor):
    # the multiply-and-two-FMA quotient must equal IEEE division bit for bit:
    # every exponent of both signs, subnormal inputs and results, exact
    # quotients, signed zeros, the largest finite values, infinities, NaN
    rng = np.random.default_rng(40 + divisor)
    n = 1 << 21
    x = _from_parts(rng, n, 0, 2046)
    x[::2] = -x[::2]
    k = rng.integers(1, 1 << 50, 1 << 16).astype(np.float64)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, np.finfo(np.float64).max, -np.finfo(np.float64).max,
                        np.finfo(np.float64).tiny, 5e-324, -5e-324, 1e-323, 2e-323, 1.0, 3.0, 5.0, 15.0, 1.5,
                        2.0 ** -1022 * 3, 2.0 ** 1023, 0.1, 1.0 / 3.0])
    x = np.concatenate([x, k * divisor, k * divisor + 1, (k * divisor) * 2.0 ** -1074, special])
    fast, hw = hc.selftest_div(torch.from_numpy(x).to(dev), divisor)
    fb, hb = _bits(fast), _bits(hw)
    nan = np.isnan(x)
    assert np.array_equal(fb[~nan], hb[~nan])
    assert np.all(np.isnan(fast.cpu().numpy()[nan]))
    ref = x / float(divisor)
    assert np.array_equal(hb[~nan], ref.view(np.uint64)[~nan])
