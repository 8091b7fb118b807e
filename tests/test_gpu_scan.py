"""GPU parity: scan family (int64 bit-exact, float64 within tolerance) and
segmented reduce, against the oracle's serial folds."""
import json
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
VARIANTS = [(False, False), (False, True), (True, False), (True, True)]  # (reverse, inclusive)


def _i64(hc, n, dev, seed=5, bound=1 << 40):
    t = torch.empty(n, dtype=torch.int64, device=dev)
    if n:
        hc.fill_uniform_i64(t, seed, bound)
    return t


def test_known_answers(hc, dev):
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        ka = json.load(f)
    c = ka["scan_family_1234"]
    x = torch.tensor(c["input"], dtype=torch.int64, device=dev)
    out = torch.empty_like(x)
    for (rev, inc), key in zip(VARIANTS, ["scan", "scan_inclusive", "scanr", "scanr_inclusive"]):
        hc.scan(x, out, 0, rev, inc)
        assert out.cpu().tolist() == c[key], key
    for key in ("segmented_reduce_test", "segmented_group_sum_example"):
        c = ka[key]
        off = torch.tensor(c["offsets"], dtype=torch.int64, device=dev)
        vals = torch.tensor(c["vals"], dtype=torch.int64, device=dev)
        out = torch.empty(len(c["offsets"]) - 1, dtype=torch.int64, device=dev)
        hc.segmented_reduce(off, vals, out)
        assert out.cpu().tolist() == c["expect"]


@pytest.mark.parametrize("n", [0, 1, 2, 31, 4095, 4096, 4097, 100_000, 1 << 20, (1 << 22) + 77])
@pytest.mark.parametrize("variant", VARIANTS)
def test_scan_i64_bit_exact(hc, orc, dev, n, variant):
    rev, inc = variant
    x = _i64(hc, n, dev)
    out = torch.empty_like(x)
    hc.scan(x, out, 12345, rev, inc)
    hc.check(hc.device_check())
    ref = orc.scan_i64(x.cpu().numpy(), 12345, rev, inc)
    assert np.array_equal(out.cpu().numpy(), ref)


def test_scan_i64_wraps(hc, orc, dev):
    x = _i64(hc, 50_000, dev, seed=6, bound=(1 << 62))
    out = torch.empty_like(x)
    hc.scan(x, out, -7, False, True)
    assert np.array_equal(out.cpu().numpy(), orc.scan_i64(x.cpu().numpy(), -7, False, True))


@pytest.mark.parametrize("n", [1, 4097, 1 << 20])
@pytest.mark.parametrize("variant", VARIANTS)
def test_scan_f64_tolerance(hc, orc, dev, n, variant):
    rev, inc = variant
    x = torch.empty(n, dtype=torch.float64, device=dev)
    hc.fill_uniform_f64(x, 7, -1.0, 1.0)
    out = torch.empty_like(x)
    hc.scan(x, out, 0.5, rev, inc)
    h = x.cpu().numpy()
    ref = orc.scan_f64(h, 0.5, rev, inc)
    bound = orc.scan_f64(np.abs(h), 0.5, rev, inc)  # prefix sums of |x|
    got = out.cpu().numpy()
    assert np.all(np.abs(got - ref) <= 1e-12 * np.maximum(bound, 1.0))
    out2 = torch.empty_like(x)
    hc.scan(x, out2, 0.5, rev, inc)
    assert torch.equal(out, out2)  # run-to-run reproducible


@pytest.mark.parametrize("nseg", [0, 1, 5, 1000, 100_000])
def test_segmented_reduce(hc, orc, dev, nseg):
    rng = np.random.default_rng(nseg)
    lens = rng.integers(0, 300, size=nseg)
    lens[::7] = 0  # empty segments
    offsets = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    nv = int(offsets[-1])
    vals_i = rng.integers(-(1 << 40), 1 << 40, size=nv).astype(np.int64)
    vals_f = rng.uniform(-1, 1, size=nv)
    d_off = torch.from_numpy(offsets).to(dev)
    out_i = torch.empty(nseg, dtype=torch.int64, device=dev)
    out_f = torch.empty(nseg, dtype=torch.float64, device=dev)
    if nseg:
        hc.segmented_reduce(d_off, torch.from_numpy(vals_i).to(dev), out_i, init=3)
        hc.segmented_reduce(d_off, torch.from_numpy(vals_f).to(dev), out_f, init=0.25)
    hc.check(hc.device_check())
    assert np.array_equal(out_i.cpu().numpy(), orc.segmented_reduce_i64(offsets, vals_i, 3))
    ref = orc.segmented_reduce_f64(offsets, vals_f, 0.25)
    absum = orc.segmented_reduce_f64(offsets, np.abs(vals_f), 0.0)
    assert np.all(np.abs(out_f.cpu().numpy() - ref) <= 1e-12 * np.maximum(absum, 1.0))


def test_segmented_reduce_bad_offsets(hc, dev):
    off = torch.tensor([0, 3, 2, 10], dtype=torch.int64, device=dev)
    vals = torch.ones(5, dtype=torch.int64, device=dev)
    out = torch.empty(3, dtype=torch.int64, device=dev)
    hc.segmented_reduce(off, vals, out, init=0)
    assert hc.device_check() == hc.ERR_BOUNDS
    assert out.cpu().tolist()[0] == 3
