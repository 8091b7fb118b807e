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


def test_scans_at_the_benchmark_size(hc, orc, dev):
    """Both scans at the benchmarked 2^27 elements (32768 tiles, 1024 blocks of
    the float64 scan's two-level fold): int64 bit-exact against the oracle's
    serial fold, float64 within the tolerance and identical over runs, forward
    exclusive (the benchmark's form) and reverse inclusive."""
    n = 1 << 27
    xi = _i64(hc, n, dev, seed=41)
    hi = xi.cpu().numpy()
    xf = torch.empty(n, dtype=torch.float64, device=dev)
    hc.fill_uniform_f64(xf, 41, -1.0, 1.0)
    hf = xf.cpu().numpy()
    for rev, inc in ((False, False), (True, True)):
        out = torch.empty_like(xi)
        hc.scan(xi, out, 3, rev, inc)
        hc.check(hc.device_check())
        assert np.array_equal(out.cpu().numpy(), orc.scan_i64(hi, 3, rev, inc))
        del out
        outs = []
        for _ in range(2):
            o = torch.empty_like(xf)
            hc.scan(xf, o, 0.5, rev, inc)
            outs.append(o)
        hc.check(hc.device_check())
        ref = orc.scan_f64(hf, 0.5, rev, inc)
        bound = orc.scan_f64(np.abs(hf), 0.5, rev, inc)
        assert np.all(np.abs(outs[0].cpu().numpy() - ref) <= 1e-12 * np.maximum(bound, 1.0))
        assert torch.equal(outs[0], outs[1])
        del outs


def test_segmented_reduce_at_the_benchmark_size(hc, orc, dev):
    """The benchmarked segmented reduce: 2^27 float64 and int64 values, segment
    lengths floor(2^U(0,16)) (seed 43, about 22,700 segments, the longest
    near 2^16): int64 bit-exact, float64 within the tolerance of the serial
    sums and identical over runs."""
    n = 1 << 27
    rng = np.random.default_rng(43)
    lens = np.floor(2.0 ** rng.uniform(0, 16, size=n // 1000)).astype(np.int64)
    cum = np.cumsum(lens)
    k = int(np.searchsorted(cum, n))
    lens = lens[:k + 1]
    lens[-1] -= int(cum[k] - n)
    offsets = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    offsets[-1] = n
    _check_segreduce(hc, orc, dev, offsets, n, seed=43)


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


def test_scan_f64_many_tiles_deterministic(hc, orc, dev):
    """The single-pass float64 scan over 2^22 + 77 elements (1025 tiles): within
    tolerance of the serial fold and bit-identical over repeated runs, whatever
    order the tiles finished their look-back in."""
    n = (1 << 22) + 77
    x = torch.empty(n, dtype=torch.float64, device=dev)
    hc.fill_uniform_f64(x, 17, -1.0, 1.0)
    h = x.cpu().numpy()
    for rev, inc in VARIANTS:
        outs = []
        for _ in range(3):
            out = torch.empty_like(x)
            hc.scan(x, out, -0.25, rev, inc)
            outs.append(out)
        hc.check(hc.device_check())
        ref = orc.scan_f64(h, -0.25, rev, inc)
        bound = orc.scan_f64(np.abs(h), 0.25, rev, inc)
        assert np.all(np.abs(outs[0].cpu().numpy() - ref) <= 1e-12 * np.maximum(bound, 1.0))
        assert torch.equal(outs[0], outs[1]) and torch.equal(outs[0], outs[2])


def _segments(rng, nseg, kind):
    if kind == "loguniform":    # a few segments far longer than a tile, most short
        lens = np.floor(2.0 ** rng.uniform(0, 20, size=nseg)).astype(np.int64)
    elif kind == "tile_aligned":  # boundaries on the 4096-value tile edges
        lens = 4096 * rng.integers(0, 4, size=nseg)
    elif kind == "one_long":
        lens = np.ones(nseg, dtype=np.int64)
        lens[nseg // 2] = 3 * (1 << 20) + 5
    else:                       # many empty segments between short ones
        lens = rng.integers(0, 3, size=nseg)
    return np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)


def _check_segreduce(hc, orc, dev, offsets, nv, seed, init_i=3, init_f=0.25, lead=0):
    rng = np.random.default_rng(seed)
    vals_i = rng.integers(-(1 << 40), 1 << 40, size=nv).astype(np.int64)
    vals_f = rng.uniform(-1, 1, size=nv)
    nseg = len(offsets) - 1
    d_off = torch.from_numpy(offsets).to(dev)
    out_i = torch.empty(nseg, dtype=torch.int64, device=dev)
    outs_f = [torch.empty(nseg, dtype=torch.float64, device=dev) for _ in range(2)]
    hc.segmented_reduce(d_off, torch.from_numpy(vals_i).to(dev), out_i, init=init_i)
    dv = torch.from_numpy(vals_f).to(dev)
    for o in outs_f:
        hc.segmented_reduce(d_off, dv, o, init=init_f)
    hc.check(hc.device_check())
    assert np.array_equal(out_i.cpu().numpy(), orc.segmented_reduce_i64(offsets, vals_i, init_i))
    ref = orc.segmented_reduce_f64(offsets, vals_f, init_f)
    absum = orc.segmented_reduce_f64(offsets, np.abs(vals_f), 0.0)
    got = outs_f[0].cpu().numpy()
    assert np.all(np.abs(got - ref) <= 1e-12 * np.maximum(absum, 1.0))
    assert torch.equal(outs_f[0], outs_f[1])  # run-to-run identical


@pytest.mark.parametrize("kind,nseg", [("loguniform", 3000), ("tile_aligned", 700), ("one_long", 20_000),
                                       ("empty_heavy", 300_000)])
def test_segmented_reduce_balanced_shapes(hc, orc, dev, kind, nseg):
    offsets = _segments(np.random.default_rng(nseg), nseg, kind)
    _check_segreduce(hc, orc, dev, offsets, int(offsets[-1]), seed=nseg)


def test_segmented_reduce_values_outside_segments(hc, orc, dev):
    # offsets[0] > 0 and offsets[-1] < n_vals: the values before the first and
    # after the last segment belong to none
    rng = np.random.default_rng(9)
    lens = rng.integers(0, 9000, size=400)
    offsets = (5000 + np.concatenate([[0], np.cumsum(lens)])).astype(np.int64)
    _check_segreduce(hc, orc, dev, offsets, int(offsets[-1]) + 12_345, seed=9)


@pytest.mark.parametrize("tail", [0, 1, 3, 7, 8, 9, 4095, 4096, 4097])
def test_segmented_reduce_ends_at_thread_and_tile_edges(hc, orc, dev, tail):
    """Segment ends at every position class a tile's threads meet (8 values
    per thread, 4096 per tile): ends on the last or first value of a thread,
    one-value segments, runs of empty segments, and the last segment ending
    `tail` values before n_vals (values outside every segment after it)."""
    ends = []
    pos = 0
    for t in range(40):  # the first 40 threads of tiles 0 and 1, then a long one
        for e in (8 * t + 7, 8 * t + 8, 8 * t + 9):
            if e > pos:
                ends += [e, e] if t % 5 == 0 else [e]  # some empty segments
                pos = e
    for e in (4095, 4096, 4097, 4103, 4104, 8191, 8192, 3 * 4096 + 5):
        if e > pos:
            ends.append(e)
            pos = e
    offsets = np.concatenate([[0], np.array(ends)]).astype(np.int64)
    _check_segreduce(hc, orc, dev, offsets, int(offsets[-1]) + tail, seed=31 + tail)


def test_segmented_reduce_empty_values_and_trailing_empties(hc, orc, dev):
    # no values at all: every segment is empty and yields init
    _check_segreduce(hc, orc, dev, np.zeros(1001, dtype=np.int64), 0, seed=1)
    # empty segments at the very end (offset == n_vals) and at a tile edge
    offsets = np.array([0, 4096, 4096, 4096, 8192, 9000, 9000, 9000], dtype=np.int64)
    _check_segreduce(hc, orc, dev, offsets, 9000, seed=2)


@pytest.mark.parametrize("where", ["middle", "first_negative", "last_beyond"])
def test_segmented_reduce_invalid_offsets_large(hc, orc, dev, where):
    """Invalid offsets deep inside a large array: the tiles detect them and the
    per-segment pass gives every valid segment its sum, every invalid one init,
    and reports the error."""
    rng = np.random.default_rng(77)
    lens = rng.integers(0, 600, size=50_000)
    offsets = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    nv = int(offsets[-1])
    if where == "middle":
        offsets[30_000] = offsets[29_990]      # decreasing pair(s) inside the array
    elif where == "first_negative":
        offsets[0] = -3
    else:
        offsets[-1] = nv + 10
    vals = rng.integers(-1000, 1000, size=nv).astype(np.int64)
    out = torch.empty(len(offsets) - 1, dtype=torch.int64, device=dev)
    hc.segmented_reduce(torch.from_numpy(offsets).to(dev), torch.from_numpy(vals).to(dev), out, init=7)
    assert hc.device_check() == hc.ERR_BOUNDS
    got = out.cpu().numpy()
    for s in range(len(offsets) - 1):
        a, b = offsets[s], offsets[s + 1]
        if a < 0 or b > nv or b < a:
            assert got[s] == 7, s
        elif s % 97 == 0 or abs(s - 30_000) < 20:
            assert got[s] == 7 + int(vals[a:b].sum()), s
