"""GPU parity: scatter (+) / weighted histogram, bit-exact against the oracle
for every privatisation strategy, including the workload's bin counts."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

STRATS = ["SCATTER_AUTO", "SCATTER_SMEM_WARP", "SCATTER_SMEM_BLOCK", "SCATTER_CLUSTER", "SCATTER_GLOBAL",
          "SCATTER_PARTITION"]


def _data(hc, n, dev, seed=2, bound=1 << 20):
    d = torch.empty(n, dtype=torch.int64, device=dev)
    hc.fill_uniform_i64(d, seed, bound)
    return d


def _run(hc, data, bins, strategy, dev):
    hist = torch.zeros(bins, dtype=torch.int64, device=dev)
    hc.weighted_histogram(data, hist, strategy=strategy)
    hc.check(hc.device_check())
    return hist.cpu().numpy()


def test_known_answer_example(hc, orc, dev):
    data = torch.arange(1024, dtype=torch.int64, device=dev)
    got = _run(hc, data, 64, hc.SCATTER_AUTO, dev)
    assert got.tolist() == [sum((k + 64 * j) ** 2 for j in range(16)) for k in range(64)]


@pytest.mark.parametrize("bins", [1, 3, 64, 1000, 4096, 65536, 300000])
@pytest.mark.parametrize("strategy", STRATS)
def test_strategies_bit_exact(hc, orc, dev, bins, strategy):
    s = getattr(hc, strategy)
    data = _data(hc, 200_003, dev)
    ref = orc.weighted_hist(data.cpu().numpy(), bins)
    try:
        got = _run(hc, data, bins, s, dev)
    except hc.HydCudaError as e:
        # a forced strategy may not fit this many bins; AUTO always must
        assert e.status == hc.ERR_UNSUPPORTED and s != hc.SCATTER_AUTO
        return
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("n", [0, 1, 2, 3, 5, 33, 4099])
def test_ragged_sizes(hc, orc, dev, n):
    data = _data(hc, n, dev) if n else torch.empty(0, dtype=torch.int64, device=dev)
    for bins in (64, 65536):
        got = _run(hc, data, bins, hc.SCATTER_AUTO, dev)
        ref = orc.weighted_hist(data.cpu().numpy(), bins) if n else np.zeros(bins, np.int64)
        assert np.array_equal(got, ref)


def test_accumulates_into_existing(hc, orc, dev):
    data = _data(hc, 10000, dev)
    hist = torch.arange(64, dtype=torch.int64, device=dev)
    hc.weighted_histogram(data, hist)
    ref = orc.weighted_hist(data.cpu().numpy(), 64) + np.arange(64)
    assert np.array_equal(hist.cpu().numpy(), ref)


def test_out_of_range_routes_reported(hc, orc, dev):
    data = torch.tensor([5, -7, 9, 12], dtype=torch.int64, device=dev)
    hist = torch.zeros(4, dtype=torch.int64, device=dev)
    hc.weighted_histogram(data, hist)
    assert hc.device_check() == hc.ERR_BOUNDS
    # the in-range routes were still applied: 5%4=1 -> 25, 9%4=1 -> 81, 12%4=0 -> 144
    assert hist.cpu().tolist() == [144, 106, 0, 0]
    assert hc.device_check() == hc.OK  # the error word was cleared


def test_non_power_of_two_bins_and_wrap(hc, orc, dev):
    # large values: x*x wraps modulo 2^64 exactly like the oracle's uint64 math
    data = _data(hc, 50000, dev, seed=9, bound=(1 << 62))
    for bins in (7, 1000, 65521):
        assert np.array_equal(_run(hc, data, bins, hc.SCATTER_AUTO, dev),
                              orc.weighted_hist(data.cpu().numpy(), bins))


def test_full_size_workload_both_bin_counts(hc, orc, dev):
    n = 1 << 27  # the workload's N (1 GiB of int64)
    data = _data(hc, n, dev)
    host = data.cpu().numpy()
    for bins in (64, 65536):
        got = _run(hc, data, bins, hc.SCATTER_AUTO, dev)
        assert np.array_equal(got, orc.weighted_hist(host, bins))
        # size-independent property: the bins sum to sum(x*x) mod 2^64
        total = int(got.astype(np.uint64).sum(dtype=np.uint64))
        sq = (host.astype(np.uint64) * host.astype(np.uint64)).sum(dtype=np.uint64)
        assert total == int(sq)


def test_unfused_scatter_add(hc, orc, dev):
    rng = np.random.default_rng(3)
    for n, dst_n in ((0, 5), (10, 1), (10007, 64), (10007, 70000)):
        idx = rng.integers(0, dst_n, size=n).astype(np.int64)
        vals = rng.integers(-1000, 1000, size=n).astype(np.int64)
        dst = torch.zeros(dst_n, dtype=torch.int64, device=dev)
        if n:
            hc.scatter_add_i64(torch.from_numpy(idx).to(dev), torch.from_numpy(vals).to(dev), dst)
        hc.check(hc.device_check())
        assert np.array_equal(dst.cpu().numpy(), orc.scatter_add_i64(idx, vals, dst_n))


def test_unfused_scatter_add_f64(hc, orc, dev):
    rng = np.random.default_rng(4)
    idx = rng.integers(0, 100, size=5000).astype(np.int64)
    vals = rng.uniform(-1, 1, size=5000)
    dst = torch.zeros(100, dtype=torch.float64, device=dev)
    hc.scatter_add_f64(torch.from_numpy(idx).to(dev), torch.from_numpy(vals).to(dev), dst)
    ref = np.zeros(100)
    orc.lib().orc_scatter_add_f64(idx, vals, 5000, ref, 100)
    assert np.allclose(dst.cpu().numpy(), ref, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("bins", [16385, 65536, 65521, 262144, 1 << 19])
@pytest.mark.parametrize("n", [1, 4095, 4097, 1_000_003])
def test_partition_ragged_and_unaligned(hc, orc, dev, bins, n):
    base = _data(hc, n + 1, dev, seed=11)
    for data in (base[:n], base[1:]):  # 32-byte aligned and 8-byte aligned starts
        assert np.array_equal(_run(hc, data, bins, hc.SCATTER_PARTITION, dev),
                              orc.weighted_hist(data.cpu().numpy(), bins))


def test_partition_skewed_ranges(hc, orc, dev):
    # every element in one bin range, then two ranges of very different sizes
    data = _data(hc, 3_000_000, dev, seed=5, bound=1 << 14)
    assert np.array_equal(_run(hc, data, 65536, hc.SCATTER_PARTITION, dev),
                          orc.weighted_hist(data.cpu().numpy(), 65536))
    data2 = torch.cat([data, _data(hc, 1000, dev, seed=6) + (1 << 15)])
    assert np.array_equal(_run(hc, data2, 65536, hc.SCATTER_PARTITION, dev),
                          orc.weighted_hist(data2.cpu().numpy(), 65536))


def test_partition_out_of_range_and_repeat(hc, orc, dev):
    data = _data(hc, 100_000, dev, seed=8)
    data[::1000] = -3  # negative x with a non-zero remainder: out of range
    hist = torch.zeros(65536, dtype=torch.int64, device=dev)
    hc.weighted_histogram(data, hist, strategy=hc.SCATTER_PARTITION)
    assert hc.device_check() == hc.ERR_BOUNDS
    keep = data.cpu().numpy()
    keep = keep[keep >= 0]
    assert np.array_equal(hist.cpu().numpy(), orc.weighted_hist(keep, 65536))
    # the work queue resets itself: a second call adds the same again
    hc.weighted_histogram(data, hist, strategy=hc.SCATTER_PARTITION)
    hc.device_check()
    assert np.array_equal(hist.cpu().numpy(), 2 * orc.weighted_hist(keep, 65536))


def test_partition_more_than_one_staging_round(hc, orc, dev):
    n = (1 << 27) + 5000  # beyond one staging round of 2^27 elements
    data = _data(hc, n, dev, seed=3)
    assert np.array_equal(_run(hc, data, 65536, hc.SCATTER_PARTITION, dev),
                          orc.weighted_hist(data.cpu().numpy(), 65536))


def test_plan_reports_strategy_and_launches(hc, dev):
    assert hc.weighted_histogram_plan(1 << 27, 64) == (hc.SCATTER_SMEM_WARP, 1)
    assert hc.weighted_histogram_plan(1 << 27, 65536) == (hc.SCATTER_PARTITION, 2)
    assert hc.weighted_histogram_plan((1 << 28) + 1, 65536) == (hc.SCATTER_PARTITION, 6)
    assert hc.weighted_histogram_plan(1 << 16, 65536) == (hc.SCATTER_GLOBAL, 1)
    assert hc.weighted_histogram_plan(1 << 27, 1 << 20) == (hc.SCATTER_GLOBAL, 1)


@pytest.mark.parametrize("bins,bound", [(65536, 1 << 14), (65536, 1 << 20), (40000, 1 << 20), (131072, 1 << 40),
                                        (20000, 1 << 20)])
def test_partition_skew_widths_and_range_counts(hc, orc, dev, bins, bound):
    # 12M elements: with bound 2^14 every element lands in the first bin range
    # (one apply range gets every CTA); bound 2^40 stages every tile as 8-byte
    # records; 131072 bins take the eight-range staging path; one wide tile
    # sits mid-stream among narrow ones
    n = 12_000_017
    data = _data(hc, n, dev, seed=21, bound=bound)
    data[5_000_000:5_004_096] = _data(hc, 4096, dev, seed=22, bound=1 << 62)
    for d in (data, data[1:]):
        assert np.array_equal(_run(hc, d, bins, hc.SCATTER_PARTITION, dev),
                              orc.weighted_hist(d.cpu().numpy(), bins))


@pytest.mark.parametrize("bins", [65536, 40000])
def test_partition_mixed_record_widths(hc, orc, dev, bins):
    # tiles of small values are staged as 4-byte records, tiles holding a value
    # with a non-zero high word as 8-byte records; both must sum alike
    data = _data(hc, 50_000, dev, seed=12)
    big = _data(hc, 50_000, dev, seed=13, bound=1 << 62)
    data[4096:8192] = big[4096:8192]          # one whole wide tile
    data[20_000] = big[20_000]                # one wide element in a narrow-looking tile
    data[30_001:30_003] = (1 << 32) + 5       # high word exactly 1
    for d in (data, data[3:]):
        assert np.array_equal(_run(hc, d, bins, hc.SCATTER_PARTITION, dev),
                              orc.weighted_hist(d.cpu().numpy(), bins))
