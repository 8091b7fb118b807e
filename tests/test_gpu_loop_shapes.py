"""GPU parity of the further fused loop shapes of the C backend: `reduce` over
the trailing axis (EReduce, Lowering.hs:723-760) and a guarded scatter phase
(Lowering.hs:1768-1790), against the oracle's serial restatements."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rows,cols", [(0, 5), (5, 0), (1, 1), (7, 3), (1000, 31), (1000, 32), (1000, 33),
                                       (3, 100_003), (5, 1_000_003), (200_000, 50), (64, 4096), (3000, 700)])
@pytest.mark.parametrize("op", [0, 1])
def test_reduce_rows(hc, orc, dev, rows, cols, op):
    rng = np.random.default_rng(rows * 7 + cols + op)
    xi = rng.integers(-(1 << 62), 1 << 62, (rows, cols))
    out = torch.empty(rows, dtype=torch.int64, device=dev)
    hc.reduce_rows(torch.from_numpy(xi).to(dev), op, 12345, out)
    hc.check(hc.device_check())
    assert np.array_equal(out.cpu().numpy(), orc.reduce_rows(xi, op, 12345))

    xf = rng.uniform(-1, 1, (rows, cols)) if op == 0 else rng.uniform(0.5, 1.5, (rows, cols))
    if op == 1 and cols > 4096:
        xf = rng.uniform(0.999, 1.001, (rows, cols))
    xt = torch.from_numpy(xf).to(dev)
    got = torch.empty(rows, dtype=torch.float64, device=dev)
    hc.reduce_rows(xt, op, 0.25, got)
    again = torch.empty_like(got)
    hc.reduce_rows(xt, op, 0.25, again)
    assert torch.equal(got, again)  # deterministic
    ref = orc.reduce_rows(xf, op, 0.25)
    g = got.cpu().numpy()
    if cols <= 32:
        assert np.array_equal(g.view(np.uint64), ref.view(np.uint64))  # the reference's order
    elif op == 0:
        assert np.all(np.abs(g - ref) <= 1e-12 * (np.abs(xf).sum(axis=1) + 0.25))
    else:
        assert np.all(np.abs(g - ref) <= 1e-12 * np.abs(ref))


@pytest.mark.parametrize("bins", [1, 64, 4096, 65536, 300_000])
@pytest.mark.parametrize("strategy", ["SCATTER_AUTO", "SCATTER_SMEM_WARP", "SCATTER_GLOBAL", "SCATTER_CLUSTER"])
def test_guarded_scatter_bit_exact(hc, orc, dev, bins, strategy):
    rng = np.random.default_rng(bins)
    n = 400_003
    idx = rng.integers(0, bins, n)
    vals = rng.integers(-(1 << 40), 1 << 40, n)
    guard = (rng.random(n) < 0.5).astype(np.int64) * rng.integers(1, 5, n)
    off = np.flatnonzero(guard == 0)[:1000]
    idx[off] = -12345  # out of range, but never read: its guard is false
    ref, st = orc.scatter_add_guarded_i64(idx, vals, guard, bins)
    assert st == 0
    dst = torch.zeros(bins, dtype=torch.int64, device=dev)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    try:
        hc.scatter_add_guarded_i64(t(idx), t(vals), t(guard), dst, getattr(hc, strategy))
    except hc.HydCudaError as e:
        assert e.status == hc.ERR_UNSUPPORTED and strategy != "SCATTER_AUTO"
        return
    assert hc.device_check() == 0
    assert np.array_equal(dst.cpu().numpy(), ref)


def test_guarded_scatter_reports_a_guarded_route_out_of_range(hc, dev):
    idx = torch.tensor([0, 9, 1], dtype=torch.int64, device=dev)
    vals = torch.tensor([1, 2, 3], dtype=torch.int64, device=dev)
    guard = torch.tensor([1, 1, 1], dtype=torch.int64, device=dev)
    dst = torch.zeros(4, dtype=torch.int64, device=dev)
    hc.scatter_add_guarded_i64(idx, vals, guard, dst)
    assert hc.device_check() == hc.ERR_BOUNDS
    assert dst.cpu().tolist() == [1, 3, 0, 0]
