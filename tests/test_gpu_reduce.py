"""GPU parity: deterministic fp64 reductions against the oracle.

Tolerance (stated by the workload): |gpu - oracle| <= 1e-12 * max(1, |ref|)
relative, where ref is the compensated (two-product + Neumaier) FP64 sum;
the C-backend restatement is checked against the same bound.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _inputs(hc, n, dev, seeds=(1, 2)):
    xs = torch.empty(n, dtype=torch.float64, device=dev)
    ys = torch.empty(n, dtype=torch.float64, device=dev)
    hc.fill_uniform_f64(xs, seeds[0], -1.0, 1.0)
    hc.fill_uniform_f64(ys, seeds[1], -1.0, 1.0)
    return xs, ys


def test_generator_matches_oracle(hc, orc, dev):
    for n in (1, 7, 1000, 65537):
        x = torch.empty(n, dtype=torch.float64, device=dev)
        hc.fill_uniform_f64(x, 11, -1.0, 1.0)
        assert np.array_equal(x.cpu().numpy(), orc.uniform_f64(n, 11, -1.0, 1.0))
        i = torch.empty(n, dtype=torch.int64, device=dev)
        hc.fill_uniform_i64(i, 12, 1 << 20)
        assert np.array_equal(i.cpu().numpy(), orc.uniform_i64(n, 12, 1 << 20))


@pytest.mark.parametrize("n", [0, 1, 3, 4, 5, 31, 1000, 4096 + 3, 1 << 20, (1 << 20) + 7])
def test_dot_matches_oracle(hc, orc, dev, n):
    xs, ys = _inputs(hc, n, dev)
    out = torch.full((1,), 123.0, dtype=torch.float64, device=dev)
    hc.dot_f64(xs, ys, out)
    got = float(out.item())
    hx, hy = xs.cpu().numpy(), ys.cpu().numpy()
    ref = orc.dot_compensated(hx, hy) if n else 0.0
    cback = orc.dot(hx, hy) if n else 0.0
    assert abs(got - ref) <= TOL * max(1.0, abs(ref))
    assert abs(cback - ref) <= TOL * max(1.0, abs(ref))
    # and directly against the C backend's own result (the workload's bound)
    assert abs(got - cback) <= TOL * max(1.0, abs(cback))


def test_dot_full_size_deterministic(hc, orc, dev):
    n = 1 << 24  # the workload's N
    xs, ys = _inputs(hc, n, dev)
    outs = []
    for _ in range(3):
        out = torch.zeros(1, dtype=torch.float64, device=dev)
        hc.dot_f64(xs, ys, out)
        outs.append(out.item())
    assert outs[0] == outs[1] == outs[2]  # bit-identical run to run
    hx, hy = xs.cpu().numpy(), ys.cpu().numpy()
    ref = orc.dot_compensated(hx, hy)
    assert abs(outs[0] - ref) <= TOL * max(1.0, abs(ref))
    cback = orc.dot(hx, hy)  # the C backend's OpenMP reduction
    assert abs(outs[0] - cback) <= TOL * max(1.0, abs(cback))


def test_dot_unaligned_views(hc, orc, dev):
    xs, ys = _inputs(hc, 10001, dev)
    a, b = xs[1:], ys[3:10003 - 2]  # 8-byte aligned, not 32-byte aligned
    n = min(a.numel(), b.numel())
    a, b = a[:n], b[:n]
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    hc.dot_f64(a, b, out)
    ref = orc.dot_compensated(a.cpu().numpy(), b.cpu().numpy())
    assert abs(out.item() - ref) <= TOL * max(1.0, abs(ref))


def test_sum_matches_oracle(hc, orc, dev):
    for n in (1, 999, 1 << 18):
        xs, _ = _inputs(hc, n, dev)
        out = torch.zeros(1, dtype=torch.float64, device=dev)
        hc.sum_f64(xs, out)
        ref = orc.lib().orc_sum_f64_compensated(xs.cpu().numpy(), n)
        assert abs(out.item() - ref) <= TOL * max(1.0, abs(ref))


def test_dot_on_side_stream(hc, orc, dev):
    s = torch.cuda.Stream()
    xs, ys = _inputs(hc, 50000, dev)
    torch.cuda.synchronize()
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    with torch.cuda.stream(s):
        hc.dot_f64(xs, ys, out, stream=s)
    s.synchronize()
    ref = orc.dot_compensated(xs.cpu().numpy(), ys.cpu().numpy())
    assert abs(out.item() - ref) <= TOL * max(1.0, abs(ref))
