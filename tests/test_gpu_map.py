"""GPU parity of fused map / zipwith / generate chains compiled at run time
(hyd_cuda_map_f64): every element bit-identical to the oracle's restatement of
the C backend's fused loop (the same IEEE operations in the same order, no
contraction), the (+) reduction within 1e-12 of the compensated sum and of the
oracle's reduction template, and identical run to run."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _map_chain_body(n):
    # bench/map_chain/map_chain.hyd: generate (i / n), x*x, x - 0.5, x*2 + 1
    return ("double s = (double)i / %d.0; double a = s * s; double b = a - 0.5; v = b * 2.0 + 1.0;" % n)


@pytest.mark.parametrize("n", [1, 2, 7, 4096, (1 << 20) + 3])
def test_map_chain_generate_and_reduce(hc, orc, dev, n):
    out = torch.empty(n, dtype=torch.float64, device=dev)
    _, s = hc.map_f64(_map_chain_body(n), [], n=n, out=out, want_sum=True)
    ref = orc.map_chain(n)
    assert np.array_equal(out.cpu().numpy().view(np.int64), ref.view(np.int64))
    exact = orc.sum_compensated(ref)
    scale = max(1.0, float(np.abs(ref).sum()))
    assert abs(s.item() - exact) <= 1e-12 * scale
    assert abs(s.item() - orc.map_chain_sum(n)) <= 2e-12 * scale
    _, s2 = hc.map_f64(_map_chain_body(n), [], n=n, want_sum=True)  # reduction only, same bits
    assert s2.item() == s.item()


@pytest.mark.parametrize("n", [3, 1001, 65536])
@pytest.mark.parametrize("offset", [0, 1])
def test_zipwith_three_inputs_elementwise(hc, orc, dev, n, offset):
    rng = np.random.default_rng(n + offset)
    host = [rng.uniform(-2, 2, n + 1) for _ in range(3)]
    xs = [torch.from_numpy(h).to(dev)[offset:offset + n] for h in host]
    out = torch.empty(n + 1, dtype=torch.float64, device=dev)[offset:offset + n]
    hc.map_f64("v = x0 * x1 + x2;", xs, out=out)
    ref = orc.zipwith_muladd(*(h[offset:offset + n] for h in host))
    assert np.array_equal(out.cpu().numpy().view(np.int64), ref.view(np.int64))


def test_zipwith_three_inputs_full_size(hc, orc, dev):
    """The memory-bound chain of the bench at its full size: 2^27 float64 per
    input (three inputs and one output, 4 GiB), bit-exact against the oracle."""
    n = 1 << 27
    xs = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(3)]
    for k, t in enumerate(xs):
        hc.fill_uniform_f64(t, 21 + k, -1.0, 1.0)
    out = torch.empty(n, dtype=torch.float64, device=dev)
    hc.map_f64("v = x0 * x1 + x2;", xs, out=out)
    ref = orc.zipwith_muladd(*(orc.uniform_f64(n, 21 + k, -1.0, 1.0) for k in range(3)))
    assert np.array_equal(out.cpu().numpy().view(np.int64), ref.view(np.int64))


def test_empty_and_sum_only(hc, dev):
    x = torch.empty(0, dtype=torch.float64, device=dev)
    _, s = hc.map_f64("v = x0 + 1.0;", [x], n=0, want_sum=True)
    assert s.item() == 0.0


def test_body_that_does_not_compile_is_reported(hc, dev):
    x = torch.ones(8, dtype=torch.float64, device=dev)
    with pytest.raises(hc.HydCudaError) as e:
        hc.map_f64("v = no_such_function(x0);", [x], out=torch.empty_like(x))
    assert e.value.status == hc.ERR_INVALID
    assert "does not compile" in str(e.value)


@pytest.mark.parametrize("n", [1, 7, 4096, (1 << 20) + 3])
def test_map_i64_generate_zipwith_and_sum(hc, orc, dev, n):
    """int64 chains: generate with C's truncating / and % (the coo_csr_build
    program's row_of), and zipwith over resident inputs with a wrapping sum."""
    out = torch.empty(n, dtype=torch.int64, device=dev)
    body = "long long g = i / 3; v = (g * 17 + 3) - (((g * 17 + 3) / 1000) * 1000);"
    _, s = hc.map_i64(body, [], n=n, out=out, want_sum=True)
    g = np.arange(n, dtype=np.int64) // 3
    ref = (g * 17 + 3) - (((g * 17 + 3) // 1000) * 1000)
    assert np.array_equal(out.cpu().numpy(), ref)
    assert s.item() == int(ref.sum())
    a = torch.empty(n, dtype=torch.int64, device=dev)
    b = torch.empty(n, dtype=torch.int64, device=dev)
    hc.fill_uniform_i64(a, 5, 1 << 62)
    hc.fill_uniform_i64(b, 6, 1 << 62)
    o2 = torch.empty_like(a)
    _, s2 = hc.map_i64("v = x0 * 3 + x1;", [a, b], out=o2, want_sum=True)
    ha, hb = a.cpu().numpy().astype(np.uint64), b.cpu().numpy().astype(np.uint64)
    ref2 = (ha * np.uint64(3) + hb).astype(np.int64)
    assert np.array_equal(o2.cpu().numpy(), ref2)
    assert s2.item() == int(ref2.astype(np.uint64).sum(dtype=np.uint64).astype(np.int64))
