"""GPU parity: 2-D clamp stencils and iterate, bit-exact against the oracle
(the C backend's split-region loops) and against the reference's own stencil
outputs stored in tests/golden."""
import json
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KINDS = [0, 1, 2, 3]  # LAPLACIAN, JACOBI, HEAT, HEAT_EXAMPLE


def _grid(hc, h, w, dev, seed=3):
    g = torch.empty((h, w), dtype=torch.float64, device=dev)
    if h * w:
        hc.fill_uniform_f64(g, seed, 0.0, 1.0)
    return g


@pytest.mark.parametrize("shape", [(1, 1), (1, 2), (1, 7), (2, 2), (3, 5), (2, 130), (17, 130),
                                   (33, 257), (64, 256), (100, 1000), (129, 4098), (513, 1024)])
@pytest.mark.parametrize("kind", KINDS)
def test_single_step_bit_exact(hc, orc, dev, shape, kind):
    h, w = shape
    g = _grid(hc, h, w, dev)
    out = torch.full_like(g, float("nan"))
    hc.stencil2d(kind, g, out)
    hc.check(hc.device_check())
    ref = orc.stencil2d(kind, g.cpu().numpy())
    assert np.array_equal(out.cpu().numpy(), ref)


def test_known_answer_laplacian_example(hc, dev):
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        c = json.load(f)["stencil2d_laplacian_example"]
    g = torch.tensor(c["input"], dtype=torch.float64, device=dev)
    out = torch.empty_like(g)
    hc.stencil2d(hc.STENCIL_LAPLACIAN, g, out)
    assert out.cpu().numpy().tolist() == c["expect"]


def test_reference_bench_vectors(hc, dev):
    z = np.load(os.path.join(GOLDEN, "witness_laplacian.npz"))
    g = torch.from_numpy(z["grid"]).to(dev)
    out = torch.empty_like(g)
    hc.stencil2d(hc.STENCIL_LAPLACIAN, g, out)
    assert np.array_equal(out.cpu().numpy(), z["out"])
    z = np.load(os.path.join(GOLDEN, "witness_jacobi5.npz"))
    b0 = torch.from_numpy(z["grid"]).to(dev).contiguous()
    b1 = torch.empty_like(b0)
    res = hc.iterate_stencil2d(hc.STENCIL_JACOBI, b0, b1, 5)
    assert np.array_equal(res.cpu().numpy(), z["out"])


@pytest.mark.parametrize("shape,iters", [((64, 128), 10), ((130, 258), 7), ((33, 257), 5), ((512, 512), 100)])
def test_iterate_graph_bit_exact(hc, orc, dev, shape, iters):
    h, w = shape
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    for kind in (hc.STENCIL_HEAT, hc.STENCIL_JACOBI):
        b0 = _grid(hc, h, w, dev)
        b1 = torch.empty_like(b0)
        torch.cuda.synchronize()
        init = b0.cpu().numpy()
        with torch.cuda.stream(side):
            res = hc.iterate_stencil2d(kind, b0, b1, iters, stream=side)
            # replay of the cached graph from the same initial state
        side.synchronize()
        first = res.cpu().numpy()
        assert np.array_equal(first, orc.iterate_stencil2d(kind, init, iters))
        b0.copy_(torch.from_numpy(init).to(dev))
        torch.cuda.synchronize()
        with torch.cuda.stream(side):
            res2 = hc.iterate_stencil2d(kind, b0, b1, iters, stream=side)
        side.synchronize()
        assert np.array_equal(res2.cpu().numpy(), first)


def test_iterate_default_stream_and_zero_iters(hc, orc, dev):
    b0 = _grid(hc, 40, 60, dev)
    b1 = torch.empty_like(b0)
    init = b0.cpu().numpy()
    res = hc.iterate_stencil2d(hc.STENCIL_HEAT, b0, b1, 3)
    assert np.array_equal(res.cpu().numpy(), orc.iterate_stencil2d(orc.HEAT, init, 3))
    res0 = hc.iterate_stencil2d(hc.STENCIL_HEAT, b0, b1, 0)
    assert res0.data_ptr() == b0.data_ptr()


def test_full_size_heat_steps(hc, orc, dev):
    """The workload's grid (8192^2 float64): a few steps bit-exact against the C backend."""
    h = w = 8192
    b0 = _grid(hc, h, w, dev)
    b1 = torch.empty_like(b0)
    init = b0.cpu().numpy()
    side = torch.cuda.Stream()
    torch.cuda.synchronize()
    with torch.cuda.stream(side):
        res = hc.iterate_stencil2d(hc.STENCIL_HEAT, b0, b1, 4, stream=side)
    side.synchronize()
    assert np.array_equal(res.cpu().numpy(), orc.iterate_stencil2d(orc.HEAT, init, 4))


def _ulp_distance(a, b):
    """Distance in units in the last place between float64 arrays, through the
    monotone map of IEEE-754 bit patterns onto the integers."""
    def ordered(x):
        i = np.ascontiguousarray(x).view(np.int64)
        return np.where(i < 0, np.int64(-0x8000000000000000) - i, i)
    return np.abs(ordered(a) - ordered(b)).astype(np.float64)


def test_full_size_heat_1000_steps_drift(hc, orc, dev, record_property):
    """The heat_2d workload end to end: 8192^2 float64, U[0,1) seed 3, 1000 steps
    as a captured graph, with the autotuned variant and with the reference's
    fixed 32x32 tile, against the oracle's 1000-step iterate of the C backend's
    split-region loops.  The final-state drift is reported in ulp (max, mean);
    every step is exact, so it must be 0 for both."""
    h = w = 8192
    iters = 1000
    init = _grid(hc, h, w, dev)
    ref = orc.iterate_stencil2d(orc.HEAT, init.cpu().numpy(), iters)
    side = torch.cuda.Stream()
    for name, variant in (("autotuned", -1), ("fixed_32x32", 0)):
        b0 = init.clone()
        b1 = torch.empty_like(b0)
        torch.cuda.synchronize()
        with torch.cuda.stream(side):
            res = hc.iterate_stencil2d(hc.STENCIL_HEAT, b0, b1, iters, stream=side, variant=variant)
        side.synchronize()
        hc.check(hc.device_check())
        got = res.cpu().numpy()
        d = _ulp_distance(got, ref)
        record_property("heat_2d_8192_1000_%s_ulp_max" % name, float(d.max()))
        record_property("heat_2d_8192_1000_%s_ulp_mean" % name, float(d.mean()))
        print("heat_2d 8192^2 x 1000 steps, %s: drift vs oracle max %g ulp, mean %g ulp"
              % (name, d.max(), d.mean()))
        assert d.max() == 0, (name, d.max(), d.mean())
        del b0, b1, res


def test_invalid_arguments(hc, dev):
    g = _grid(hc, 4, 4, dev)
    assert hc.lib().hyd_cuda_stencil2d_f64(7, g.data_ptr(), g.data_ptr(), 4, 4, None) == hc.ERR_INVALID
    assert hc.lib().hyd_cuda_stencil2d_f64(0, g.data_ptr(), g.data_ptr(), 4, 4, None) == hc.ERR_INVALID


@pytest.mark.parametrize("boundary", ["wrap", "mirror", "constant"])
@pytest.mark.parametrize("h,w", [(2, 2), (3, 7), (9, 1), (1, 6), (33, 65), (257, 130)])
def test_other_boundaries_bit_exact(hc, orc, dev, boundary, h, w):
    # stencil wrap / mirror / (constant c): every kind, one step and a captured
    # 12-step iterate, bit for bit against the oracle's restatement of the
    # reference's index arithmetic; mirror on an extent of 1 is refused
    bmap = {"wrap": (hc.BOUNDARY_WRAP, orc.WRAP), "mirror": (hc.BOUNDARY_MIRROR, orc.MIRROR),
            "constant": (hc.BOUNDARY_CONSTANT, orc.CONST)}
    hb, ob = bmap[boundary]
    fill = -0.75 if boundary == "constant" else 0.0
    rng = np.random.default_rng(h * 1000 + w)
    g = rng.uniform(-1, 1, (h, w))
    src = torch.from_numpy(g).to(dev)
    dst = torch.empty_like(src)
    for kind in (hc.STENCIL_LAPLACIAN, hc.STENCIL_JACOBI, hc.STENCIL_HEAT, hc.STENCIL_HEAT_EXAMPLE):
        if boundary == "mirror" and min(h, w) < 2:
            with pytest.raises(hc.HydCudaError) as e:
                hc.stencil2d_bnd(kind, hb, src, dst, fill)
            assert e.value.status == hc.ERR_INVALID
            continue
        hc.stencil2d_bnd(kind, hb, src, dst, fill)
        torch.cuda.synchronize()
        ref = orc.stencil2d_bnd(kind, ob, g, fill)
        assert np.array_equal(dst.cpu().numpy().view(np.uint64), ref.view(np.uint64)), kind
        b0, b1 = src.clone(), torch.empty_like(src)
        side = torch.cuda.Stream()
        with torch.cuda.stream(side):
            res = hc.iterate_stencil2d_bnd(kind, hb, b0, b1, 12, fill, stream=side)
        side.synchronize()
        ref = orc.stencil2d_bnd(kind, ob, g, fill, iters=12)
        assert np.array_equal(res.cpu().numpy().view(np.uint64), ref.view(np.uint64)), kind


def test_clamp_boundary_takes_the_tuned_path(hc, orc, dev):
    g = np.random.default_rng(3).uniform(-1, 1, (40, 50))
    src = torch.from_numpy(g).to(dev)
    a, b = torch.empty_like(src), torch.empty_like(src)
    hc.stencil2d_bnd(hc.STENCIL_LAPLACIAN, hc.BOUNDARY_CLAMP, src, a)
    hc.stencil2d(hc.STENCIL_LAPLACIAN, src, b)
    assert torch.equal(a, b)
