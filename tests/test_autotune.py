"""Autotuner: the on-disk choice table (CPU) and tuning runs (GPU)."""
import os
import tempfile

import numpy as np
import pytest


def test_table_record_query_and_persistence(hc):
    L = hc.lib()
    path = os.path.join(tempfile.mkdtemp(prefix="hyd_tune_t_"), "sub", "t.tsv")
    assert L.hyd_cuda_tune_set_cache_path(path.encode()) == 0
    assert L.hyd_cuda_tune_query(b"devA", b"stencil2d", b"k2_h13_w13") == -1
    assert L.hyd_cuda_tune_record(b"devA", b"stencil2d", b"k2_h13_w13", 3, 123.5) == 0
    assert L.hyd_cuda_tune_record(b"devB", b"stencil2d", b"k2_h13_w13", 1, 99.0) == 0
    assert L.hyd_cuda_tune_query(b"devA", b"stencil2d", b"k2_h13_w13") == 3
    # a later record for the same key wins, also after reloading from disk
    assert L.hyd_cuda_tune_record(b"devA", b"stencil2d", b"k2_h13_w13", 5, 80.0) == 0
    assert L.hyd_cuda_tune_set_cache_path(path.encode()) == 0
    assert L.hyd_cuda_tune_query(b"devA", b"stencil2d", b"k2_h13_w13") == 5
    assert L.hyd_cuda_tune_query(b"devB", b"stencil2d", b"k2_h13_w13") == 1
    lines = open(path).read().strip().splitlines()
    assert len(lines) == 3 and lines[0].split("\t")[:3] == ["devA", "stencil2d", "k2_h13_w13"]
    assert L.hyd_cuda_tune_record(b"devA", None, b"x", 1, 1.0) == hc.ERR_INVALID
    # restore the session cache path
    L.hyd_cuda_tune_set_cache_path(os.environ["HYD_CUDA_TUNE_CACHE"].encode())


@pytest.mark.gpu
@pytest.mark.parametrize("variant", list(range(21)))
def test_every_stencil_variant_bit_exact(hc, orc, dev, variant):
    import torch
    for (h, w) in ((37, 130), (256, 512), (1000, 2050)):
        g = torch.empty((h, w), dtype=torch.float64, device=dev)
        hc.fill_uniform_f64(g, 5, 0.0, 1.0)
        out = torch.full_like(g, float("nan"))
        hc.stencil2d(hc.STENCIL_HEAT, g, out, variant=variant)
        assert np.array_equal(out.cpu().numpy(), orc.stencil2d(orc.HEAT, g.cpu().numpy())), (variant, h, w)


@pytest.mark.gpu
@pytest.mark.parametrize("variant", [1, 6, 8, 13, 15, 20])
@pytest.mark.parametrize("kind", ["LAPLACIAN", "JACOBI", "HEAT", "HEAT_EXAMPLE"])
def test_integer_pipe_variants_every_kind_and_sign(hc, orc, dev, variant, kind):
    """Mixed signs, zeros, subnormals and huge values take the FP64 fallback
    inside the integer-pipe sums; every kind stays bit-identical."""
    import torch
    rng = np.random.default_rng(7)
    h, w = 129, 260
    a = rng.uniform(-1.0, 1.0, (h, w))
    a[::7, ::5] = 0.0
    a[3::11, 2::13] = 5e-324 * rng.integers(1, 1000, a[3::11, 2::13].shape)
    a[5::17, 1::9] = 1.7e308
    a[::3, 4::7] = np.abs(a[::3, 4::7])
    g = torch.from_numpy(a).to(dev)
    out = torch.full_like(g, float("nan"))
    hc.stencil2d(getattr(hc, "STENCIL_" + kind), g, out, variant=variant)
    ref = orc.stencil2d(getattr(orc, kind), a)
    assert np.array_equal(out.cpu().numpy().view(np.int64), ref.view(np.int64)), (variant, kind)


@pytest.mark.gpu
def test_autotune_stencil_records_choice(hc, dev):
    best, times = hc.autotune_stencil2d(hc.STENCIL_HEAT, 1024, 1024, reps=3)
    assert 0 <= best < 21 and (times > 0).all()
    assert times[best] == times.min()
    assert hc.lib().hyd_cuda_tune_query(None, b"stencil2d", b"k2_h10_w10") == best


@pytest.mark.gpu
def test_autotune_histogram_records_choice(hc, orc, dev):
    import torch
    best, times = hc.autotune_histogram(1 << 20, 4096, reps=3)
    assert best in (1, 2, 3, 4, 5)
    assert hc.lib().hyd_cuda_tune_query(None, b"weighted_histogram", b"b12") == best
    # the AUTO path now uses the tuned strategy and stays bit-exact
    data = torch.empty(100_000, dtype=torch.int64, device=dev)
    hc.fill_uniform_i64(data, 3, 1 << 20)
    hist = torch.zeros(4096, dtype=torch.int64, device=dev)
    hc.weighted_histogram(data, hist)
    assert np.array_equal(hist.cpu().numpy(), orc.weighted_hist(data.cpu().numpy(), 4096))
