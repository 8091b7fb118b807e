"""GPU parity: coo_sum_duplicates / csr_from_sorted_coo (bit-exact), SpMV
(within 1e-12 of sum |v*x|), and the batched COO -> CSR -> SpMV pipeline
(CSR bit-exact per instance, y within tolerance) against the oracle."""
import json
import os

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _t(a, dev, dtype=torch.int64):
    return torch.tensor(np.asarray(a), dtype=dtype, device=dev)


def test_known_answers(hc, dev):
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        ka = json.load(f)
    c = ka["coo_csr_test"]
    r, cc, v, k = hc.coo_sum_duplicates(_t(c["rows"], dev), _t(c["cols"], dev), _t(c["vals"], dev))
    assert int(k.item()) == c["canonical_nnz"]
    row_ptr, _, _ = hc.csr_from_sorted_coo(c["nrows"], int(k.item()), r, cc, v)
    assert row_ptr.cpu().tolist() == c["row_ptr"]
    # full pipeline of examples/coo_to_csr_pipeline.hyd on the GPU
    c = ka["coo_to_csr_pipeline_example"]
    rows, cols, vals = (_t(c[k2], dev) for k2 in ("rows", "cols", "vals"))
    keys = rows * c["ncols"] + cols
    perm = torch.empty_like(keys)
    hc.sort_indices(keys, perm)
    assert perm.cpu().tolist() == c["perm"]
    sr, sc, sv = (torch.empty_like(rows) for _ in range(3))
    hc.gather(perm, rows, sr)
    hc.gather(perm, cols, sc)
    hc.gather(perm, vals, sv)
    r, cc, v, k = hc.coo_sum_duplicates(sr, sc, sv)
    assert int(k.item()) == c["canonical_nnz"]
    row_ptr, col_idx, cv = hc.csr_from_sorted_coo(c["nrows"], int(k.item()), r, cc, v)
    assert row_ptr.cpu().tolist() == c["row_ptr"]
    assert col_idx.cpu().tolist() == c["col_idx"]
    assert cv.cpu().tolist() == c["csr_vals"]


def test_reference_coo_csr_bench(hc, orc, dev):
    z = np.load(os.path.join(GOLDEN, "witness_coo_csr.npz"))
    nrows, ncols, nnz, dup = (int(z[k]) for k in ("nrows", "ncols", "nnz", "dup"))
    rows, cols, vals = (np.zeros(nnz, dtype=np.int64) for _ in range(3))
    orc.lib().orc_coo_csr_bench_inputs(nrows, ncols, nnz, dup, rows, cols, vals)
    keys = torch.from_numpy(rows * ncols + cols).to(dev)
    perm = torch.empty_like(keys)
    hc.sort_indices(keys, perm)
    sr, sc, sv = (torch.empty_like(keys) for _ in range(3))
    for src, dst in ((rows, sr), (cols, sc), (vals, sv)):
        hc.gather(perm, torch.from_numpy(src).to(dev), dst)
    r, c, v, k = hc.coo_sum_duplicates(sr, sc, sv)
    k = int(k.item())
    assert k == int(z["count"])
    assert np.array_equal(r.cpu().numpy()[:k], z["rows"]) and np.array_equal(c.cpu().numpy()[:k], z["cols"])
    assert np.array_equal(v.cpu().numpy()[:k], z["vals"])
    assert not r.cpu().numpy()[k:].any()
    row_ptr, _, _ = hc.csr_from_sorted_coo(nrows, k, r, c, v)
    assert np.array_equal(row_ptr.cpu().numpy(), z["row_ptr"])


@pytest.mark.parametrize("nnz,nrows,ncols", [(1, 1, 1), (1000, 50, 40), (200_000, 3000, 5000)])
def test_random_dedup_and_csr(hc, orc, dev, nnz, nrows, ncols):
    rng = np.random.default_rng(nnz)
    rows = np.sort(rng.integers(0, nrows, size=nnz))
    cols = rng.integers(0, max(ncols // 50, 1), size=nnz)
    order = np.lexsort((cols, rows))
    rows, cols = rows[order].astype(np.int64), cols[order].astype(np.int64)
    vals = rng.integers(-(1 << 40), 1 << 40, size=nnz).astype(np.int64)
    r, c, v, k = hc.coo_sum_duplicates(_t(rows, dev), _t(cols, dev), _t(vals, dev))
    orr, oc, ov, ok = orc.coo_sum_duplicates(rows, cols, vals)
    assert int(k.item()) == ok
    assert np.array_equal(r.cpu().numpy(), orr) and np.array_equal(c.cpu().numpy(), oc)
    assert np.array_equal(v.cpu().numpy(), ov)
    rp, ci, cv = hc.csr_from_sorted_coo(nrows, ok, r, c, v)
    orp, oci, ocv = orc.csr_from_sorted_coo(nrows, ok, orr, oc, ov)
    assert np.array_equal(rp.cpu().numpy(), orp)
    assert np.array_equal(ci.cpu().numpy(), oci) and np.array_equal(cv.cpu().numpy(), ocv)


def test_csr_bad_row_reported(hc, dev):
    hc.csr_from_sorted_coo(2, 3, _t([0, 1, 5], dev), _t([0, 0, 0], dev), _t([1, 1, 1], dev))
    assert hc.device_check() == hc.ERR_BOUNDS


@pytest.mark.parametrize("lanes", [0, 1, 4, 32])
def test_spmv_reference_bench(hc, orc, dev, lanes):
    z = np.load(os.path.join(GOLDEN, "witness_spmv.npz"))
    y = torch.zeros(len(z["row_ptr"]) - 1, dtype=torch.float64, device=dev)
    hc.spmv_csr(_t(z["row_ptr"], dev), _t(z["col_idx"], dev), _t(z["vals"], dev, torch.float64),
                _t(z["x"], dev, torch.float64), y, lanes_per_row=lanes)
    bound = orc.spmv_csr(z["row_ptr"], z["col_idx"], np.abs(z["vals"]), np.abs(z["x"]))
    assert np.all(np.abs(y.cpu().numpy() - z["y"]) <= 1e-12 * np.maximum(bound, 1e-300))


def _check_batch(hc, orc, desc, rows, cols, vals, x, row_ptr, csr_cols, csr_vals, y):
    h_rows, h_cols, h_vals, h_x = (t.cpu().numpy() for t in (rows, cols, vals, x))
    h_rp, h_cc, h_cv, h_y = (t.cpu().numpy() for t in (row_ptr, csr_cols, csr_vals, y))
    e0 = xr = yr = rp0 = 0  # entries, x (by ncols), y (by nrows), row_ptr (by nrows + 1)
    for n, ncols, nnz in desc:
        sl = slice(e0, e0 + nnz)
        rp, ci, cv, yy = orc.coo_to_csr_spmv(n, ncols, h_rows[sl], h_cols[sl], h_vals[sl], h_x[xr:xr + ncols])
        assert np.array_equal(h_rp[rp0:rp0 + n + 1], rp)
        assert np.array_equal(h_cc[sl], ci) and np.array_equal(h_cv[sl], cv)
        bound = orc.spmv_csr(rp, ci.astype(np.int64), np.abs(cv), np.abs(h_x[xr:xr + ncols]))
        assert np.all(np.abs(h_y[yr:yr + n] - yy) <= 1e-12 * np.maximum(bound, 1e-300))
        e0 += nnz
        xr += ncols
        yr += n
        rp0 += n + 1


def test_synth_batch_properties(hc, dev):
    desc, rows, cols, vals, x = hc.synth_coo_batch(6, seed0=4, min_log2=8, max_log2=12)
    desc2, rows2, cols2, vals2, x2 = hc.synth_coo_batch(6, seed0=4, min_log2=8, max_log2=12)
    assert np.array_equal(desc, desc2) and torch.equal(rows, rows2) and torch.equal(vals, vals2)
    h_r, h_c = rows.cpu().numpy(), cols.cpu().numpy()
    e0 = 0
    for n, _, nnz in desc:
        r, c = h_r[e0:e0 + nnz].astype(np.int64), h_c[e0:e0 + nnz].astype(np.int64)
        assert r.min() >= 0 and r.max() < n and c.min() >= 0 and c.max() < n
        assert len(np.unique(r * n + c)) == nnz  # no duplicate (row, col)
        assert np.bincount(r, minlength=n).max() <= 256
        e0 += nnz


@pytest.mark.parametrize("ninst,lo,hi", [(1, 6, 6), (7, 8, 12), (24, 10, 14)])
def test_batched_pipeline(hc, orc, dev, ninst, lo, hi):
    desc, rows, cols, vals, x = hc.synth_coo_batch(ninst, seed0=100 + ninst, min_log2=lo, max_log2=hi,
                                                   max_row_len=min(256, 1 << lo))
    out = hc.batched_coo_csr_spmv(desc, rows, cols, vals, x)
    hc.check(hc.device_check())
    _check_batch(hc, orc, desc, rows, cols, vals, x, *out)
    # result is the same alone and in the batch
    alone = hc.synth_coo_batch(ninst, seed0=100 + ninst, min_log2=lo, max_log2=hi, max_row_len=min(256, 1 << lo))
    out2 = hc.batched_coo_csr_spmv(*alone)
    for a, b in zip(out, out2):
        assert torch.equal(a, b)


def test_batched_workload_instances_subset(hc, orc, dev):
    """A slice of the workload's 512-instance batch (seed 4 + i, n in 2^10..2^18)."""
    desc, rows, cols, vals, x = hc.synth_coo_batch(8, seed0=4, min_log2=10, max_log2=18)
    out = hc.batched_coo_csr_spmv(desc, rows, cols, vals, x)
    hc.check(hc.device_check())
    _check_batch(hc, orc, desc, rows, cols, vals, x, *out)


def test_batched_full_workload_512_instances(hc, orc, dev):
    """The whole batched workload: 512 instances (seed 4 + i, n = 2^U(10,18),
    Zipf(1.5) row lengths capped at 256, about 2.9e8 entries) in one batched
    call, every instance's row_ptr, col_idx and vals bit-exact against the
    oracle's stable-sort COO -> CSR and y within 1e-12 * sum |v * x| of its
    sequential row sums."""
    desc, rows, cols, vals, x = hc.synth_coo_batch(512, seed0=4, min_log2=10, max_log2=18, max_row_len=256)
    out = hc.batched_coo_csr_spmv(desc, rows, cols, vals, x)
    hc.check(hc.device_check())
    assert int(desc[:, 2].sum()) > 2 * 10**8
    _check_batch(hc, orc, desc, rows, cols, vals, x, *out)


def test_bucketed_and_row_atomic_forms_agree(hc, orc, dev, monkeypatch):
    """Both internal forms of the batched pipeline give identical CSR and y."""
    desc, rows, cols, vals, x = hc.synth_coo_batch(12, seed0=321, min_log2=10, max_log2=15)
    monkeypatch.setenv("HYD_CUDA_BATCH_PIPELINE", "rows")
    a = hc.batched_coo_csr_spmv(desc, rows, cols, vals, x)
    monkeypatch.delenv("HYD_CUDA_BATCH_PIPELINE")
    b = hc.batched_coo_csr_spmv(desc, rows, cols, vals, x)
    hc.check(hc.device_check())
    for u, v in zip(a, b):
        assert torch.equal(u, v)
    _check_batch(hc, orc, desc, rows, cols, vals, x, *b)


@pytest.mark.parametrize("pipeline", ["bucketed", "rows"])
def test_batched_pipeline_duplicates_keep_coo_order(hc, orc, dev, pipeline, monkeypatch):
    """Equal (row, col) entries keep their COO order in the CSR (the runtime's
    stable sort_indices), in small buckets and in buckets above 2048 entries."""
    if pipeline == "rows":
        monkeypatch.setenv("HYD_CUDA_BATCH_PIPELINE", "rows")
    rng = np.random.default_rng(41)
    descs, R, Cc, V, X = [], [], [], [], []
    for n, nnz, ncols, dense in ((50, 400, 7, False), (300, 5000, 300, False), (64, 9000, 40, True),
                                 (1, 200, 3, False), (4096, 30000, 4096, False)):
        if dense:  # 64 rows x up to 256 entries: one bucket above the fast kernel's 2048
            r = np.repeat(np.arange(n), nnz // n)[:nnz]
            nnz = len(r)
        else:
            r = rng.integers(0, n, nnz)
        c = rng.integers(0, ncols, nnz)  # few columns: many duplicate (row, col)
        descs.append((n, ncols, nnz))
        R.append(r); Cc.append(c); V.append(rng.uniform(-1, 1, nnz)); X.append(rng.uniform(-1, 1, ncols))
    desc = np.array(descs, dtype=np.int64)
    rows = torch.from_numpy(np.concatenate(R).astype(np.int32)).to(dev)
    cols = torch.from_numpy(np.concatenate(Cc).astype(np.int32)).to(dev)
    vals = torch.from_numpy(np.concatenate(V)).to(dev)
    x = torch.from_numpy(np.concatenate(X)).to(dev)
    out = hc.batched_coo_csr_spmv(desc, rows, cols, vals, x)
    hc.check(hc.device_check())
    _check_batch(hc, orc, desc, rows, cols, vals, x, *out)


def test_batched_pipeline_column_widths(hc, orc, dev):
    """Column counts that give the bucket sort one, two and three 8-bit passes
    (ncols 1 .. 2^18), and wider instances (ncols 2^18 + 1, 2^20) whose
    buckets go to the block-wide kernel, in one batch."""
    rng = np.random.default_rng(59)
    descs, R, Cc, V, X = [], [], [], [], []
    for n, ncols, nnz in ((70, 1, 60), (130, 4, 700), (90, 5, 900), (200, 256, 4000), (150, 257, 3000),
                          (3000, 1 << 18, 40000), (2000, (1 << 18) + 1, 30000), (1000, 1 << 20, 20000)):
        r = rng.integers(0, n, nnz)
        c = rng.integers(0, ncols, nnz)
        descs.append((n, ncols, nnz))
        R.append(r); Cc.append(c); V.append(rng.uniform(-1, 1, nnz)); X.append(rng.uniform(-1, 1, ncols))
    desc = np.array(descs, dtype=np.int64)
    rows = torch.from_numpy(np.concatenate(R).astype(np.int32)).to(dev)
    cols = torch.from_numpy(np.concatenate(Cc).astype(np.int32)).to(dev)
    vals = torch.from_numpy(np.concatenate(V)).to(dev)
    x = torch.from_numpy(np.concatenate(X)).to(dev)
    out = hc.batched_coo_csr_spmv(desc, rows, cols, vals, x)
    hc.check(hc.device_check())
    _check_batch(hc, orc, desc, rows, cols, vals, x, *out)


@pytest.mark.parametrize("pipeline", ["bucketed", "rows"])
@pytest.mark.parametrize("bad", ["row", "col"])
def test_batched_out_of_range_entry_reported(hc, orc, dev, pipeline, bad, monkeypatch):
    if pipeline == "rows":
        monkeypatch.setenv("HYD_CUDA_BATCH_PIPELINE", "rows")
    desc, rows, cols, vals, x = hc.synth_coo_batch(3, seed0=77, min_log2=8, max_log2=10)
    if bad == "row":
        rows[5] = int(desc[0, 0])       # one past the first instance's last row
    else:
        cols[7] = -1
    hc.batched_coo_csr_spmv(desc, rows, cols, vals, x)
    assert hc.device_check() == hc.ERR_BOUNDS
    assert hc.device_check() == hc.OK


@pytest.mark.parametrize("pipeline", ["bucketed", "rows"])
def test_batched_row_above_256_entries_reported(hc, orc, dev, pipeline, monkeypatch):
    """A row with more than 256 entries is outside the batched pipeline's
    contract: both forms report it through hyd_cuda_check, and the device
    stays usable for the next call."""
    if pipeline == "rows":
        monkeypatch.setenv("HYD_CUDA_BATCH_PIPELINE", "rows")
    rng = np.random.default_rng(17)
    n, ncols, long_len = 200, 4096, 300
    r = np.concatenate([np.full(long_len, 7), rng.integers(0, n, 2000)])
    c = np.concatenate([rng.permutation(ncols)[:long_len], rng.integers(0, ncols, 2000)])
    desc = np.array([(n, ncols, len(r))], dtype=np.int64)
    rows = torch.from_numpy(r.astype(np.int32)).to(dev)
    cols = torch.from_numpy(c.astype(np.int32)).to(dev)
    vals = torch.from_numpy(rng.uniform(-1, 1, len(r))).to(dev)
    x = torch.from_numpy(rng.uniform(-1, 1, ncols)).to(dev)
    hc.batched_coo_csr_spmv(desc, rows, cols, vals, x)
    assert hc.device_check() == hc.ERR_BOUNDS
    assert hc.device_check() == hc.OK
    # a batch within the contract right after gives the oracle's results
    desc2, rows2, cols2, vals2, x2 = hc.synth_coo_batch(2, seed0=11, min_log2=8, max_log2=10)
    out = hc.batched_coo_csr_spmv(desc2, rows2, cols2, vals2, x2)
    hc.check(hc.device_check())
    _check_batch(hc, orc, desc2, rows2, cols2, vals2, x2, *out)
