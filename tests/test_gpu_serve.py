"""GPU tests of the resident request server: correctness per kind against the
oracle, the same result alone and in a mix, HBM-budget admission, rejection
and cancellation, and the plain per-call path."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _f64(hc, n, seed, dev):
    t = torch.empty(n, dtype=torch.float64, device=dev)
    hc.fill_uniform_f64(t, seed, -1.0, 1.0)
    return t


def _i64(hc, n, seed, dev):
    t = torch.empty(n, dtype=torch.int64, device=dev)
    hc.fill_uniform_i64(t, seed, 1 << 20)
    return t


class Pool:
    """Device-resident inputs and outputs for a set of requests."""

    def __init__(self, hc, dev):
        self.hc, self.dev, self.keep = hc, dev, []

    def dot(self, n, seed):
        xs, ys = _f64(self.hc, n, seed, self.dev), _f64(self.hc, n, seed + 1, self.dev)
        out = torch.full((1,), float("nan"), dtype=torch.float64, device=self.dev)
        self.keep += [xs, ys, out]
        r = self.hc.Request(self.hc.REQ_DOT, n, 0, xs.data_ptr(), ys.data_ptr(), None, None, out.data_ptr())
        return r, (xs, ys, out)

    def hist(self, n, bins, seed):
        data = _i64(self.hc, n, seed, self.dev)
        out = torch.full((bins,), -1, dtype=torch.int64, device=self.dev)
        self.keep += [data, out]
        return self.hc.Request(self.hc.REQ_HIST, n, bins, data.data_ptr(), None, None, None, out.data_ptr()), (data, out)

    def lap(self, h, w, seed):
        g = torch.empty((h, w), dtype=torch.float64, device=self.dev)
        self.hc.fill_uniform_f64(g, seed, 0.0, 1.0)
        out = torch.full_like(g, float("nan"))
        self.keep += [g, out]
        return self.hc.Request(self.hc.REQ_LAPLACIAN, h, w, g.data_ptr(), None, None, None, out.data_ptr()), (g, out)

    def spmv(self, log2, seed):
        desc, rows, cols, vals, x = self.hc.synth_coo_batch(1, seed0=seed, min_log2=log2, max_log2=log2)
        n, _, nnz = (int(v) for v in desc[0])
        y = torch.zeros(n, dtype=torch.float64, device=self.dev)
        rp = torch.zeros(n + 1, dtype=torch.int64, device=self.dev)
        cc = torch.zeros(max(nnz, 1), dtype=torch.int32, device=self.dev)
        cv = torch.zeros(max(nnz, 1), dtype=torch.float64, device=self.dev)
        self.keep += [rows, cols, vals, x, y, rp, cc, cv]
        r = self.hc.Request(self.hc.REQ_SPMV, n, nnz, rows.data_ptr(), cols.data_ptr(), vals.data_ptr(), x.data_ptr(),
                            y.data_ptr(), rp.data_ptr(), cc.data_ptr(), cv.data_ptr())
        return r, (desc, rows, cols, vals, x, y, rp, cc, cv)


def _mixed(pool):
    reqs = []
    reqs.append(pool.dot(1 << 20, 10))
    reqs.append(pool.hist(300_001, 64, 11))
    reqs.append(pool.lap(257, 300, 12))
    reqs.append(pool.spmv(10, 13))
    reqs.append(pool.dot(4097, 14))
    reqs.append(pool.hist(100_000, 4096, 15))
    reqs.append(pool.lap(64, 64, 16))
    reqs.append(pool.spmv(12, 17))
    reqs.append(pool.dot(0, 18))
    return reqs


def _outputs(kind, bufs):
    if kind == 1:
        return [bufs[2].clone()]
    if kind in (2, 3):
        return [bufs[-1].clone()]
    return [b.clone() for b in bufs[5:]]


def _check_against_oracle(hc, orc, kind, bufs):
    if kind == 1:
        xs, ys, out = bufs
        ref = orc.dot_compensated(xs.cpu().numpy(), ys.cpu().numpy()) if xs.numel() else 0.0
        assert abs(out.item() - ref) <= 1e-12 * max(1.0, abs(ref))
    elif kind == 2:
        data, out = bufs
        assert np.array_equal(out.cpu().numpy(), orc.weighted_hist(data.cpu().numpy(), out.numel()))
    elif kind == 3:
        g, out = bufs
        assert np.array_equal(out.cpu().numpy(), orc.stencil2d(orc.LAPLACIAN, g.cpu().numpy()))
    else:
        desc, rows, cols, vals, x, y, rp, cc, cv = bufs
        n, _, nnz = (int(v) for v in desc[0])
        orp, oci, ocv, oy = orc.coo_to_csr_spmv(n, n, rows.cpu().numpy()[:nnz], cols.cpu().numpy()[:nnz],
                                                 vals.cpu().numpy()[:nnz], x.cpu().numpy())
        assert np.array_equal(rp.cpu().numpy(), orp)
        assert np.array_equal(cc.cpu().numpy()[:nnz], oci) and np.array_equal(cv.cpu().numpy()[:nnz], ocv)
        bound = orc.spmv_csr(orp, oci.astype(np.int64), np.abs(ocv), np.abs(x.cpu().numpy()))
        assert np.all(np.abs(y.cpu().numpy() - oy) <= 1e-12 * np.maximum(bound, 1e-300))


def test_mixed_batch_correct_and_same_alone(hc, orc, dev):
    pool = Pool(hc, dev)
    reqs = _mixed(pool)
    torch.cuda.synchronize()
    srv = hc.Server(streams=2)
    try:
        # each alone (one at a time)
        alone = []
        for r, bufs in reqs:
            st, t = srv.submit(r)
            assert st == hc.OK
            assert srv.wait(t)[0] == hc.OK, srv.error()
            _check_against_oracle(hc, orc, r.kind, bufs)
            alone.append(_outputs(r.kind, bufs))
        # all together (coalesced), outputs reset first
        for r, bufs in reqs:
            if r.kind == 1:
                bufs[2].fill_(float("nan"))
            elif r.kind in (2, 3):
                bufs[-1].fill_(-1 if r.kind == 2 else float("nan"))
            else:
                for b in bufs[5:]:
                    b.zero_()
        torch.cuda.synchronize()
        tickets = [srv.submit(r)[1] for r, _ in reqs]
        for t in tickets:
            assert srv.wait(t)[0] == hc.OK
        for (r, bufs), a in zip(reqs, alone):
            for x, y in zip(_outputs(r.kind, bufs), a):
                assert torch.equal(x, y), r.kind  # bit-identical alone and in the mix
        assert srv.stats().launches < 2 * len(reqs)
    finally:
        srv.close()


def test_plain_path_matches(hc, orc, dev):
    pool = Pool(hc, dev)
    for r, bufs in _mixed(pool):
        hc.check(hc.lib().hyd_cuda_request_run(ctypes.addressof(r), None))
        _check_against_oracle(hc, orc, r.kind, bufs)


def test_budget_admission_and_rejection(hc, dev):
    pool = Pool(hc, dev)
    big, _ = pool.dot(1 << 20, 30)  # 16 MiB working set
    budget = 40 << 20
    srv = hc.Server(budget_bytes=budget, streams=4)
    try:
        tickets = [srv.submit(big)[1] for _ in range(40)]
        for t in tickets:
            assert srv.wait(t)[0] == hc.OK
        s = srv.stats()
        assert 0 < s.peak_inflight_bytes <= budget
        huge, _ = pool.dot(1 << 22, 31)  # 64 MiB > budget
        st, t = srv.submit(huge)
        assert st == hc.ERR_BUDGET and srv.wait(t)[0] == hc.ERR_BUDGET
        bad = hc.Request(hc.REQ_HIST, 10, 0, None, None, None, None, None)
        st, t = srv.submit(bad)
        assert st == hc.ERR_INVALID and srv.wait(t)[0] == hc.ERR_INVALID
        assert srv.stats().rejected == 2
    finally:
        srv.close()


def test_shutdown_cancels_queued(hc, dev):
    pool = Pool(hc, dev)
    big, _ = pool.lap(2048, 2048, 40)  # 64 MiB working set, about 0.5 ms each
    srv = hc.Server(budget_bytes=70 << 20, streams=1, max_batch=1)
    try:
        tickets = [srv.submit(big)[1] for _ in range(50)]
        srv.shutdown()
        sts = [srv.wait(t)[0] for t in tickets]
        assert all(s in (hc.OK, hc.ERR_CANCELLED) for s in sts)
        assert sts.count(hc.ERR_CANCELLED) > 0
        st, t = srv.submit(big)
        assert st == hc.ERR_CANCELLED
    finally:
        srv.close()


def test_trace_drivers(hc, orc, dev):
    # requests in flight together must not share output arrays: one pool each
    pool = Pool(hc, dev)
    reqs = _mixed(pool) + _mixed(pool) + _mixed(pool)
    rq = [r for r, _ in reqs]
    arr = np.cumsum(np.full(len(rq), 50e-6))
    lat_p, st_p, el_p = hc.plain_trace(rq, arr)
    assert (st_p == 0).all() and el_p > 0
    srv = hc.Server(streams=4)
    try:
        lat_s, st_s, el_s = srv.trace(rq, arr)
    finally:
        srv.close()
    assert (st_s == 0).all() and (lat_s > 0).all() and el_s > 0
    for r, bufs in reqs:
        _check_against_oracle(hc, orc, r.kind, bufs)
