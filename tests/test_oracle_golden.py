"""Pin the CPU oracle: reference known answers and the reference's own kernels.

The oracle (oracle/hyd_oracle.c) is the checker for every GPU parity test, so it
is itself checked here against (a) the literal expected values of the
reference's tests/examples and (b) vectors produced by the reference's own C
code (bench/*_ref.c, runtime/hydrangea_runtime.h) stored in tests/golden/.
When the reference witness library can be built (reference tree present) the
same comparisons also run live on fresh random inputs.
"""
import glob
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ka():
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        return json.load(f)


def load(name):
    return np.load(os.path.join(GOLDEN, "witness_%s.npz" % name))


# ---- known answers ------------------------------------------------------------

def test_weighted_histogram_example(orc, ka):
    c = ka["weighted_histogram_example"]
    got = orc.weighted_hist(np.array(c["data"], dtype=np.int64), c["bins"])
    assert got.tolist() == c["expect"]
    got_atomic = orc.weighted_hist(np.array(c["data"], dtype=np.int64), c["bins"], atomic=True)
    assert got_atomic.tolist() == c["expect"]


def test_scatter_cases(orc, ka):
    for c in ka["scatter_tests"]["cases"]:
        assert orc.scatter_add_i64(c["idx"], c["vals"], c["n"]).tolist() == c["expect"]


def test_stencil1d_known(orc, ka):
    for key in ("stencil1d_clamp_box3", "stencil1d_clamp_single"):
        c = ka[key]
        x = np.array(c["input"], dtype=np.int64)
        out = np.empty_like(x)
        orc.lib().orc_stencil1d_box3_i64(x, out, len(x))
        assert out.tolist() == c["expect"]


def test_stencil2d_known(orc, ka):
    c = ka["stencil2d_laplacian_example"]
    out = orc.stencil2d(orc.LAPLACIAN, np.array(c["input"], dtype=np.float64))
    assert out.tolist() == c["expect"]
    c = ka["stencil2d_clamp_corner"]
    g = np.array(c["input"], dtype=np.float64)
    # a+b+c+d at the corner = laplacian + 4*centre
    lap = orc.stencil2d(orc.LAPLACIAN, g)
    assert lap[0, 0] + 4 * g[0, 0] == c["expect_sum4"]


def test_scan_known(orc, ka):
    c = ka["scan_family_1234"]
    x = c["input"]
    assert orc.scan_i64(x).tolist() == c["scan"]
    assert orc.scan_i64(x, inclusive=True).tolist() == c["scan_inclusive"]
    assert orc.scan_i64(x, reverse=True).tolist() == c["scanr"]
    assert orc.scan_i64(x, reverse=True, inclusive=True).tolist() == c["scanr_inclusive"]
    c = ka["scan_prefix_sum_example"]
    assert orc.scan_i64(c["input"]).tolist() == c["expect"]
    assert orc.scan_f64(np.array(c["input"], float)).tolist() == [float(v) for v in c["expect"]]


def test_segmented_reduce_known(orc, ka):
    for key in ("segmented_reduce_test", "segmented_group_sum_example"):
        c = ka[key]
        assert orc.segmented_reduce_i64(c["offsets"], c["vals"]).tolist() == c["expect"]
        f = orc.segmented_reduce_f64(c["offsets"], np.array(c["vals"], float))
        assert f.tolist() == [float(v) for v in c["expect"]]


def test_sort_gather_known(orc, ka):
    c = ka["sort_indices_gather_test"]
    perm = orc.sort_indices(c["keys"])
    assert perm.tolist() == c["perm"]
    vals = np.arange(10, 15, dtype=np.int64)
    assert vals[perm].tolist() == c["sorted_vals"]


def test_coo_csr_known(orc, ka):
    c = ka["coo_csr_test"]
    r, cc, v, k = orc.coo_sum_duplicates(c["rows"], c["cols"], c["vals"])
    assert k == c["canonical_nnz"]
    row_ptr, _, _ = orc.csr_from_sorted_coo(c["nrows"], k, r, cc, v)
    assert row_ptr.tolist() == c["row_ptr"]

    c = ka["coo_to_csr_pipeline_example"]
    rows, cols, vals = (np.array(c[k], dtype=np.int64) for k in ("rows", "cols", "vals"))
    keys = rows * c["ncols"] + cols
    perm = orc.sort_indices(keys)
    assert perm.tolist() == c["perm"]
    r, cc, v, k = orc.coo_sum_duplicates(rows[perm], cols[perm], vals[perm])
    assert k == c["canonical_nnz"]
    row_ptr, col_idx, cv = orc.csr_from_sorted_coo(c["nrows"], k, r, cc, v)
    assert row_ptr.tolist() == c["row_ptr"]
    assert col_idx.tolist() == c["col_idx"]
    assert cv.tolist() == c["csr_vals"]


def test_float_dot_known(orc, ka):
    c = ka["float_dot_test"]
    xs, ys = np.array(c["xs"]), np.array(c["ys"])
    assert orc.dot(xs, ys) == c["expect"]
    assert orc.dot_serial(xs, ys) == c["expect"]
    assert orc.dot_compensated(xs, ys) == c["expect"]


def test_jacobi_1d_known(orc, ka):
    c = ka["jacobi_1d_example"]
    # 1-D stencil on a 1-row grid: the 2-D clamp Jacobi with h = 1 averages
    # 4 values; check the 1-D example's invariant (constant stays constant)
    g = np.ones((1, c["n"]))
    out = orc.iterate_stencil2d(orc.JACOBI, g, c["iters"])
    assert out.reshape(-1).tolist() == c["expect"]


# ---- the reference's own kernels (stored vectors) -------------------------------

def test_sort_matches_reference_runtime(orc):
    for f in sorted(glob.glob(os.path.join(GOLDEN, "witness_sort_*.npz"))):
        z = np.load(f)
        assert np.array_equal(orc.sort_indices(z["keys"]), z["perm"]), f


def test_whist_matches_reference_bench(orc):
    for f in sorted(glob.glob(os.path.join(GOLDEN, "witness_whist_*.npz"))):
        z = np.load(f)
        hist = np.zeros(int(z["bins"]), dtype=np.int64)
        assert orc.lib().orc_hist_generate_i64(int(z["n"]), int(z["bins"]), hist) == 0
        assert np.array_equal(hist, z["hist"]), f


def test_spmv_matches_reference_bench(orc):
    z = load("spmv")
    y = orc.spmv_csr(z["row_ptr"], z["col_idx"], z["vals"], z["x"])
    assert np.array_equal(y, z["y"])  # same sequential order per row: bit-exact


def test_laplacian_matches_reference_bench(orc):
    z = load("laplacian")
    assert np.array_equal(orc.stencil2d(orc.LAPLACIAN, z["grid"]), z["out"])


def test_jacobi_matches_reference_bench(orc):
    z = load("jacobi5")
    assert np.array_equal(orc.iterate_stencil2d(orc.JACOBI, z["grid"], 5), z["out"])


def test_coo_csr_matches_reference_bench(orc):
    z = load("coo_csr")
    nrows, ncols, nnz, dup = (int(z[k]) for k in ("nrows", "ncols", "nnz", "dup"))
    rows, cols, vals = (np.zeros(nnz, dtype=np.int64) for _ in range(3))
    orc.lib().orc_coo_csr_bench_inputs(nrows, ncols, nnz, dup, rows, cols, vals)
    perm = orc.sort_indices(rows * ncols + cols)
    r, c, v, k = orc.coo_sum_duplicates(rows[perm], cols[perm], vals[perm])
    assert k == int(z["count"])
    assert np.array_equal(r[:k], z["rows"]) and np.array_equal(c[:k], z["cols"])
    assert np.array_equal(v[:k], z["vals"])
    row_ptr, _, _ = orc.csr_from_sorted_coo(nrows, k, r, c, v)
    assert np.array_equal(row_ptr, z["row_ptr"])


# ---- live comparisons against the reference kernels (reference tree present) ----

@pytest.fixture(scope="module")
def wit(orc):
    w = orc.witness()
    if w is None:
        pytest.skip("reference witness library not built (reference tree absent)")
    return w


def test_live_sort_random(orc, wit):
    rng = np.random.default_rng(7)
    for n, hi in ((1, 5), (1000, 3), (5000, 1 << 20), (3000, 1 << 62)):
        keys = rng.integers(0, hi, size=n).astype(np.int64)
        perm = np.empty_like(keys)
        wit.wit_sort_indices(keys, n, perm)
        assert np.array_equal(orc.sort_indices(keys), perm)


def test_live_stencils_random(orc, wit):
    rng = np.random.default_rng(8)
    for h, w in ((1, 1), (1, 7), (2, 2), (3, 5), (64, 65)):
        g = rng.uniform(0, 1, size=(h, w))
        out = np.zeros_like(g)
        wit.wit_laplacian(h, w, g.reshape(-1).copy(), out.reshape(-1))
        assert np.array_equal(orc.stencil2d(orc.LAPLACIAN, g), out), (h, w)
        b0, b1 = g.reshape(-1).copy(), np.zeros(h * w)
        which = wit.wit_jacobi(h, w, 3, b0, b1)
        ref = (b0 if which == 0 else b1).reshape(h, w)
        assert np.array_equal(orc.iterate_stencil2d(orc.JACOBI, g, 3), ref), (h, w)


def test_live_whist(orc, wit):
    for n, bins in ((1, 1), (100, 7), (12345, 300), (50000, 65536)):
        a = np.zeros(bins, dtype=np.int64)
        wit.wit_whist(n, bins, a)
        b = np.zeros(bins, dtype=np.int64)
        orc.lib().orc_hist_generate_i64(n, bins, b)
        assert np.array_equal(a, b)


# ---- oracle self-consistency ------------------------------------------------------

def test_generators_deterministic(orc):
    a = orc.uniform_f64(1000, 1, -1.0, 1.0)
    b = orc.uniform_f64(1000, 1, -1.0, 1.0)
    assert np.array_equal(a, b) and a.min() >= -1.0 and a.max() < 1.0
    i = orc.uniform_i64(1000, 2, 1 << 20)
    assert i.min() >= 0 and i.max() < (1 << 20)
    # element i depends only on (seed, i)
    assert np.array_equal(orc.uniform_f64(10, 1, -1.0, 1.0), a[:10])


def test_dot_variants_agree(orc):
    xs = orc.uniform_f64(1 << 16, 1, -1.0, 1.0)
    ys = orc.uniform_f64(1 << 16, 2, -1.0, 1.0)
    ref = orc.dot_compensated(xs, ys)
    assert abs(orc.dot(xs, ys) - ref) <= 1e-12 * abs(ref)
    assert abs(orc.dot_serial(xs, ys) - ref) <= 1e-12 * abs(ref)


def test_hist_privatized_equals_atomic(orc):
    data = orc.uniform_i64(100000, 2, 1 << 20)
    for bins in (1, 64, 4096, 65536, 300000):
        assert np.array_equal(orc.weighted_hist(data, bins), orc.weighted_hist(data, bins, atomic=True))


def test_hist_rejects_negative_routes(orc):
    with pytest.raises(ValueError):
        orc.weighted_hist(np.array([-3, 5], dtype=np.int64), 4)


def test_jacobi_1d_example_and_clamp(orc):
    """examples/jacobi_1d.hyd: three steps over ones stay ones; one step of
    1..5 is the clamped 3-point sums of StencilSpec.hs (4, 6, 9, 12, 14) / 3."""
    import numpy as np
    assert orc.jacobi1d(np.ones(5), 3).tolist() == [1.0] * 5
    assert orc.jacobi1d(np.arange(1.0, 6.0), 1).tolist() == [4.0 / 3.0, 2.0, 3.0, 4.0, 14.0 / 3.0]


def test_gray_scott_fixed_point(orc):
    """U = 1, V = 0 is a fixed point of the Gray-Scott step (no reaction, no
    diffusion), exactly."""
    import numpy as np
    u, v = orc.gray_scott(np.ones((9, 7)), np.zeros((9, 7)), 10)
    assert (u == 1.0).all() and (v == 0.0).all()


def test_stencil_boundaries_known(orc, ka):
    # StencilSpec.hs's clamp / wrap / mirror / constant cases, through the
    # oracle's restatement of the reference's index arithmetic
    modes = {"clamp": orc.CLAMP, "wrap": orc.WRAP, "mirror": orc.MIRROR, "constant": orc.CONST}
    c = ka["stencil_boundaries"]
    for case in c["cases"]:
        out = orc.stencil1d_offsets(case["input"], case["offsets"], modes[case["mode"]], case.get("fill", 0))
        if "expect" in case:
            assert out.tolist() == case["expect"], case["line"]
        else:
            assert int(out.sum()) == case["expect_sum"], case["line"]
    for case in c["cases2d"]:
        out = orc.stencil2d_offsets(case["input"], case["offsets"], modes[case["mode"]], case.get("fill", 0))
        assert out.tolist() == case["expect"], case["line"]


def test_stencil_boundary_forms_agree(orc):
    # the 5-point kinds under `clamp` equal the pinned clamp path; `wrap` and
    # `mirror` read the neighbours the index arithmetic names; mirror on an
    # extent of 1 is refused (the reference divides by zero there)
    rng = np.random.default_rng(17)
    for h, w in ((1, 1), (1, 7), (6, 1), (2, 2), (5, 9)):
        g = rng.uniform(-1, 1, (h, w))
        for kind in (orc.LAPLACIAN, orc.JACOBI, orc.HEAT, orc.HEAT_EXAMPLE):
            assert np.array_equal(orc.stencil2d_bnd(kind, orc.CLAMP, g), orc.stencil2d(kind, g))
    g = np.arange(12, dtype=np.float64).reshape(3, 4)
    lap = orc.stencil2d_bnd(orc.LAPLACIAN, orc.WRAP, g)
    # wrap at (0, 0): up = row 2, left = column 3
    assert lap[0, 0] == g[2, 0] + g[1, 0] + g[0, 3] + g[0, 1] - 4 * g[0, 0]
    lap = orc.stencil2d_bnd(orc.LAPLACIAN, orc.MIRROR, g)
    assert lap[0, 0] == g[1, 0] + g[1, 0] + g[0, 1] + g[0, 1] - 4 * g[0, 0]
    lap = orc.stencil2d_bnd(orc.LAPLACIAN, orc.CONST, g, fill=7.0)
    assert lap[0, 0] == 7.0 + g[1, 0] + 7.0 + g[0, 1] - 4 * g[0, 0]
    with pytest.raises(ValueError):
        orc.stencil2d_bnd(orc.LAPLACIAN, orc.MIRROR, np.zeros((1, 5)))
    assert [orc.lib().orc_bound_index(r, 4, orc.MIRROR) for r in range(-7, 11)] == \
        [1, 0, 1, 2, 3, 2, 1, 0, 1, 2, 3, 2, 1, 0, 1, 2, 3, 2]


def test_reduce_trailing_axis_known(orc, ka):
    c = ka["reduce_trailing_axis_2d"]
    x = np.array(c["input"], dtype=np.int64)
    assert orc.reduce_rows(x, 0, c["init"]).tolist() == c["expect"]
    # the same rows as floats, and (*) with a wrapping int64 product
    assert orc.reduce_rows(x.astype(np.float64), 0, 0.0).tolist() == [3.0, 33.0]
    big = np.array([[1 << 40, 1 << 40]], dtype=np.int64)
    assert orc.reduce_rows(big, 1, 1).tolist() == [0]  # 2^80 wraps to 0


def test_guarded_scatter_skips_unguarded_routes(orc):
    # an unguarded element's index is not read: out of range there is fine
    idx = np.array([0, 5, 1, -7, 1], np.int64)
    vals = np.array([10, 20, 30, 40, 50], np.int64)
    guard = np.array([1, 1, 1, 0, 2], np.int64)
    dst, st = orc.scatter_add_guarded_i64(idx, vals, guard, 6)
    assert st == 0 and dst.tolist() == [10, 80, 0, 0, 0, 20]


def test_map_chain_restatement(orc):
    """bench/map_chain/map_chain.hyd: the program text fixes every element
    (((i/n)^2 - 0.5) * 2 + 1, IEEE operations in order) and the sum has the
    closed form 2/n^2 * (n-1) n (2n-1) / 6."""
    for n in (1, 7, 4096, 100003):
        i = np.arange(n, dtype=np.float64)
        s = i / float(n)
        expect = ((s * s) - 0.5) * 2.0 + 1.0
        got = orc.map_chain(n)
        assert np.array_equal(got.view(np.int64), expect.view(np.int64))
        exact = 2.0 * (n - 1) * n * (2 * n - 1) / 6.0 / float(n) / float(n)
        assert abs(orc.map_chain_sum(n) - exact) <= 1e-12 * max(1.0, exact)
        assert abs(orc.sum_compensated(got) - exact) <= 1e-13 * max(1.0, exact)


def test_zipwith_muladd_restatement(orc):
    rng = np.random.default_rng(5)
    a, b, c = (rng.uniform(-3, 3, 10001) for _ in range(3))
    got = orc.zipwith_muladd(a, b, c)
    assert np.array_equal(got.view(np.int64), (a * b + c).view(np.int64))
    # two roundings, not one: differs from a fused multiply-add somewhere
    fused = np.array([float(np.longdouble(x) * np.longdouble(y) + np.longdouble(z)) for x, y, z in
                      zip(a[:2000], b[:2000], c[:2000])])
    assert not np.array_equal(got[:2000], fused) or np.finfo(np.longdouble).nmant <= 52
