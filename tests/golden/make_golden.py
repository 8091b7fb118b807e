"""Generate the committed golden fixtures in this directory.

Two kinds of fixture:

* ``known_answers.json`` -- the literal expected values of the reference's own
  tests and examples for this path, worked out by hand from the program text
  (the reference's interpreter, which produced them there, cannot run here).
  Each entry names its source file:line in hydrangea-compiler.
* ``witness_*.npz`` -- inputs and outputs of the reference's own C kernels
  (``bench/*_ref.c`` and ``runtime/hydrangea_runtime.h``), compiled from the
  reference tree by ``oracle/build.py`` and run here through
  ``oracle/_ref/libhyd_refwitness.so``.  The reference tree is not available
  where the GPU tests run, so the vectors are stored.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def known_answers():
    ka = {}
    ka["weighted_histogram_example"] = {
        "source": "examples/weighted_histogram.hyd:13-25",
        "data": list(range(1024)), "bins": 64,
        "expect": [sum((k + 64 * j) ** 2 for j in range(16)) for k in range(64)],
    }
    ka["stencil1d_clamp_box3"] = {
        "source": "test/Language/Hydrangea/StencilSpec.hs:26-34",
        "input": [1, 2, 3, 4, 5], "expect": [4, 6, 9, 12, 14],
    }
    ka["stencil1d_clamp_single"] = {
        "source": "test/Language/Hydrangea/StencilSpec.hs:54-58",
        "input": [42], "expect": [126],
    }
    # the boundary conditions of StencilSpec.hs: arrays, offsets, expected
    # outputs (generate [4] (i + 1) is [1, 2, 3, 4])
    ka["stencil_boundaries"] = {
        "source": "test/Language/Hydrangea/StencilSpec.hs:37-148, :185-190",
        "cases": [
            {"line": 37, "mode": "clamp", "input": [0, 2, 4, 6], "offsets": [0], "expect": [0, 2, 4, 6]},
            {"line": 43, "mode": "clamp", "input": [10, 11, 12], "offsets": [-5], "expect": [10, 10, 10]},
            {"line": 50, "mode": "clamp", "input": [10, 11, 12], "offsets": [5], "expect": [12, 12, 12]},
            {"line": 74, "mode": "wrap", "input": [1, 2, 3, 4], "offsets": [-1], "expect": [4, 1, 2, 3]},
            {"line": 83, "mode": "wrap", "input": [1, 2, 3, 4], "offsets": [1], "expect": [2, 3, 4, 1]},
            {"line": 91, "mode": "wrap", "input": [1, 2, 3, 4], "offsets": [-1, 0, 1], "expect_sum": 30},
            {"line": 103, "mode": "mirror", "input": [1, 2, 3, 4], "offsets": [-1], "expect": [2, 1, 2, 3]},
            {"line": 114, "mode": "mirror", "input": [1, 2, 3, 4], "offsets": [1], "expect": [2, 3, 4, 3]},
            {"line": 126, "mode": "constant", "fill": 0, "input": [1, 2, 3], "offsets": [-1, 0, 1],
             "expect": [3, 6, 5]},
            {"line": 136, "mode": "constant", "fill": -1, "input": [10, 10, 10], "offsets": [-1],
             "expect": [-1, 10, 10]},
            {"line": 143, "mode": "constant", "fill": 99, "input": [0, 0], "offsets": [-5], "expect": [99, 99]},
        ],
        "cases2d": [
            {"line": 161, "mode": "clamp", "input": [[1, 2, 3], [4, 5, 6]], "offsets": [[0, 1]],
             "expect": [[2, 3, 3], [5, 6, 6]]},
            {"line": 185, "mode": "constant", "fill": 0, "input": [[1, 1], [1, 1]], "offsets": [[-1, 0]],
             "expect": [[0, 0], [1, 1]]},
        ],
    }
    # reduce over the trailing axis of generate [2,3] (i*10 + j)
    ka["reduce_trailing_axis_2d"] = {
        "source": "test/Language/Hydrangea/InterpreterSpec.hs:337-342",
        "input": [[0, 1, 2], [10, 11, 12]], "init": 0, "expect": [3, 33],
    }
    ka["stencil2d_clamp_corner"] = {
        "source": "test/Language/Hydrangea/StencilSpec.hs:171-179",
        "input": [[1, 2, 3], [4, 5, 6], [7, 8, 9]], "index": [0, 0], "expect_sum4": 8,
    }
    # examples/stencil_2d.hyd: clamp Laplacian of [[1,2,3],[4,5,6],[7,8,9]];
    # every output worked out from a+b+c+d-4e with clamped neighbours.
    ka["stencil2d_laplacian_example"] = {
        "source": "examples/stencil_2d.hyd:1-18",
        "input": [[1, 2, 3], [4, 5, 6], [7, 8, 9]],
        "expect": [[4, 3, 2], [1, 0, -1], [-2, -3, -4]],
    }
    ka["scan_family_1234"] = {
        "source": "test/Language/Hydrangea/EndToEndSpec.hs:804-826",
        "input": [1, 2, 3, 4],
        "scan": [0, 1, 3, 6], "scan_inclusive": [1, 3, 6, 10],
        "scanr": [9, 7, 4, 0], "scanr_inclusive": [10, 9, 7, 4],
    }
    ka["scan_prefix_sum_example"] = {
        "source": "examples/scan_prefix_sum.hyd:1-3",
        "input": [1, 2, 3, 4, 5, 6], "expect": [0, 1, 3, 6, 10, 15],
    }
    ka["segmented_reduce_test"] = {
        "source": "test/Language/Hydrangea/EndToEndSpec.hs:828-840",
        "offsets": [0, 2, 5, 5], "vals": [1, 2, 10, 20, 30], "expect": [3, 60, 0],
    }
    ka["segmented_group_sum_example"] = {
        "source": "examples/segmented_group_sum.hyd:1-21",
        "offsets": [0, 2, 5, 5, 7], "vals": [1, 2, 10, 20, 30, 7, 8], "expect": [3, 60, 0, 15],
    }
    ka["sort_indices_gather_test"] = {
        "source": "test/Language/Hydrangea/EndToEndSpec.hs:842-854",
        "keys": [3, 1, 3, 2, 1], "perm": [1, 4, 3, 0, 2], "sorted_vals": [11, 14, 13, 10, 12],
    }
    ka["coo_csr_test"] = {
        "source": "test/Language/Hydrangea/EndToEndSpec.hs:856-880",
        "nrows": 3, "ncols": 4,
        "rows": [0, 0, 1, 1, 2, 2], "cols": [1, 1, 0, 2, 0, 0], "vals": [1, 2, 10, 12, 20, 21],
        "canonical_nnz": 4, "row_ptr": [0, 1, 3, 4],
    }
    ka["coo_to_csr_pipeline_example"] = {
        "source": "examples/coo_to_csr_pipeline.hyd:1-76",
        "nrows": 3, "ncols": 4,
        "rows": [2, 0, 1, 0, 2, 1, 1, 0], "cols": [1, 3, 0, 1, 0, 2, 2, 1],
        "vals": [21, 3, 10, 1, 20, 12, 5, 4],
        "perm": [3, 7, 1, 2, 5, 6, 4, 0],
        "canonical_nnz": 6, "row_ptr": [0, 2, 4, 6],
        "col_idx": [1, 3, 0, 2, 0, 1, 0, 0], "csr_vals": [5, 3, 10, 17, 20, 21, 0, 0],
    }
    ka["float_dot_test"] = {
        "source": "test/Language/Hydrangea/EndToEndSpec.hs:991-996",
        "xs": [1.0, 2.0, 3.0, 4.0], "ys": [1.0, 2.0, 3.0, 4.0], "expect": 30.0,
    }
    ka["jacobi_1d_example"] = {
        "source": "examples/jacobi_1d.hyd:1-6",
        "n": 5, "iters": 3, "expect": [1.0] * 5,
    }
    ka["scatter_tests"] = {
        "source": "test/Language/Hydrangea/EndToEndSpec.hs:579-640",
        "cases": [
            {"idx": [0, 1, 2], "vals": [10, 11, 12], "n": 3, "expect": [10, 11, 12]},
            {"idx": [0, 0, 1, 1], "vals": [1, 1, 1, 1], "n": 2, "expect": [2, 2]},
            {"idx": [0, 0, 0, 0, 0], "vals": [1, 1, 1, 1, 1], "n": 1, "expect": [5]},
            {"idx": [0, 0, 1, 1], "vals": [0, 3, 6, 9], "n": 2, "expect": [3, 15]},
            {"idx": [0, 0, 1, 1, 2, 2, 3, 3], "vals": [1, 4, 7, 10, 13, 16, 19, 22], "n": 4,
             "expect": [5, 17, 29, 41]},
        ],
    }
    return ka


def witness_fixtures(W):
    rng = np.random.default_rng(20261203)
    out = {}
    # sort_indices (runtime radix sort), with ties, zeros and a wide key range
    for name, keys in {
        "small_range": rng.integers(0, 17, size=997),
        "wide": rng.integers(0, 1 << 40, size=1500),
        "zeros": np.zeros(64, dtype=np.int64),
    }.items():
        keys = np.ascontiguousarray(keys, dtype=np.int64)
        perm = np.empty_like(keys)
        W.wit_sort_indices(keys, len(keys), perm)
        out["sort_" + name] = {"keys": keys, "perm": perm}
    # weighted_histogram_ref.c (generate-bucket histogram)
    for n, bins in ((10007, 64), (10007, 1000), (4096, 4096)):
        hist = np.zeros(bins, dtype=np.int64)
        W.wit_whist(n, bins, hist)
        out["whist_%d_%d" % (n, bins)] = {"n": np.int64(n), "bins": np.int64(bins), "hist": hist}
    # spmv_ref.c
    nrows, ncols = 211, 173
    lens = rng.integers(0, 9, size=nrows)
    row_ptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    nnz = int(row_ptr[-1])
    col_idx = rng.integers(0, ncols, size=nnz).astype(np.int64)
    vals = rng.uniform(-1, 1, size=nnz)
    x = rng.uniform(-1, 1, size=ncols)
    y = np.zeros(nrows)
    W.wit_spmv(nrows, ncols, nnz, vals, col_idx, row_ptr, x, y)
    out["spmv"] = {"row_ptr": row_ptr, "col_idx": col_idx, "vals": vals, "x": x, "y": y}
    # stencil_ref.c (one clamp Laplacian sweep)
    h, w = 37, 53
    grid = rng.uniform(0, 1, size=(h, w))
    lap = np.zeros_like(grid)
    W.wit_laplacian(h, w, grid.reshape(-1).copy(), lap.reshape(-1))
    out["laplacian"] = {"grid": grid, "out": lap}
    # jacobi_2d_ref.c (clamp Jacobi, 5 sweeps)
    h, w = 19, 23
    grid = rng.uniform(0, 1, size=(h, w))
    b0 = grid.reshape(-1).copy()
    b1 = np.zeros_like(b0)
    which = W.wit_jacobi(h, w, 5, b0, b1)
    out["jacobi5"] = {"grid": grid, "out": (b0 if which == 0 else b1).reshape(h, w)}
    # coo_csr_build_ref.c
    nrows, ncols, nnz, dup = 50, 40, 1000, 3
    row_ptr = np.zeros(nrows + 1, dtype=np.int64)
    cr, cc, cv = (np.zeros(nnz, dtype=np.int64) for _ in range(3))
    cnt = W.wit_coo_csr(nrows, ncols, nnz, dup, row_ptr, cr, cc, cv)
    out["coo_csr"] = {"nrows": np.int64(nrows), "ncols": np.int64(ncols), "nnz": np.int64(nnz),
                      "dup": np.int64(dup), "count": np.int64(cnt), "row_ptr": row_ptr,
                      "rows": cr[:cnt], "cols": cc[:cnt], "vals": cv[:cnt]}
    return out


def main():
    with open(os.path.join(HERE, "known_answers.json"), "w") as f:
        json.dump(known_answers(), f, indent=1)
    W = O.witness()
    if W is None:
        raise SystemExit("reference witness library unavailable; known answers written only")
    for name, arrays in witness_fixtures(W).items():
        np.savez_compressed(os.path.join(HERE, "witness_%s.npz" % name), **arrays)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
