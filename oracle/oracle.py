"""ctypes binding of the CPU oracle (test infrastructure only).

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, always as the checker.  The product library
(``libhyd_cuda.so``) never calls into it.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
_ref = None

_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64 = C.c_int64
_u64 = C.c_uint64

LAPLACIAN, JACOBI, HEAT, HEAT_EXAMPLE = 0, 1, 2, 3
# stencil boundary conditions (Syntax.hs:416-426)
CLAMP, WRAP, MIRROR, CONST = 0, 1, 2, 3


def lib():
    """Load (building if needed) libhyd_oracle.so."""
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        sig = {
            "orc_rand_u64": (_u64, [_u64, _u64]),
            "orc_fill_uniform_f64": (None, [_f64p, _i64, _u64, C.c_double, C.c_double]),
            "orc_fill_uniform_i64": (None, [_i64p, _i64, _u64, _i64]),
            "orc_dot_f64": (C.c_double, [_f64p, _f64p, _i64]),
            "orc_dot_f64_serial": (C.c_double, [_f64p, _f64p, _i64]),
            "orc_dot_f64_compensated": (C.c_double, [_f64p, _f64p, _i64]),
            "orc_sum_f64_compensated": (C.c_double, [_f64p, _i64]),
            "orc_map_chain_f64": (None, [_i64, _f64p]),
            "orc_map_chain_sum_f64": (C.c_double, [_i64]),
            "orc_zipwith_muladd_f64": (None, [_f64p, _f64p, _f64p, _f64p, _i64]),
            "orc_weighted_hist_i64": (C.c_int, [_i64p, _i64, _i64, _i64p]),
            "orc_weighted_hist_i64_atomic": (C.c_int, [_i64p, _i64, _i64, _i64p]),
            "orc_hist_generate_i64": (C.c_int, [_i64, _i64, _i64p]),
            "orc_scatter_add_i64": (C.c_int, [_i64p, _i64p, _i64, _i64p, _i64]),
            "orc_scatter_add_f64": (C.c_int, [_i64p, _f64p, _i64, _f64p, _i64]),
            "orc_stencil2d_f64": (None, [C.c_int, _f64p, _f64p, _i64, _i64]),
            "orc_iterate_stencil2d_f64": (C.c_int, [C.c_int, _f64p, _f64p, _i64, _i64, _i64]),
            "orc_stencil1d_box3_i64": (None, [_i64p, _i64p, _i64]),
            "orc_bound_index": (_i64, [_i64, _i64, C.c_int]),
            "orc_reduce_rows_i64": (None, [_i64p, _i64, _i64, C.c_int, _i64, _i64p]),
            "orc_reduce_rows_f64": (None, [_f64p, _i64, _i64, C.c_int, C.c_double, _f64p]),
            "orc_scatter_add_guarded_i64": (C.c_int, [_i64p, _i64p, _i64p, _i64, _i64p, _i64]),
            "orc_stencil1d_offsets_i64": (C.c_int, [_i64p, _i64p, _i64, _i64p, C.c_int, C.c_int, _i64]),
            "orc_stencil2d_offsets_i64": (C.c_int, [_i64p, _i64p, _i64, _i64, _i64p, C.c_int, C.c_int, _i64]),
            "orc_stencil2d_bnd_f64": (C.c_int, [C.c_int, C.c_int, C.c_double, _f64p, _f64p, _i64, _i64]),
            "orc_iterate_stencil2d_bnd_f64": (C.c_int, [C.c_int, C.c_int, C.c_double, _f64p, _f64p, _i64, _i64,
                                                        _i64]),
            "orc_stencil1d_jacobi3_f64": (None, [_f64p, _f64p, _i64]),
            "orc_iterate_stencil1d_jacobi3_f64": (C.c_int, [_f64p, _f64p, _i64, _i64]),
            "orc_gray_scott_step_f64": (None, [_f64p, _f64p, _f64p, _f64p, _i64, _i64, C.c_double, C.c_double,
                                                C.c_double, C.c_double, C.c_double]),
            "orc_scan_i64": (None, [_i64p, _i64p, _i64, _i64, C.c_int, C.c_int]),
            "orc_scan_f64": (None, [_f64p, _f64p, _i64, C.c_double, C.c_int, C.c_int]),
            "orc_segmented_reduce_i64": (C.c_int, [_i64p, _i64, _i64p, _i64, _i64, _i64p]),
            "orc_segmented_reduce_f64": (C.c_int, [_i64p, _i64, _f64p, _i64, C.c_double, _f64p]),
            "orc_sort_indices_i64": (None, [_i64p, _i64, _i64p]),
            "orc_gather_i64": (None, [_i64p, _i64, _i64p, _i64p]),
            "orc_gather_f64": (None, [_i64p, _i64, _f64p, _f64p]),
            "orc_coo_sum_duplicates_i64": (_i64, [_i64p, _i64p, _i64p, _i64, _i64p, _i64p, _i64p]),
            "orc_csr_from_sorted_coo_i64": (C.c_int, [_i64, _i64, _i64p, _i64p, _i64p, _i64p, _i64p, _i64p]),
            "orc_spmv_csr_f64": (None, [_i64, _i64p, _i64p, _f64p, _f64p, _f64p]),
            "orc_coo_to_csr_spmv_f64": (C.c_int, [_i64, _i64, _i64, _i32p, _i32p, _f64p, _f64p,
                                                   _i64p, _i32p, _f64p, _f64p]),
            "orc_coo_csr_bench_inputs": (None, [_i64, _i64, _i64, _i64, _i64p, _i64p, _i64p]),
            "orc_max_threads": (C.c_int, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def witness():
    """The reference's own kernels (oracle/_ref), or None when not built."""
    global _ref
    if _ref is None:
        path = _build.REF_SO
        if not os.path.exists(path):
            try:
                path = _build.build_reference_witness()
            except RuntimeError:
                path = None
        if not path or not os.path.exists(path):
            return None
        W = C.CDLL(path)
        sig = {
            "wit_sort_indices": (None, [_i64p, _i64, _i64p]),
            "wit_read_array_csv": (None, [C.c_char_p, _i64, _i64p]),
            "wit_read_float_array_csv": (None, [C.c_char_p, _i64, _f64p]),
            "wit_write_array_csv": (_i64, [_i64p, C.c_int, _i64, _i64, C.c_char_p]),
            "wit_write_array_csv_float": (_i64, [_f64p, C.c_int, _i64, _i64, C.c_char_p]),
            "wit_nd_to_flat2": (_i64, [_i64, _i64, _i64, _i64]),
            "wit_whist": (None, [_i64, _i64, _i64p]),
            "wit_spmv": (None, [_i64, _i64, _i64, _f64p, _i64p, _i64p, _f64p, _f64p]),
            "wit_laplacian": (None, [C.c_int, C.c_int, _f64p, _f64p]),
            "wit_jacobi": (C.c_int, [C.c_int, C.c_int, C.c_int, _f64p, _f64p]),
            "wit_coo_csr": (_i64, [_i64, _i64, _i64, _i64, _i64p, _i64p, _i64p, _i64p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(W, name)
            fn.restype = res
            fn.argtypes = args
        _ref = W
    return _ref


# ---- numpy-level helpers ----------------------------------------------------

def uniform_f64(n, seed, lo, hi):
    out = np.empty(n, dtype=np.float64)
    lib().orc_fill_uniform_f64(out, n, seed, lo, hi)
    return out


def uniform_i64(n, seed, bound):
    out = np.empty(n, dtype=np.int64)
    lib().orc_fill_uniform_i64(out, n, seed, bound)
    return out


def dot(xs, ys):
    return lib().orc_dot_f64(np.ascontiguousarray(xs), np.ascontiguousarray(ys), len(xs))


def dot_serial(xs, ys):
    return lib().orc_dot_f64_serial(np.ascontiguousarray(xs), np.ascontiguousarray(ys), len(xs))


def dot_compensated(xs, ys):
    return lib().orc_dot_f64_compensated(np.ascontiguousarray(xs), np.ascontiguousarray(ys), len(xs))


def sum_compensated(xs):
    return lib().orc_sum_f64_compensated(np.ascontiguousarray(xs, dtype=np.float64), len(xs))


def map_chain(n):
    """Elements of bench/map_chain/map_chain.hyd's fused chain."""
    out = np.empty(n, dtype=np.float64)
    lib().orc_map_chain_f64(n, out)
    return out


def map_chain_sum(n):
    """The same chain reduced by the C backend's reduction template."""
    return lib().orc_map_chain_sum_f64(n)


def zipwith_muladd(a, b, c):
    """zipwith (+.) (zipwith ( *. ) a b) c, fused: a*b + c elementwise."""
    a, b, c = (np.ascontiguousarray(t, dtype=np.float64) for t in (a, b, c))
    out = np.empty(len(a), dtype=np.float64)
    lib().orc_zipwith_muladd_f64(a, b, c, out, len(a))
    return out


def weighted_hist(data, bins, atomic=False):
    hist = np.zeros(bins, dtype=np.int64)
    fn = lib().orc_weighted_hist_i64_atomic if atomic else lib().orc_weighted_hist_i64
    rc = fn(np.ascontiguousarray(data, dtype=np.int64), len(data), bins, hist)
    if rc != 0:
        raise ValueError("weighted histogram route out of bounds (rc=%d)" % rc)
    return hist


def scatter_add_i64(idx, vals, dst_n):
    dst = np.zeros(dst_n, dtype=np.int64)
    rc = lib().orc_scatter_add_i64(np.ascontiguousarray(idx, dtype=np.int64),
                                   np.ascontiguousarray(vals, dtype=np.int64), len(idx), dst, dst_n)
    if rc != 0:
        raise ValueError("scatter route out of bounds")
    return dst


def stencil2d(kind, grid):
    grid = np.ascontiguousarray(grid, dtype=np.float64)
    h, w = grid.shape
    out = np.empty_like(grid)
    lib().orc_stencil2d_f64(kind, grid.reshape(-1), out.reshape(-1), h, w)
    return out


def iterate_stencil2d(kind, grid, iters):
    b0 = np.ascontiguousarray(grid, dtype=np.float64).copy()
    b1 = np.empty_like(b0)
    h, w = b0.shape
    which = lib().orc_iterate_stencil2d_f64(kind, b0.reshape(-1), b1.reshape(-1), h, w, iters)
    return b0 if which == 0 else b1


def reduce_rows(x, op, init):
    """`reduce` (op 0: +, 1: *) over the trailing axis of a 2-D array, serially."""
    rows, cols = x.shape
    if x.dtype == np.float64:
        out = np.empty(rows, np.float64)
        lib().orc_reduce_rows_f64(np.ascontiguousarray(x).reshape(-1), rows, cols, op, float(init), out)
    else:
        out = np.empty(rows, np.int64)
        lib().orc_reduce_rows_i64(np.ascontiguousarray(x, dtype=np.int64).reshape(-1), rows, cols, op, int(init),
                                  out)
    return out


def scatter_add_guarded_i64(idx, vals, guard, dst_n):
    dst = np.zeros(dst_n, np.int64)
    st = lib().orc_scatter_add_guarded_i64(np.ascontiguousarray(idx, dtype=np.int64),
                                           np.ascontiguousarray(vals, dtype=np.int64),
                                           np.ascontiguousarray(guard, dtype=np.int64), len(idx), dst, dst_n)
    return dst, st


def stencil1d_offsets(x, offsets, mode, fill=0):
    """Sum of `acc d` over `offsets` under a boundary condition (int64)."""
    x = np.ascontiguousarray(x, dtype=np.int64)
    out = np.empty_like(x)
    offs = np.ascontiguousarray(offsets, dtype=np.int64)
    if lib().orc_stencil1d_offsets_i64(x, out, len(x), offs, len(offs), mode, fill) != 0:
        raise ValueError("mirror boundary on an extent of 1")
    return out


def stencil2d_offsets(grid, offsets, mode, fill=0):
    """2-D form; `offsets` is a list of (d0, d1) pairs."""
    grid = np.ascontiguousarray(grid, dtype=np.int64)
    h, w = grid.shape
    out = np.empty_like(grid)
    offs = np.ascontiguousarray(np.array(offsets, dtype=np.int64).reshape(-1))
    if lib().orc_stencil2d_offsets_i64(grid.reshape(-1), out.reshape(-1), h, w, offs, len(offs) // 2, mode,
                                        fill) != 0:
        raise ValueError("mirror boundary on an extent of 1")
    return out


def stencil2d_bnd(kind, mode, grid, fill=0.0, iters=1):
    """`iters` steps of a 5-point kind under a boundary condition."""
    b0 = np.ascontiguousarray(grid, dtype=np.float64).copy()
    b1 = np.empty_like(b0)
    h, w = b0.shape
    which = lib().orc_iterate_stencil2d_bnd_f64(kind, mode, fill, b0.reshape(-1), b1.reshape(-1), h, w, iters)
    if which < 0:
        raise ValueError("mirror boundary on an extent of 1")
    return b0 if which == 0 else b1


def jacobi1d(x, iters=1):
    """iters clamped 3-point Jacobi steps (examples/jacobi_1d.hyd)."""
    b0 = np.ascontiguousarray(x, dtype=np.float64).copy()
    b1 = np.empty_like(b0)
    which = lib().orc_iterate_stencil1d_jacobi3_f64(b0, b1, len(b0), iters)
    return b0 if which == 0 else b1


# demo/gray_scott/gray_scott.hyd:19-25
GRAY_SCOTT = dict(du=0.21, dv=0.105, feed=0.0545, kill=0.0620, dt=1.0)


def gray_scott(u, v, steps=1, du=0.21, dv=0.105, feed=0.0545, kill=0.0620, dt=1.0):
    u = np.ascontiguousarray(u, dtype=np.float64).copy()
    v = np.ascontiguousarray(v, dtype=np.float64).copy()
    h, w = u.shape
    un, vn = np.empty_like(u), np.empty_like(v)
    for _ in range(steps):
        lib().orc_gray_scott_step_f64(u.reshape(-1), v.reshape(-1), un.reshape(-1), vn.reshape(-1), h, w,
                                      du, dv, feed, kill, dt)
        u, un = un, u
        v, vn = vn, v
    return u, v


def scan_i64(x, init=0, reverse=False, inclusive=False):
    x = np.ascontiguousarray(x, dtype=np.int64)
    out = np.empty_like(x)
    lib().orc_scan_i64(x, out, len(x), init, int(reverse), int(inclusive))
    return out


def scan_f64(x, init=0.0, reverse=False, inclusive=False):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    lib().orc_scan_f64(x, out, len(x), init, int(reverse), int(inclusive))
    return out


def segmented_reduce_i64(offsets, vals, init=0):
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    vals = np.ascontiguousarray(vals, dtype=np.int64)
    out = np.zeros(max(len(offsets) - 1, 0), dtype=np.int64)
    if lib().orc_segmented_reduce_i64(offsets, len(offsets), vals, len(vals), init, out) != 0:
        raise ValueError("bad offsets")
    return out


def segmented_reduce_f64(offsets, vals, init=0.0):
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    out = np.zeros(max(len(offsets) - 1, 0), dtype=np.float64)
    if lib().orc_segmented_reduce_f64(offsets, len(offsets), vals, len(vals), init, out) != 0:
        raise ValueError("bad offsets")
    return out


def sort_indices(keys):
    keys = np.ascontiguousarray(keys, dtype=np.int64)
    perm = np.empty_like(keys)
    lib().orc_sort_indices_i64(keys, len(keys), perm)
    return perm


def coo_sum_duplicates(rows, cols, vals):
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    vals = np.ascontiguousarray(vals, dtype=np.int64)
    n = len(rows)
    o_r, o_c, o_v = (np.zeros(n, dtype=np.int64) for _ in range(3))
    k = lib().orc_coo_sum_duplicates_i64(rows, cols, vals, n, o_r, o_c, o_v)
    return o_r, o_c, o_v, k


def csr_from_sorted_coo(nrows, nnz, rows, cols, vals):
    row_ptr = np.zeros(nrows + 1, dtype=np.int64)
    col_idx = np.zeros(len(cols), dtype=np.int64)
    o_v = np.zeros(len(vals), dtype=np.int64)
    rc = lib().orc_csr_from_sorted_coo_i64(nrows, nnz, np.ascontiguousarray(rows, dtype=np.int64),
                                           np.ascontiguousarray(cols, dtype=np.int64),
                                           np.ascontiguousarray(vals, dtype=np.int64),
                                           row_ptr, col_idx, o_v)
    if rc != 0:
        raise ValueError("row out of range")
    return row_ptr, col_idx, o_v


def spmv_csr(row_ptr, col_idx, vals, x):
    nrows = len(row_ptr) - 1
    y = np.zeros(nrows, dtype=np.float64)
    lib().orc_spmv_csr_f64(nrows, np.ascontiguousarray(row_ptr, dtype=np.int64),
                           np.ascontiguousarray(col_idx, dtype=np.int64),
                           np.ascontiguousarray(vals, dtype=np.float64),
                           np.ascontiguousarray(x, dtype=np.float64), y)
    return y


def coo_to_csr_spmv(nrows, ncols, rows, cols, vals, x):
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    nnz = len(rows)
    row_ptr = np.zeros(nrows + 1, dtype=np.int64)
    col_idx = np.zeros(nnz, dtype=np.int32)
    cvals = np.zeros(nnz, dtype=np.float64)
    y = np.zeros(nrows, dtype=np.float64)
    rc = lib().orc_coo_to_csr_spmv_f64(nrows, ncols, nnz, rows, cols, vals, x, row_ptr, col_idx, cvals, y)
    if rc != 0:
        raise ValueError("COO entry out of range (rc=%d)" % rc)
    return row_ptr, col_idx, cvals, y
