"""Python mirror of the libhyd_cuda.so C ABI (include/hyd_cuda.h).

This is the host-side binding the tests and ``bench.py`` use.  It calls the
C entry points through ctypes with plain pointers; device buffers are torch
CUDA tensors (torch is only the allocator/stream plumbing here) and streams are
passed as their raw ``cudaStream_t``.  There is no CPU fallback: if the
library is missing, importing this module raises.
"""
import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhyd_cuda.so")
HEADER_DIR = os.path.join(os.path.dirname(HERE), "include")

OK = 0
ERR_INVALID, ERR_NOMEM, ERR_CUDA, ERR_NO_DEVICE, ERR_BOUNDS = 1, 2, 3, 4, 5
ERR_TIMEOUT, ERR_BUDGET, ERR_CANCELLED, ERR_UNSUPPORTED = 6, 7, 8, 9

STENCIL_LAPLACIAN, STENCIL_JACOBI, STENCIL_HEAT, STENCIL_HEAT_EXAMPLE = 0, 1, 2, 3
SCATTER_AUTO, SCATTER_SMEM_WARP, SCATTER_SMEM_BLOCK, SCATTER_CLUSTER, SCATTER_GLOBAL, SCATTER_PARTITION = 0, 1, 2, 3, 4, 5

_p = C.c_void_p
_i64 = C.c_int64
_u64 = C.c_uint64
_d = C.c_double
_i = C.c_int

# name -> (restype, argtypes); every function declared in include/*.h that the
# Python side calls is listed here.
SIGNATURES = {
    "hyd_cuda_init": (_i, []),
    "hyd_cuda_cleanup": (None, []),
    "hyd_cuda_last_error": (C.c_char_p, []),
    "hyd_cuda_status_string": (C.c_char_p, [_i]),
    "hyd_cuda_version": (_i, []),
    "hyd_cuda_device_sm_count": (_i, []),
    "hyd_cuda_check": (_i, [_p]),
    "hyd_cuda_fill_uniform_f64": (_i, [_p, _i64, _u64, _d, _d, _p]),
    "hyd_cuda_fill_uniform_i64": (_i, [_p, _i64, _u64, _i64, _p]),
    "hyd_cuda_dot_f64": (_i, [_p, _p, _i64, _p, _p]),
    "hyd_cuda_sum_f64": (_i, [_p, _i64, _p, _p]),
    "hyd_cuda_dot_f64_noalloc": (_i, [_p, _p, _i64, _p, _p]),
    "hyd_cuda_weighted_histogram_i64": (_i, [_p, _i64, _i64, _p, _i, _p]),
    "hyd_cuda_weighted_histogram_plan": (_i, [_i64, _i64, _i, _p, _p]),
    "hyd_cuda_scatter_add_i64": (_i, [_p, _p, _i64, _p, _i64, _i, _p]),
    "hyd_cuda_scatter_add_f64": (_i, [_p, _p, _i64, _p, _i64, _p]),
    "hyd_cuda_stencil2d_f64": (_i, [_i, _p, _p, _i64, _i64, _p]),
    "hyd_cuda_iterate_stencil2d_f64": (_i, [_i, _p, _p, _i64, _i64, _i64, C.POINTER(C.c_int), _p]),
    "hyd_cuda_stencil2d_bnd_f64": (_i, [_i, _i, C.c_double, _p, _p, _i64, _i64, _p]),
    "hyd_cuda_iterate_stencil2d_bnd_f64": (_i, [_i, _i, C.c_double, _p, _p, _i64, _i64, _i64, C.POINTER(C.c_int),
                                               _p]),
    "hyd_cuda_stencil_release_graphs": (None, []),
    "hyd_cuda_stencil2d_f64_variant": (_i, [_i, _p, _p, _i64, _i64, _i, _p]),
    "hyd_cuda_selftest_dadd": (_i, [_p, _p, _p, _p, _i64, _p]),
    "hyd_cuda_selftest_div": (_i, [_p, _i, _p, _p, _i64, _p]),
    "hyd_cuda_probe_fp64_rate": (_i, [_i64, _p, C.POINTER(C.c_int64), _p]),
    "hyd_cuda_selftest_timeout": (_i, [_i, C.c_uint32, _p]),
    "hyd_cuda_iterate_stencil2d_f64_variant": (_i, [_i, _p, _p, _i64, _i64, _i64, _i, C.POINTER(C.c_int), _p]),
    "hyd_cuda_tune_cache_path": (C.c_char_p, []),
    "hyd_cuda_tune_set_cache_path": (_i, [C.c_char_p]),
    "hyd_cuda_tune_record": (_i, [C.c_char_p, C.c_char_p, C.c_char_p, _i, _d]),
    "hyd_cuda_tune_query": (_i, [C.c_char_p, C.c_char_p, C.c_char_p]),
    "hyd_cuda_autotune_stencil2d": (_i, [_i, _i64, _i64, _i, C.POINTER(C.c_int), _p]),
    "hyd_cuda_autotune_histogram": (_i, [_i64, _i64, _i, C.POINTER(C.c_int), _p]),
    "hyd_cuda_scan_i64": (_i, [_p, _p, _i64, _i64, _i, _i, _p]),
    "hyd_cuda_scan_f64": (_i, [_p, _p, _i64, _d, _i, _i, _p]),
    "hyd_cuda_segmented_reduce_i64": (_i, [_p, _i64, _p, _i64, _i64, _p, _p]),
    "hyd_cuda_segmented_reduce_f64": (_i, [_p, _i64, _p, _i64, _d, _p, _p]),
    "hyd_cuda_sort_indices_i64": (_i, [_p, _i64, _p, _p]),
    "hyd_cuda_sort_indices_bits_i64": (_i, [_p, _i64, _i, _p, _p]),
    "hyd_cuda_gather_i64": (_i, [_p, _i64, _p, _i64, _p, _p]),
    "hyd_cuda_gather_f64": (_i, [_p, _i64, _p, _i64, _p, _p]),
    "hyd_cuda_gather_i32": (_i, [_p, _i64, _p, _i64, _p, _p]),
    "hyd_cuda_coo_sum_duplicates_i64": (_i, [_p, _p, _p, _i64, _p, _p, _p, _p, _p]),
    "hyd_cuda_csr_from_sorted_coo_i64": (_i, [_i64, _i64, _p, _p, _p, _p, _p, _p, _p]),
    "hyd_cuda_spmv_csr_f64": (_i, [_i64, _i64, _p, _p, _p, _p, _p, _i, _p]),
    "hyd_cuda_spmv_csr_i32_f64": (_i, [_i64, _i64, _p, _p, _p, _p, _p, _i, _p]),
    "hyd_cuda_batched_coo_csr_spmv_f64": (_i, [_i64, _p, _p, _p, _p, _p, _p, _p, _p, _p, _p]),
    "hyd_cuda_synth_coo_batch": (_i, [_i64, _u64, _i, _i, _i, _p, _p, _p, _p, _p, _i64, _p]),
    "hyd_cuda_server_create": (_i, [_p, C.POINTER(C.c_void_p)]),
    "hyd_cuda_server_submit": (_i, [_p, _p, C.POINTER(C.c_int64)]),
    "hyd_cuda_server_wait": (_i, [_p, _i64, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "hyd_cuda_server_stats": (_i, [_p, _p]),
    "hyd_cuda_server_shutdown": (_i, [_p]),
    "hyd_cuda_server_error": (C.c_char_p, [_p]),
    "hyd_cuda_server_destroy": (_i, [_p]),
    "hyd_cuda_request_run": (_i, [_p, _p]),
    "hyd_cuda_serve_trace": (_i, [_p, _p, _p, _i64, _p, _p, C.POINTER(C.c_double)]),
    "hyd_cuda_plain_trace": (_i, [_p, _p, _i64, _p, _p, C.POINTER(C.c_double), _p]),
    "hyd_cuda_weighted_histogram_host": (_i, [_p, _i64, _i64, _p, _i]),
    "hyd_cuda_dot_f64_host": (_i, [_p, _p, _i64, _p]),
    "hyd_cuda_array_alloc": (_p, [None, C.c_size_t]),
    "hyd_export_weighted_histogram": (_p, [_p, _i64]),
    "hyd_export_dot": (_d, [_p, _p]),
    "hyd_export_gray_scott": (_p, []),
    "hyd_cuda_read_array_csv": (_p, [C.c_char_p, None]),
    "hyd_cuda_read_float_array_csv": (_p, [C.c_char_p, None]),
    "hyd_cuda_write_array_csv": (_i64, [_p, C.c_char_p]),
    "hyd_cuda_write_array_csv_float": (_i64, [_p, C.c_char_p]),
    "hyd_cuda_read_csv_i64_to_device": (_i, [C.c_char_p, _i64, _p, _p]),
    "hyd_cuda_read_csv_f64_to_device": (_i, [C.c_char_p, _i64, _p, _p]),
    "hyd_cuda_write_csv_i64_from_device": (_i, [_p, None, C.c_char_p, _p]),
    "hyd_cuda_write_csv_f64_from_device": (_i, [_p, None, C.c_char_p, _p]),
    "hyd_cuda_scatter_add_guarded_i64": (_i, [_p, _p, _p, _i64, _p, _i64, _i, _p]),
    "hyd_cuda_reduce_rows_i64": (_i, [_p, _i64, _i64, _i, _i64, _p, _p]),
    "hyd_cuda_reduce_rows_f64": (_i, [_p, _i64, _i64, _i, C.c_double, _p, _p]),
    "hyd_cuda_array_attach": (_i, [_p]),
    "hyd_cuda_array_host_modified": (_i, [_p]),
    "hyd_cuda_array_detach": (_i, [_p]),
    "hyd_cuda_array_device_data": (_p, [_p]),
    "hyd_cuda_array_resident_stats": (_i, [_p, _p, _p]),
    "hyd_cuda_map_f64": (_i, [C.c_char_p, _p, _i, _i64, _p, _p, _p]),
    "hyd_cuda_map_i64": (_i, [C.c_char_p, _p, _i, _i64, _p, _p, _p]),
    "hyd_cuda_gen_check": (None, [_i, C.c_char_p]),
    "hyd_cuda_gen_alloc": (_p, [_i64]),
    "hyd_cuda_gen_free": (None, [_p]),
    "hyd_cuda_gen_zero": (None, [_p, _i64]),
    "hyd_cuda_gen_upload": (_p, [_p]),
    "hyd_cuda_gen_download": (_p, [_p, None, C.c_size_t]),
    "hyd_cuda_gen_read_i64": (_i64, [_p]),
    "hyd_cuda_gen_read_f64": (_d, [_p]),
    "hyd_cuda_gen_array_free": (None, [_p]),
    "hyd_cuda_gen_get_env_int": (_i64, [C.c_char_p]),
    "hyd_cuda_gen_print_int": (None, [_i64]),
    "hyd_cuda_gen_print_double": (None, [_d]),
    "hyd_cuda_gen_print_array": (None, [_p]),
    "hyd_cuda_gen_print_float_array": (None, [_p]),
    "hyd_cuda_jacobi1d_f64": (_i, [_p, _p, _i64, _p]),
    "hyd_cuda_iterate_jacobi1d_f64": (_i, [_p, _p, _i64, _i64, C.POINTER(C.c_int), _p]),
    "hyd_cuda_gray_scott_step_f64": (_i, [_p, _p, _p, _p, _i64, _i64, _p, _p]),
    "hyd_cuda_iterate_gray_scott_f64": (_i, [_p, _p, _p, _p, _i64, _i64, _p, _i64, C.POINTER(C.c_int), _p]),
}


class Tuple(C.Structure):
    """hyd_tuple_t (runtime/hydrangea_runtime.h:220-223)."""
    _fields_ = [("elems", C.c_int64 * 8), ("ndims", C.c_int)]


class Storage(C.Structure):
    _fields_ = [("data", C.c_void_p), ("refcount", C.c_int64)]


class Array(C.Structure):
    """hyd_array_t (runtime/hydrangea_runtime.h:230-235)."""
    _fields_ = [("storage", C.POINTER(Storage)), ("data", C.c_void_p), ("elem_size", C.c_size_t),
                ("shape", Tuple)]


REQ_DOT, REQ_HIST, REQ_LAPLACIAN, REQ_SPMV = 1, 2, 3, 4


class Request(C.Structure):
    """hyd_request_t."""
    _fields_ = [("kind", C.c_int), ("n", C.c_int64), ("m", C.c_int64),
                ("in0", C.c_void_p), ("in1", C.c_void_p), ("in2", C.c_void_p), ("in3", C.c_void_p),
                ("out0", C.c_void_p), ("out1", C.c_void_p), ("out2", C.c_void_p), ("out3", C.c_void_p)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("streams", C.c_int), ("max_batch", C.c_int),
                ("max_batch_bytes", C.c_int64)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("rejected", C.c_int64), ("cancelled", C.c_int64), ("launches", C.c_int64),
                ("peak_inflight_bytes", C.c_int64), ("inflight_bytes", C.c_int64), ("queued", C.c_int64)]


class HydCudaError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("hyd_cuda status %d: %s" % (status, msg))
        self.status = status


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libhyd_cuda.so is not built (run __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            args = [Tuple if a is None else a for a in args]
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def header_functions():
    """Names of all functions declared in include/*.h."""
    names = []
    for f in sorted(os.listdir(HEADER_DIR)):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(HEADER_DIR, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b(hyd_[A-Za-z0-9_]+)\s*\(", text):
            if m.group(1) not in names:
                names.append(m.group(1))
    return names


def last_error():
    return (lib().hyd_cuda_last_error() or b"").decode()


def check(status):
    if status != OK:
        raise HydCudaError(status, last_error())
    return status


def ptr(t):
    """Raw device pointer of a torch tensor (or an int pointer)."""
    if t is None:
        return None
    if isinstance(t, int):
        return t
    return t.data_ptr()


def stream_handle(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def call(name, *args):
    return check(getattr(lib(), name)(*args))


# ---- convenience wrappers over torch tensors -----------------------------------

def fill_uniform_f64(out, seed, lo, hi, stream=None):
    call("hyd_cuda_fill_uniform_f64", ptr(out), out.numel(), seed, lo, hi, stream_handle(stream))


def fill_uniform_i64(out, seed, bound, stream=None):
    call("hyd_cuda_fill_uniform_i64", ptr(out), out.numel(), seed, bound, stream_handle(stream))


def dot_f64(xs, ys, out, stream=None):
    call("hyd_cuda_dot_f64", ptr(xs), ptr(ys), xs.numel(), ptr(out), stream_handle(stream))


def sum_f64(xs, out, stream=None):
    call("hyd_cuda_sum_f64", ptr(xs), xs.numel(), ptr(out), stream_handle(stream))


def weighted_histogram(data, hist, strategy=SCATTER_AUTO, stream=None):
    call("hyd_cuda_weighted_histogram_i64", ptr(data), data.numel(), hist.numel(), ptr(hist),
         strategy, stream_handle(stream))


def weighted_histogram_plan(n, bins, strategy=SCATTER_AUTO):
    """(strategy a call of this shape runs, kernels it launches)."""
    chosen, launches = C.c_int(0), C.c_int(0)
    call("hyd_cuda_weighted_histogram_plan", n, bins, strategy, C.byref(chosen), C.byref(launches))
    return chosen.value, launches.value


STRATEGY_NAMES = {0: "AUTO", 1: "SMEM_WARP", 2: "SMEM_BLOCK", 3: "CLUSTER", 4: "GLOBAL", 5: "PARTITION"}


def scatter_add_i64(idx, vals, dst, strategy=SCATTER_AUTO, stream=None):
    call("hyd_cuda_scatter_add_i64", ptr(idx), ptr(vals), idx.numel(), ptr(dst), dst.numel(),
         strategy, stream_handle(stream))


def scatter_add_f64(idx, vals, dst, stream=None):
    call("hyd_cuda_scatter_add_f64", ptr(idx), ptr(vals), idx.numel(), ptr(dst), dst.numel(),
         stream_handle(stream))


_STENCIL_SHAPES = [(32, 32), (16, 128), (16, 64), (32, 64), (8, 128), (32, 128), "plain"]
_STENCIL_EMU = [0, 2, 3]  # sum additions on the integer pipe, per level
STENCIL_VARIANTS = {s + 7 * l: (_STENCIL_SHAPES[s] if l == 0 else (_STENCIL_SHAPES[s], "int-add x%d" % _STENCIL_EMU[l]))
                    for l in range(3) for s in range(7)}


def stencil2d(kind, src, dst, stream=None, variant=-1):
    h, w = src.shape
    call("hyd_cuda_stencil2d_f64_variant", kind, ptr(src), ptr(dst), h, w, variant, stream_handle(stream))


def iterate_stencil2d(kind, buf0, buf1, iters, stream=None, variant=-1):
    """Runs `iters` steps ping-ponging buf0/buf1; returns the buffer holding the result."""
    h, w = buf0.shape
    fb = C.c_int(-1)
    call("hyd_cuda_iterate_stencil2d_f64_variant", kind, ptr(buf0), ptr(buf1), h, w, iters, variant,
         C.byref(fb), stream_handle(stream))
    return buf0 if fb.value == 0 else buf1


BOUNDARY_CLAMP, BOUNDARY_WRAP, BOUNDARY_MIRROR, BOUNDARY_CONSTANT = 0, 1, 2, 3
REDOP_ADD, REDOP_MUL = 0, 1


def reduce_rows(x, op, init, out, stream=None):
    """`reduce` over the trailing axis of a 2-D device tensor into `out` (rows,)."""
    rows, cols = x.shape
    if x.dtype.is_floating_point:
        call("hyd_cuda_reduce_rows_f64", ptr(x), rows, cols, op, float(init), ptr(out), stream_handle(stream))
    else:
        call("hyd_cuda_reduce_rows_i64", ptr(x), rows, cols, op, int(init), ptr(out), stream_handle(stream))


def scatter_add_guarded_i64(idx, vals, guard, dst, strategy=SCATTER_AUTO, stream=None):
    call("hyd_cuda_scatter_add_guarded_i64", ptr(idx), ptr(vals), ptr(guard), idx.numel(), ptr(dst), dst.numel(),
         strategy, stream_handle(stream))


def stencil2d_bnd(kind, boundary, src, dst, fill=0.0, stream=None):
    """One step of a 5-point kind under a boundary condition."""
    h, w = src.shape
    call("hyd_cuda_stencil2d_bnd_f64", kind, boundary, fill, ptr(src), ptr(dst), h, w, stream_handle(stream))


def iterate_stencil2d_bnd(kind, boundary, buf0, buf1, iters, fill=0.0, stream=None):
    """`iters` steps under a boundary condition; returns the buffer holding the result."""
    h, w = buf0.shape
    fb = C.c_int(-1)
    call("hyd_cuda_iterate_stencil2d_bnd_f64", kind, boundary, fill, ptr(buf0), ptr(buf1), h, w, iters,
         C.byref(fb), stream_handle(stream))
    return buf0 if fb.value == 0 else buf1


def map_f64(body, inputs, n=None, out=None, want_sum=False, stream=None, _fn="hyd_cuda_map_f64", _dtype=None):
    """Fused element chain: `body` (C statements assigning v from x0.., i) over
    device tensors `inputs`; returns (out, sum or None)."""
    import torch
    dtype = torch.float64 if _dtype is None else _dtype
    n = inputs[0].numel() if n is None else n
    table = (C.c_void_p * max(len(inputs), 1))(*[t.data_ptr() for t in inputs])
    s = None
    if want_sum:
        dev = inputs[0].device if inputs else torch.device("cuda")
        s = torch.zeros(1, dtype=dtype, device=dev)
    call(_fn, body.encode(), C.cast(table, C.c_void_p), len(inputs), n,
         ptr(out) if out is not None else None, ptr(s) if s is not None else None, stream_handle(stream))
    return out, s


def map_i64(body, inputs, n=None, out=None, want_sum=False, stream=None):
    """The int64 form of map_f64 (C int64 semantics, wrapping sum)."""
    import torch
    return map_f64(body, inputs, n, out, want_sum, stream, _fn="hyd_cuda_map_i64", _dtype=torch.int64)


class GrayScott(C.Structure):
    """hyd_gray_scott_t; defaults are demo/gray_scott/gray_scott.hyd:19-25."""
    _fields_ = [("du", C.c_double), ("dv", C.c_double), ("feed", C.c_double), ("kill", C.c_double),
                ("dt", C.c_double)]

    def __init__(self, du=0.21, dv=0.105, feed=0.0545, kill=0.0620, dt=1.0):
        super().__init__(du, dv, feed, kill, dt)


def jacobi1d(src, dst, stream=None):
    call("hyd_cuda_jacobi1d_f64", ptr(src), ptr(dst), src.numel(), stream_handle(stream))


def iterate_jacobi1d(buf0, buf1, iters, stream=None):
    """Runs iters steps; returns the buffer holding the result."""
    which = C.c_int(0)
    call("hyd_cuda_iterate_jacobi1d_f64", ptr(buf0), ptr(buf1), buf0.numel(), iters, C.byref(which),
         stream_handle(stream))
    return buf1 if which.value else buf0


def gray_scott_step(u, v, u_out, v_out, params=None, stream=None):
    h, w = u.shape
    p = C.byref(params) if params is not None else None
    call("hyd_cuda_gray_scott_step_f64", ptr(u), ptr(v), ptr(u_out), ptr(v_out), h, w, p, stream_handle(stream))


def iterate_gray_scott(u0, v0, u1, v1, steps, params=None, stream=None):
    """Runs steps steps; returns the (u, v) buffers holding the result."""
    h, w = u0.shape
    which = C.c_int(0)
    p = C.byref(params) if params is not None else None
    call("hyd_cuda_iterate_gray_scott_f64", ptr(u0), ptr(v0), ptr(u1), ptr(v1), h, w, p, steps, C.byref(which),
         stream_handle(stream))
    return (u1, v1) if which.value else (u0, v0)


def selftest_dadd(x, y):
    """(integer-pipe sums, FP64-unit sums) of two float64 device tensors."""
    import torch
    emu, hw = torch.empty_like(x), torch.empty_like(x)
    call("hyd_cuda_selftest_dadd", ptr(x), ptr(y), ptr(emu), ptr(hw), x.numel(), None)
    return emu, hw


def selftest_div(x, divisor):
    """(the multiply-and-two-FMA quotient, the IEEE quotient) of x / divisor,
    divisor 3 or 5, both computed on the device."""
    import torch
    fast, hw = torch.empty_like(x), torch.empty_like(x)
    call("hyd_cuda_selftest_div", ptr(x), divisor, ptr(fast), ptr(hw), x.numel(), None)
    return fast, hw


def autotune_stencil2d(kind, h, w, reps=5):
    import numpy as np
    best = C.c_int(-1)
    times = np.zeros(len(STENCIL_VARIANTS))
    call("hyd_cuda_autotune_stencil2d", kind, h, w, reps, C.byref(best), times.ctypes.data)
    return best.value, times


def autotune_histogram(n, bins, reps=5):
    import numpy as np
    best = C.c_int(-1)
    times = np.zeros(6)
    call("hyd_cuda_autotune_histogram", n, bins, reps, C.byref(best), times.ctypes.data)
    return best.value, times


def scan(x, out, init=0, reverse=False, inclusive=False, stream=None):
    import torch
    fn = "hyd_cuda_scan_i64" if x.dtype == torch.int64 else "hyd_cuda_scan_f64"
    call(fn, ptr(x), ptr(out), x.numel(), init, int(reverse), int(inclusive), stream_handle(stream))


def segmented_reduce(offsets, vals, out, init=0, stream=None):
    import torch
    fn = "hyd_cuda_segmented_reduce_i64" if vals.dtype == torch.int64 else "hyd_cuda_segmented_reduce_f64"
    call(fn, ptr(offsets), offsets.numel(), ptr(vals), vals.numel(), init, ptr(out), stream_handle(stream))


def sort_indices(keys, perm, key_bits=None, stream=None):
    if key_bits is None:
        call("hyd_cuda_sort_indices_i64", ptr(keys), keys.numel(), ptr(perm), stream_handle(stream))
    else:
        call("hyd_cuda_sort_indices_bits_i64", ptr(keys), keys.numel(), key_bits, ptr(perm),
             stream_handle(stream))


def gather(perm, src, out, stream=None):
    import torch
    fn = {torch.int64: "hyd_cuda_gather_i64", torch.float64: "hyd_cuda_gather_f64",
          torch.int32: "hyd_cuda_gather_i32"}[src.dtype]
    call(fn, ptr(perm), perm.numel(), ptr(src), src.numel(), ptr(out), stream_handle(stream))


def coo_sum_duplicates(rows, cols, vals, stream=None):
    import torch
    n = rows.numel()
    o_r, o_c, o_v = (torch.empty_like(rows) for _ in range(3))
    k = torch.zeros(1, dtype=torch.int64, device=rows.device)
    call("hyd_cuda_coo_sum_duplicates_i64", ptr(rows), ptr(cols), ptr(vals), n, ptr(o_r), ptr(o_c), ptr(o_v),
         ptr(k), stream_handle(stream))
    return o_r, o_c, o_v, k


def csr_from_sorted_coo(nrows, nnz, rows, cols, vals, stream=None):
    import torch
    row_ptr = torch.zeros(nrows + 1, dtype=torch.int64, device=rows.device)
    col_idx = torch.zeros_like(cols)
    out_vals = torch.zeros_like(vals)
    call("hyd_cuda_csr_from_sorted_coo_i64", nrows, nnz, ptr(rows), ptr(cols), ptr(vals), ptr(row_ptr),
         ptr(col_idx), ptr(out_vals), stream_handle(stream))
    return row_ptr, col_idx, out_vals


def spmv_csr(row_ptr, col_idx, vals, x, y, lanes_per_row=0, stream=None):
    import torch
    fn = "hyd_cuda_spmv_csr_f64" if col_idx.dtype == torch.int64 else "hyd_cuda_spmv_csr_i32_f64"
    call(fn, row_ptr.numel() - 1, x.numel(), ptr(row_ptr), ptr(col_idx), ptr(vals), ptr(x), ptr(y),
         lanes_per_row, stream_handle(stream))


def synth_coo_batch(ninst, seed0=4, min_log2=10, max_log2=18, max_row_len=256, device="cuda", stream=None):
    """Allocates and fills a synthetic batch; returns (desc ndarray, rows, cols, vals, x)."""
    import numpy as np
    import torch
    desc = np.zeros((ninst, 3), dtype=np.int64)
    call("hyd_cuda_synth_coo_batch", ninst, seed0, min_log2, max_log2, max_row_len, desc.ctypes.data,
         None, None, None, None, 0, stream_handle(stream))
    nnz = int(desc[:, 2].sum())
    nx = int(desc[:, 1].sum())
    rows = torch.empty(max(nnz, 1), dtype=torch.int32, device=device)
    cols = torch.empty(max(nnz, 1), dtype=torch.int32, device=device)
    vals = torch.empty(max(nnz, 1), dtype=torch.float64, device=device)
    x = torch.empty(nx, dtype=torch.float64, device=device)
    call("hyd_cuda_synth_coo_batch", ninst, seed0, min_log2, max_log2, max_row_len, desc.ctypes.data,
         ptr(rows), ptr(cols), ptr(vals), ptr(x), rows.numel(), stream_handle(stream))
    return desc, rows, cols, vals, x


def batched_coo_csr_spmv(desc, rows, cols, vals, x, stream=None):
    """Returns (row_ptr, csr_cols, csr_vals, y) for a concatenated batch."""
    import numpy as np
    import torch
    desc = np.ascontiguousarray(desc, dtype=np.int64)
    ninst = desc.shape[0]
    nnz = int(desc[:, 2].sum())
    nr = int(desc[:, 0].sum())
    dev = x.device
    # every element is written by the pipeline: no fill kernels
    row_ptr = torch.empty(nr + ninst, dtype=torch.int64, device=dev)
    csr_cols = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    csr_vals = torch.empty(max(nnz, 1), dtype=torch.float64, device=dev)
    y = torch.empty(nr, dtype=torch.float64, device=dev)
    call("hyd_cuda_batched_coo_csr_spmv_f64", ninst, desc.ctypes.data, ptr(rows), ptr(cols), ptr(vals), ptr(x),
         ptr(row_ptr), ptr(csr_cols), ptr(csr_vals), ptr(y), stream_handle(stream))
    return row_ptr, csr_cols, csr_vals, y


class Server:
    """Thin owner of a hyd_server_t."""

    def __init__(self, budget_bytes=0, streams=0, max_batch=0, max_batch_bytes=0):
        cfg = ServerConfig(budget_bytes, streams, max_batch, max_batch_bytes)
        h = C.c_void_p()
        call("hyd_cuda_server_create", C.addressof(cfg), C.byref(h))
        self.h = h

    def submit(self, req):
        t = C.c_int64(-1)
        st = lib().hyd_cuda_server_submit(self.h, C.addressof(req), C.byref(t))
        return st, t.value

    def wait(self, ticket):
        st = C.c_int(-1)
        lat = C.c_double(0.0)
        call("hyd_cuda_server_wait", self.h, ticket, C.byref(st), C.byref(lat))
        return st.value, lat.value

    def stats(self):
        out = ServerStats()
        call("hyd_cuda_server_stats", self.h, C.addressof(out))
        return out

    def trace(self, reqs, arrivals):
        import numpy as np
        n = len(reqs)
        arr = (Request * n)(*reqs)
        t = np.ascontiguousarray(arrivals, dtype=np.float64)
        lat = np.zeros(n)
        st = np.zeros(n, dtype=np.int32)
        el = C.c_double(0.0)
        call("hyd_cuda_serve_trace", self.h, C.addressof(arr), t.ctypes.data, n, lat.ctypes.data, st.ctypes.data,
             C.byref(el))
        return lat, st, el.value

    def error(self):
        return (lib().hyd_cuda_server_error(self.h) or b"").decode()

    def shutdown(self):
        call("hyd_cuda_server_shutdown", self.h)

    def close(self):
        if self.h:
            lib().hyd_cuda_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plain_trace(reqs, arrivals, stream=None):
    import numpy as np
    n = len(reqs)
    arr = (Request * n)(*reqs)
    t = np.ascontiguousarray(arrivals, dtype=np.float64)
    lat = np.zeros(n)
    st = np.zeros(n, dtype=np.int32)
    el = C.c_double(0.0)
    call("hyd_cuda_plain_trace", C.addressof(arr), t.ctypes.data, n, lat.ctypes.data, st.ctypes.data, C.byref(el),
         stream_handle(stream))
    return lat, st, el.value


def resident_stats():
    """(attached arrays, uploads so far, resident bytes) of the export path's
    device-resident array copies."""
    e, u, b = C.c_int64(0), C.c_int64(0), C.c_int64(0)
    call("hyd_cuda_array_resident_stats", C.byref(e), C.byref(u), C.byref(b))
    return e.value, u.value, b.value


def make_array(np_array):
    """A hyd_array_t view of a C-contiguous numpy array (no copy; storage is
    borrowed, so never pass it to hyd_array_free)."""
    st = Storage(np_array.ctypes.data, 1)
    t = Tuple()
    t.ndims = np_array.ndim
    for i, e in enumerate(np_array.shape):
        t.elems[i] = e
    a = Array(C.pointer(st), np_array.ctypes.data, np_array.itemsize, t)
    a._keep = (st, np_array)
    return a


_libc = None


def array_free(p):
    """Release a hyd_array_t* that an export returned, as the reference
    runtime's hyd_array_free does (runtime/hydrangea_runtime.h:333-343): drop
    one reference to the storage, free data and storage record at zero, then
    the header.  The runtime allocates them with malloc/calloc for this."""
    global _libc
    if _libc is None:
        _libc = C.CDLL(None)
        _libc.free.argtypes = [C.c_void_p]
    a = p.contents
    st = a.storage.contents
    st.refcount -= 1
    if st.refcount == 0:
        _libc.free(st.data)
        _libc.free(C.cast(a.storage, C.c_void_p))
    _libc.free(C.cast(p, C.c_void_p))


def export_weighted_histogram(arr, bins):
    """hyd_export_weighted_histogram(hyd_array_t*, bins): returns the result as
    a caller-owned hyd_array_t* (free it with array_free)."""
    fn = lib().hyd_export_weighted_histogram
    fn.restype = C.POINTER(Array)
    fn.argtypes = [C.POINTER(Array), C.c_int64]
    return fn(C.byref(arr), bins)


def weighted_histogram_host(data, bins, strategy=SCATTER_AUTO):
    import numpy as np
    data = np.ascontiguousarray(data, dtype=np.int64)
    out = np.zeros(bins, dtype=np.int64)
    call("hyd_cuda_weighted_histogram_host", data.ctypes.data, data.size, bins, out.ctypes.data, strategy)
    return out


def dot_f64_host(xs, ys):
    import numpy as np
    xs = np.ascontiguousarray(xs, dtype=np.float64)
    ys = np.ascontiguousarray(ys, dtype=np.float64)
    r = C.c_double(0.0)
    call("hyd_cuda_dot_f64_host", xs.ctypes.data, ys.ctypes.data, xs.size, C.addressof(r))
    return r.value


def device_check(stream=None):
    return lib().hyd_cuda_check(stream_handle(stream))
