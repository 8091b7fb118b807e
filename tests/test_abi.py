"""The C-ABI library loads, exports every symbol include/*.h declares, and
rejects bad arguments before touching a GPU (runs without one)."""
import ctypes as C

import pytest


def test_library_exports_header_symbols(hc):
    names = hc.header_functions()
    assert "hyd_cuda_init" in names and "hyd_cuda_dot_f64" in names
    missing = [n for n in names if not hasattr(hc.lib(), n)]
    assert not missing, missing


def test_binding_covers_header(hc):
    # every declared function has a ctypes signature in the Python mirror
    missing = [n for n in hc.header_functions() if n not in hc.SIGNATURES]
    assert not missing, missing


def test_version_and_status_strings(hc):
    L = hc.lib()
    assert L.hyd_cuda_version() >= 100
    assert L.hyd_cuda_status_string(0) == b"ok"
    assert L.hyd_cuda_status_string(hc.ERR_BOUNDS) == b"index out of bounds"


@pytest.mark.parametrize("call", [
    lambda L: L.hyd_cuda_dot_f64(None, None, -1, C.c_void_p(8), None),
    lambda L: L.hyd_cuda_dot_f64(None, None, 10, C.c_void_p(8), None),
    lambda L: L.hyd_cuda_dot_f64(C.c_void_p(8), C.c_void_p(8), 10, None, None),
    lambda L: L.hyd_cuda_sum_f64(None, 5, C.c_void_p(8), None),
    lambda L: L.hyd_cuda_weighted_histogram_i64(C.c_void_p(8), 10, 0, C.c_void_p(8), 0, None),
    lambda L: L.hyd_cuda_weighted_histogram_i64(C.c_void_p(8), 10, 64, None, 0, None),
    lambda L: L.hyd_cuda_weighted_histogram_i64(C.c_void_p(8), 10, 64, C.c_void_p(8), 99, None),
    lambda L: L.hyd_cuda_scatter_add_i64(None, None, 3, C.c_void_p(8), 4, 0, None),
    lambda L: L.hyd_cuda_scatter_add_f64(C.c_void_p(8), C.c_void_p(8), 3, C.c_void_p(8), 0, None),
    lambda L: L.hyd_cuda_fill_uniform_i64(C.c_void_p(8), 4, 1, 0, None),
])
def test_invalid_arguments_rejected(hc, call):
    assert call(hc.lib()) == hc.ERR_INVALID
    assert hc.last_error()


def test_server_requires_device_or_rejects_cleanly(hc):
    import ctypes as C
    import torch
    L = hc.lib()
    assert L.hyd_cuda_server_submit(None, None, None) == hc.ERR_INVALID
    assert L.hyd_cuda_server_wait(None, 0, None, None) == hc.ERR_INVALID
    assert L.hyd_cuda_request_run(None, None) == hc.ERR_INVALID
    if not torch.cuda.is_available():
        h = C.c_void_p()
        assert L.hyd_cuda_server_create(None, C.byref(h)) == hc.ERR_NO_DEVICE
