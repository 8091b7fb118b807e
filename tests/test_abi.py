"""The C-ABI library loads, exports every symbol include/*.h declares, and
rejects bad arguments before touching a GPU (runs without one)."""
import ctypes as C
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


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


def test_gray_scott_demo_host_links_unchanged(tmp_path):
    """The reference's embedding demo host links against the runtime without a
    change: its generated header (CodegenC.hs:427-460 form) only needs to
    declare hyd_export_gray_scott.  Link only -- there is no GPU to run it."""
    import shutil
    import subprocess
    sys.path.insert(0, ROOT)
    from oracle import build as ob
    root = os.environ.get("HYD_REFERENCE_ROOT", ob.DEFAULT_REFERENCE_ROOT)
    main = os.path.join(root, "demo", "gray_scott", "main.cpp")
    if not os.path.exists(main) or shutil.which("g++") is None:
        pytest.skip("reference demo sources not present")
    (tmp_path / "gray_scott.h").write_text(
        "#ifndef HYDRANGEA_EXPORT_GRAY_SCOTT_H\n#define HYDRANGEA_EXPORT_GRAY_SCOTT_H\n"
        '#include "hydrangea_runtime.h"\n#include "hyd_cuda.h"\n#endif\n')
    pkg = os.path.join(ROOT, "hydrangea-compiler_gb300")
    out = tmp_path / "gs_demo"
    cmd = ["g++", "-O1", "-fopenmp", "-I", str(tmp_path), "-I", os.path.join(root, "runtime"),
           "-I", os.path.join(ROOT, "oracle"), "-I", os.path.join(ROOT, "include"), main,
           "-L", pkg, "-lhyd_cuda", "-Wl,-rpath," + pkg, "-o", str(out)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-2000:]
    assert out.exists()
