"""The host I/O path (csrc/csv_io.cu) against the reference runtime's own CSV
reader and writer (hyd_read_array_csv / hyd_read_float_array_csv,
runtime/hydrangea_runtime.h:549-592; runtime/hyd_write_csv.c), compiled
unmodified into the witness library: the same values, the same output bytes,
and on malformed input the same exit status and message.  Needs the reference
tree (the witness is built from it); no GPU."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

LIBC = C.CDLL(None)
LIBC.free.argtypes = [C.c_void_p]


@pytest.fixture(scope="module")
def W():
    w = O.witness()
    if w is None:
        pytest.skip("the reference tree (for the witness library) is not present")
    return w


def _shape(hc, *dims):
    t = hc.Tuple()
    t.ndims = len(dims)
    for i, d in enumerate(dims):
        t.elems[i] = d
    return t


def _free(p):
    a = p.contents
    st = a.storage.contents
    st.refcount -= 1
    if st.refcount == 0:
        LIBC.free(st.data)
        LIBC.free(C.cast(a.storage, C.c_void_p))
    LIBC.free(C.cast(p, C.c_void_p))


def _ours(hc, path, n, is_float):
    L = hc.lib()
    fn = L.hyd_cuda_read_float_array_csv if is_float else L.hyd_cuda_read_array_csv
    fn.restype = C.POINTER(hc.Array)
    p = fn(path.encode(), _shape(hc, n))
    ct = C.c_double if is_float else C.c_int64
    out = np.ctypeslib.as_array(C.cast(p.contents.data, C.POINTER(ct)), shape=(n,)).copy() if n else \
        np.zeros(0, np.float64 if is_float else np.int64)
    _free(p)
    return out


def _theirs(W, path, n, is_float):
    out = np.zeros(n, np.float64 if is_float else np.int64)
    (W.wit_read_float_array_csv if is_float else W.wit_read_array_csv)(path.encode(), n, out)
    return out


def _same(a, b):
    return a.dtype == b.dtype and np.array_equal(a.view(np.uint64), b.view(np.uint64))


VALID_INT = [
    ("1,2,3", 3), ("1, 2 ,3\n", 3), ("  7\n8\r\n9", 3), ("1,,2,,,3", 3), ("+4 -5 006 -0", 4),
    ("1\t2\t3", 3), ("1,\t2, \t 3", 3), ("9223372036854775807,-9223372036854775808", 2),
    ("1,2,3,junk,more", 3), ("5", 1), ("1 2 3", 0), ("12abc", 1), ("1,2\n3,4\n", 4),
    ("99999999999999999999,1", 2), ("-99999999999999999999", 1),
]
VALID_FLOAT = [
    ("1.5,2.25,-3", 3), (".5 5. 1e3 -2E-2", 4), ("0.1,0.2,0.3", 3), ("1.7976931348623157e308, 4.9e-324", 2),
    ("-0.0,0", 2), ("inf,-inf,nan", 3), ("infinity -Infinity NAN(123)", 3), ("0x1.8p3,0X10", 2),
    ("1e400,-1e400,1e-400", 3), ("3.14159265358979323846264338327950288", 1), ("2.5e+3x", 1),
    ("1,2\n3,4\n", 4), ("123456789012345678901234567890.5", 1), ("1e", 1), ("1e+,2", 1),
]


@pytest.mark.parametrize("text,n", VALID_INT)
def test_int_reader_matches_reference(hc, W, tmp_path, text, n):
    p = str(tmp_path / "a.csv")
    open(p, "w").write(text)
    assert _same(_ours(hc, p, n, False), _theirs(W, p, n, False))


@pytest.mark.parametrize("text,n", VALID_FLOAT)
def test_float_reader_matches_reference(hc, W, tmp_path, text, n):
    p = str(tmp_path / "a.csv")
    open(p, "w").write(text)
    assert _same(_ours(hc, p, n, True), _theirs(W, p, n, True))


@pytest.mark.parametrize("is_float", [False, True])
def test_large_file_threaded_reader_matches_reference(hc, W, tmp_path, is_float):
    # several MiB: the threaded path, slices split inside separator runs
    rng = np.random.default_rng(5 + is_float)
    n = 600_000
    if is_float:
        vals = rng.standard_normal(n) * 10.0 ** rng.integers(-300, 300, n)
        toks = ["%.17g" % v for v in vals]
    else:
        toks = [str(v) for v in rng.integers(-(1 << 62), 1 << 62, n)]
    seps = [",", " ", "\n", ", ", " ,\r\n", "\t", ",,  "]
    pick = rng.integers(0, len(seps), n)
    text = "  " + "".join(t + seps[k] for t, k in zip(toks, pick))
    p = str(tmp_path / "big.csv")
    open(p, "w").write(text)
    for m in (n, n - 1, 12345):
        assert _same(_ours(hc, p, m, is_float), _theirs(W, p, m, is_float))


@pytest.mark.parametrize("shape", [(7,), (3, 4), (0,), (2, 0), (0, 5), (1, 1), (200_000,), (300, 700)])
@pytest.mark.parametrize("is_float", [False, True])
def test_writer_matches_reference_bytes(hc, W, tmp_path, shape, is_float):
    rng = np.random.default_rng(9)
    size = int(np.prod(shape))
    if is_float:
        data = rng.standard_normal(size) * 10.0 ** rng.integers(-20, 20, size)
        data[:3] = [0.1, -0.0, 1e308][:min(3, size)] if size else data[:0]
    else:
        data = rng.integers(-(1 << 63), (1 << 63) - 1, size, dtype=np.int64)
    d0 = shape[0]
    d1 = shape[1] if len(shape) == 2 else 0
    a, b = str(tmp_path / "ours.csv"), str(tmp_path / "theirs.csv")
    L = hc.lib()
    arr = hc.make_array(np.ascontiguousarray(data.reshape(shape)))
    (L.hyd_cuda_write_array_csv_float if is_float else L.hyd_cuda_write_array_csv)(C.byref(arr), a.encode())
    (W.wit_write_array_csv_float if is_float else W.wit_write_array_csv)(
        np.ascontiguousarray(data), len(shape), d0, d1, b.encode())
    assert open(a, "rb").read() == open(b, "rb").read()


_PROBE = r"""
import ctypes as C, sys
sys.path.insert(0, %r)
import numpy as np
which, path, n, is_float = sys.argv[1], sys.argv[2], int(sys.argv[3]), sys.argv[4] == "1"
if which == "ours":
    import __graft_entry__ as g
    hc = g.package()
    L = hc.lib()
    t = hc.Tuple(); t.ndims = 1; t.elems[0] = n
    fn = L.hyd_cuda_read_float_array_csv if is_float else L.hyd_cuda_read_array_csv
    fn.restype = C.c_void_p
    fn(path.encode(), t)
else:
    from oracle import oracle as O
    W = O.witness()
    out = np.zeros(n, np.float64 if is_float else np.int64)
    (W.wit_read_float_array_csv if is_float else W.wit_read_array_csv)(path.encode(), n, out)
print("read ok")
""" % ROOT

MALFORMED = [
    ("1,2", 3, False), ("1,,x", 3, False), (",1", 1, False), ("1\t,2", 2, False), ("", 1, False),
    ("1\t", 2, False), ("1 ", 2, False), ("1, \n", 2, False), ("12abc,3", 2, False), ("  ", 1, False),
    ("1.5,", 2, True), ("1.5 abc", 2, True), ("x", 1, True), ("1,2\t ,3", 3, True),
]


@pytest.mark.parametrize("text,n,is_float", MALFORMED)
def test_malformed_input_fails_like_reference(W, tmp_path, text, n, is_float):
    p = str(tmp_path / "bad.csv")
    open(p, "w").write(text)
    res = {}
    for which in ("ours", "theirs"):
        r = subprocess.run([sys.executable, "-c", _PROBE, which, p, str(n), "1" if is_float else "0"],
                           capture_output=True, text=True, timeout=120)
        res[which] = (r.returncode, r.stderr.strip().splitlines()[-1:] if r.stderr.strip() else [])
    assert res["ours"] == res["theirs"], res
    assert res["ours"][0] == 1


def test_missing_file_fails_like_reference(W, tmp_path):
    p = str(tmp_path / "absent.csv")
    res = {}
    for which in ("ours", "theirs"):
        r = subprocess.run([sys.executable, "-c", _PROBE, which, p, "3", "0"], capture_output=True, text=True,
                           timeout=120)
        res[which] = (r.returncode, r.stderr.strip())
    assert res["ours"] == res["theirs"] and res["ours"][0] == 1
