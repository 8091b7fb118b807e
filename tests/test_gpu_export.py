"""GPU parity of the embedding boundary: host-pointer entry points (the
host->device copies pipelined against the kernels in chunks), the
`hyd_export_<name>` symbols on the reference's `hyd_array_t`
(CodegenC.hs:372-460) and arrays that the reference's `hyd_array_free`
(runtime/hydrangea_runtime.h:333-343) releases."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LIBC = C.CDLL(None)
LIBC.free.argtypes = [C.c_void_p]


def _array_free(hc, p):
    """What the reference runtime's hyd_array_free does: drop one reference
    to the storage, free data + storage at zero, then the header."""
    a = p.contents
    st = a.storage.contents
    st.refcount -= 1
    if st.refcount == 0:
        LIBC.free(st.data)
        LIBC.free(C.cast(a.storage, C.c_void_p))
    LIBC.free(C.cast(p, C.c_void_p))


@pytest.mark.parametrize("n", [0, 5, 4099, 20_000_003])  # the last spans three 64 MiB chunks
@pytest.mark.parametrize("bins", [64, 65536])
def test_histogram_host_path(hc, orc, n, bins):
    data = orc.uniform_i64(n, 21, 1 << 20) if n else np.zeros(0, np.int64)
    got = hc.weighted_histogram_host(data, bins)
    ref = orc.weighted_hist(data, bins) if n else np.zeros(bins, np.int64)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("n", [0, 1, 1000, 20_000_001])
def test_dot_host_path(hc, orc, n):
    rng = np.random.default_rng(22)
    xs, ys = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    got = hc.dot_f64_host(xs, ys)
    ref = orc.dot_compensated(xs, ys) if n else 0.0
    assert abs(got - ref) <= 1e-12 * max(1.0, np.abs(xs * ys).sum())


def test_export_symbols_on_hyd_array(hc, orc):
    L = hc.lib()
    data = orc.uniform_i64(100_000, 23, 1 << 20)
    fn = L.hyd_export_weighted_histogram
    fn.restype = C.POINTER(hc.Array)
    fn.argtypes = [C.POINTER(hc.Array), C.c_int64]
    arr = hc.make_array(data)
    out = fn(C.byref(arr), 4096)
    a = out.contents
    assert a.shape.ndims == 1 and a.shape.elems[0] == 4096 and a.elem_size == 8
    assert a.storage.contents.refcount == 1
    got = np.ctypeslib.as_array(C.cast(a.data, C.POINTER(C.c_int64)), shape=(4096,)).copy()
    assert np.array_equal(got, orc.weighted_hist(data, 4096))
    _array_free(hc, out)  # allocated with malloc/calloc, as the reference allocator

    xs, ys = np.linspace(-1, 1, 7777), np.linspace(2, -2, 7777)
    dot = L.hyd_export_dot
    dot.restype = C.c_double
    dot.argtypes = [C.POINTER(hc.Array), C.POINTER(hc.Array)]
    ax, ay = hc.make_array(xs), hc.make_array(ys)
    assert abs(dot(C.byref(ax), C.byref(ay)) - orc.dot_compensated(xs, ys)) < 1e-12 * 7777


def test_runtime_array_alloc_is_zeroed_and_freeable(hc):
    L = hc.lib()
    f = L.hyd_cuda_array_alloc
    f.restype = C.POINTER(hc.Array)
    f.argtypes = [hc.Tuple, C.c_size_t]
    t = hc.Tuple()
    t.ndims = 2
    t.elems[0], t.elems[1] = 3, 5
    p = f(t, 8)
    a = p.contents
    assert a.shape.ndims == 2 and a.elem_size == 8
    vals = np.ctypeslib.as_array(C.cast(a.data, C.POINTER(C.c_int64)), shape=(15,))
    assert not vals.any()
    _array_free(hc, p)


def test_gray_scott_export_is_memoised(hc):
    # like the reference's zero-argument array procedures (CodegenC.hs:812-833):
    # one computation, then views over the same storage with the reference
    # count raised; hyd_array_free of a view leaves the others valid
    L = hc.lib()
    f = L.hyd_export_gray_scott
    f.restype = C.POINTER(hc.Array)
    f.argtypes = []
    a, b = f(), f()
    sa, sb = a.contents, b.contents
    assert C.cast(sa.storage, C.c_void_p).value == C.cast(sb.storage, C.c_void_p).value
    assert sa.data == sb.data and sa.shape.elems[0] == 256 and sb.shape.elems[1] == 256
    rc = sa.storage.contents.refcount
    assert rc >= 3  # the runtime's own reference and these two views
    first = np.ctypeslib.as_array(C.cast(sa.data, C.POINTER(C.c_double)), shape=(256, 256)).copy()
    _array_free(hc, a)
    assert sb.storage.contents.refcount == rc - 1
    again = np.ctypeslib.as_array(C.cast(sb.data, C.POINTER(C.c_double)), shape=(256, 256))
    assert np.array_equal(first, again)
    _array_free(hc, b)


def test_resident_arrays_skip_the_upload(hc, orc):
    L = hc.lib()
    n = 100_000
    rng = np.random.default_rng(24)
    xs, ys = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    ax, ay = hc.make_array(xs), hc.make_array(ys)
    dot = L.hyd_export_dot
    dot.restype = C.c_double
    dot.argtypes = [C.POINTER(hc.Array), C.POINTER(hc.Array)]
    streamed = dot(C.byref(ax), C.byref(ay))  # not attached: the host data is streamed
    e0, u0, b0 = hc.resident_stats()
    hc.check(L.hyd_cuda_array_attach(C.byref(ax)))
    hc.check(L.hyd_cuda_array_attach(C.byref(ay)))
    assert hc.resident_stats() == (e0 + 2, u0 + 2, b0 + 16 * n)
    assert L.hyd_cuda_array_device_data(C.byref(ax)) is not None
    # two calls read the device copies: same bits as the streamed call, no upload
    assert dot(C.byref(ax), C.byref(ay)) == streamed
    assert dot(C.byref(ax), C.byref(ay)) == streamed
    assert hc.resident_stats()[1] == u0 + 2
    # a declared host write is uploaded once, at the next use (doubling is exact)
    xs *= 2.0
    hc.check(L.hyd_cuda_array_host_modified(C.byref(ax)))
    assert dot(C.byref(ax), C.byref(ay)) == 2.0 * streamed
    assert hc.resident_stats()[1] == u0 + 3
    hc.check(L.hyd_cuda_array_detach(C.byref(ax)))
    hc.check(L.hyd_cuda_array_detach(C.byref(ay)))
    assert hc.resident_stats()[0] == e0
    assert L.hyd_cuda_array_device_data(C.byref(ax)) is None
    assert L.hyd_cuda_array_detach(C.byref(ax)) == hc.ERR_INVALID  # not attached any more
    hc.lib().hyd_cuda_check(None)

    # the histogram export through a resident array
    data = orc.uniform_i64(300_001, 25, 1 << 20)
    ad = hc.make_array(data)
    hc.check(L.hyd_cuda_array_attach(C.byref(ad)))
    fn = L.hyd_export_weighted_histogram
    fn.restype = C.POINTER(hc.Array)
    fn.argtypes = [C.POINTER(hc.Array), C.c_int64]
    for bins in (64, 65536):
        out = fn(C.byref(ad), bins)
        got = np.ctypeslib.as_array(C.cast(out.contents.data, C.POINTER(C.c_int64)), shape=(bins,)).copy()
        assert np.array_equal(got, orc.weighted_hist(data, bins))
        _array_free(hc, out)
    assert hc.resident_stats()[1] == u0 + 4  # one upload, at attach
    hc.check(L.hyd_cuda_array_detach(C.byref(ad)))


def test_csv_to_and_from_device(hc, tmp_path):
    # the device forms of the host I/O path: what the host reader returns,
    # copied to the device; what the host writer writes, read back from it;
    # malformed input is a status, not an exit
    import torch
    L = hc.lib()
    rng = np.random.default_rng(31)
    ints = rng.integers(-(1 << 62), 1 << 62, 250_001)
    flts = rng.standard_normal(250_001) * 1e-3
    pi, pf = str(tmp_path / "i.csv"), str(tmp_path / "f.csv")
    open(pi, "w").write(" ,".join(str(v) for v in ints) + "\n")
    open(pf, "w").write("\n".join("%.17g" % v for v in flts))
    di = torch.empty(len(ints), dtype=torch.int64, device="cuda")
    df = torch.empty(len(flts), dtype=torch.float64, device="cuda")
    hc.check(L.hyd_cuda_read_csv_i64_to_device(pi.encode(), len(ints), di.data_ptr(), None))
    hc.check(L.hyd_cuda_read_csv_f64_to_device(pf.encode(), len(flts), df.data_ptr(), None))
    assert np.array_equal(di.cpu().numpy(), ints)
    assert np.array_equal(df.cpu().numpy().view(np.uint64), flts.view(np.uint64))
    t = hc.Tuple()
    t.ndims, t.elems[0], t.elems[1] = 2, 500, 500
    oi, hi = str(tmp_path / "oi.csv"), str(tmp_path / "hi.csv")
    hc.check(L.hyd_cuda_write_csv_i64_from_device(di.data_ptr(), t, oi.encode(), None))
    block = np.ascontiguousarray(ints[:250_000].reshape(500, 500))
    L.hyd_cuda_write_array_csv(C.byref(hc.make_array(block)), hi.encode())
    assert open(oi, "rb").read() == open(hi, "rb").read()
    bad = str(tmp_path / "bad.csv")
    open(bad, "w").write("1,2,x")
    assert L.hyd_cuda_read_csv_i64_to_device(bad.encode(), 3, di.data_ptr(), None) == hc.ERR_INVALID
    assert L.hyd_cuda_read_csv_i64_to_device(str(tmp_path / "none.csv").encode(), 3, di.data_ptr(), None) == \
        hc.ERR_INVALID
