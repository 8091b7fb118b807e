"""GPU parity of the other iterate loops: jacobi_1d (examples/jacobi_1d.hyd)
and Gray-Scott (demo/gray_scott/gray_scott.hyd), bit-exact against the oracle's
restatement of the C backend, single steps and captured iterations, plus the
demo's exported procedure."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)


def _bits(a):
    return np.ascontiguousarray(a).view(np.int64)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 1000, (1 << 20) + 3])
def test_jacobi1d_step(hc, orc, dev, n):
    rng = np.random.default_rng(n)
    x = rng.uniform(-1, 1, n)
    x[::7] = np.abs(x[::7])
    out = torch.empty(n, dtype=torch.float64, device=dev)
    hc.jacobi1d(_t(x, dev), out)
    assert np.array_equal(_bits(out.cpu().numpy()), _bits(orc.jacobi1d(x, 1)))


def test_jacobi1d_known_answers(hc, orc, dev):
    # examples/jacobi_1d.hyd: 3 steps of ones stay ones; one step of 1..5
    b0, b1 = _t(np.ones(5), dev), torch.empty(5, dtype=torch.float64, device=dev)
    assert hc.iterate_jacobi1d(b0, b1, 3).cpu().tolist() == [1.0] * 5
    out = torch.empty(5, dtype=torch.float64, device=dev)
    hc.jacobi1d(_t(np.arange(1.0, 6.0), dev), out)
    assert out.cpu().tolist() == [4.0 / 3.0, 2.0, 3.0, 4.0, 14.0 / 3.0]


@pytest.mark.parametrize("iters", [1, 2, 7, 50])
def test_jacobi1d_iterate_graph(hc, orc, dev, iters):
    rng = np.random.default_rng(iters)
    x = rng.uniform(0, 1, 100_001)
    ref = orc.jacobi1d(x, iters)
    s = torch.cuda.Stream()
    b0, b1 = _t(x, dev), torch.empty(len(x), dtype=torch.float64, device=dev)
    with torch.cuda.stream(s):
        res = hc.iterate_jacobi1d(b0, b1, iters, stream=s)
        s.synchronize()
        got1 = res.cpu().numpy()
        b0.copy_(_t(x, dev))
        res = hc.iterate_jacobi1d(b0, b1, iters, stream=s)  # replays the cached graph
        s.synchronize()
    assert np.array_equal(_bits(got1), _bits(ref)) and np.array_equal(_bits(res.cpu().numpy()), _bits(ref))


@pytest.mark.parametrize("h,w", [(1, 1), (1, 7), (5, 3), (64, 64), (257, 130)])
def test_gray_scott_step(hc, orc, dev, h, w):
    rng = np.random.default_rng(h * 1000 + w)
    u, v = rng.uniform(0, 1, (h, w)), rng.uniform(0, 1, (h, w))
    v[::3, ::2] = -v[::3, ::2]  # negative values too
    un, vn = torch.empty((h, w), dtype=torch.float64, device=dev), torch.empty((h, w), dtype=torch.float64, device=dev)
    p = hc.GrayScott(du=0.2, dv=0.1, feed=0.05, kill=0.06, dt=0.9)
    hc.gray_scott_step(_t(u, dev), _t(v, dev), un, vn, params=p)
    ru, rv = orc.gray_scott(u, v, 1, du=0.2, dv=0.1, feed=0.05, kill=0.06, dt=0.9)
    assert np.array_equal(_bits(un.cpu().numpy()), _bits(ru)) and np.array_equal(_bits(vn.cpu().numpy()), _bits(rv))


def test_gray_scott_iterate_graph_default_params(hc, orc, dev):
    h, w, steps = 96, 80, 40
    rng = np.random.default_rng(5)
    u, v = np.ones((h, w)), np.where(rng.uniform(size=(h, w)) < 0.1, 0.5, 0.0)
    s = torch.cuda.Stream()
    bufs = [_t(u, dev), _t(v, dev), torch.empty((h, w), dtype=torch.float64, device=dev),
            torch.empty((h, w), dtype=torch.float64, device=dev)]
    with torch.cuda.stream(s):
        ru, rv = hc.iterate_gray_scott(bufs[0], bufs[1], bufs[2], bufs[3], steps, stream=s)
        s.synchronize()
    ou, ov = orc.gray_scott(u, v, steps)
    assert np.array_equal(_bits(ru.cpu().numpy()), _bits(ou)) and np.array_equal(_bits(rv.cpu().numpy()), _bits(ov))


def _demo_init(h=256, w=256):
    i, j = np.meshgrid(np.arange(h), np.arange(w), indexing="ij")
    di, dj = i - h // 2, j - w // 2
    v = np.where(di * di + dj * dj < 400, 0.5, np.where((i * 251 + j * 127) % 100 < 2, 0.5, 0.0))
    return np.ones((h, w)), v


def test_export_gray_scott_matches_program(hc, orc, dev):
    L = hc.lib()
    f = L.hyd_export_gray_scott
    f.restype = C.POINTER(hc.Array)
    f.argtypes = []
    out = f()
    a = out.contents
    assert a.shape.ndims == 2 and a.shape.elems[0] == 256 and a.shape.elems[1] == 256
    got = np.ctypeslib.as_array(C.cast(a.data, C.POINTER(C.c_double)), shape=(256, 256)).copy()
    u, v = _demo_init()
    _, ref_v = orc.gray_scott(u, v, 5000)
    assert np.array_equal(_bits(got), _bits(ref_v))
    # what the reference's hyd_array_free does: the export is memoised, so this
    # drops one reference of the storage and frees the header
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    st = a.storage.contents
    st.refcount -= 1
    if st.refcount == 0:
        libc.free(st.data)
        libc.free(C.cast(a.storage, C.c_void_p))
    libc.free(C.cast(out, C.c_void_p))
