"""GPU test of hyd_cuda_dot_f64_noalloc, the dot product for callers that may
not allocate device memory (latency-critical loops where cudaMalloc can stall
other streams, or processes held to a fixed device-memory budget).

It calls the allocation-free entry point through the C ABI twice in a row and
checks each result:
  * bit for bit against hyd_cuda_dot_f64, which runs the same kernel with the
    same grid and combines the partials in the same order;
  * against the oracle's compensated dot within the reduction tolerance of the
    other parity tests (relative 1e-12).
The cases cover the 32-byte vector path, the scalar path (inputs offset by one
element, so not 32-byte aligned) and the empty input, which must write 0.0.
The second call checks that the shared static scratch left by the first call
does not leak into the next result.  This file is collected last so that a run
stopping at the first failure has already run every other test; it also passes
alone in a fresh process, where its first call is the one that looks up the
scratch address.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _dot_noalloc(L, xs, ys, out, stream):
    return L.hyd_cuda_dot_f64_noalloc(C.c_void_p(xs.data_ptr()), C.c_void_p(ys.data_ptr()),
                                      xs.numel(), C.c_void_p(out.data_ptr()), C.c_void_p(stream))


def _dot_existing(L, xs, ys, out, stream):
    return L.hyd_cuda_dot_f64(C.c_void_p(xs.data_ptr()), C.c_void_p(ys.data_ptr()),
                              xs.numel(), C.c_void_p(out.data_ptr()), C.c_void_p(stream))


@pytest.mark.parametrize("n,offset", [((1 << 20) + 3, 0), (1 << 24, 0), ((1 << 20) + 3, 1), (4097, 1), (0, 0)])
def test_noalloc_dot_matches_existing_entry_point(hc, orc, n, offset):
    L = hc.lib()
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    total = n + offset
    xs_full = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    ys_full = torch.empty(max(total, 1), dtype=torch.float64, device=dev)
    hc.fill_uniform_f64(xs_full, 11, -1.0, 1.0)
    hc.fill_uniform_f64(ys_full, 12, -1.0, 1.0)
    xs, ys = xs_full[offset:total], ys_full[offset:total]
    if offset:
        assert xs.data_ptr() % 32 != 0  # the scalar path
    stream = torch.cuda.current_stream().cuda_stream

    got = []
    for _ in range(2):  # two calls in a row through the shared static scratch
        out = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        assert _dot_noalloc(L, xs, ys, out, stream) == hc.OK, hc.last_error()
        torch.cuda.synchronize()
        got.append(float(out.item()))
    ref_out = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    assert _dot_existing(L, xs, ys, ref_out, stream) == hc.OK, hc.last_error()
    torch.cuda.synchronize()
    ref = float(ref_out.item())

    hx = orc.uniform_f64(total, 11, -1.0, 1.0)[offset:]
    hy = orc.uniform_f64(total, 12, -1.0, 1.0)[offset:]
    truth = orc.dot_compensated(hx, hy) if n else 0.0
    for v in got:
        assert np.float64(v).tobytes() == np.float64(ref).tobytes(), (v, ref)
        assert abs(v - truth) <= TOL * max(1.0, abs(truth)), (v, truth)
    if n == 0:
        assert got == [0.0, 0.0]
