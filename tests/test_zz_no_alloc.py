"""GPU test of hyd_cuda_dot_f64_noalloc, the dot product for callers that may
not allocate device memory (latency-critical loops where cudaMalloc can stall
other streams, or processes held to a fixed device-memory budget).

It calls the allocation-free entry point through the C ABI twice in a row and
checks each result against hyd_cuda_dot_f64 within the reduction tolerance used
by the other parity tests (relative 1e-12).  The second call checks that the
shared static scratch left by the first call does not leak into the next
result.  This file is collected last so that a run stopping at the first
failure has already run every other test; it also passes alone in a fresh
process, where its first call is the one that looks up the scratch address.
"""
import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _dot_noalloc(L, xs, ys, out, stream):
    return L.hyd_cuda_dot_f64_noalloc(C.c_void_p(xs.data_ptr()), C.c_void_p(ys.data_ptr()),
                                      xs.numel(), C.c_void_p(out.data_ptr()), C.c_void_p(stream))


@pytest.mark.parametrize("n", [(1 << 20) + 3, 1 << 24])
def test_noalloc_dot_matches_existing_entry_point(hc, n):
    L = hc.lib()
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    g = torch.Generator(device=dev)
    g.manual_seed(1234 + n)
    xs = torch.rand(n, dtype=torch.float64, device=dev, generator=g) * 2 - 1
    ys = torch.rand(n, dtype=torch.float64, device=dev, generator=g) * 2 - 1
    stream = torch.cuda.current_stream().cuda_stream
    got = []
    for _ in range(2):  # two calls in a row through the shared static scratch
        out = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        assert _dot_noalloc(L, xs, ys, out, stream) == hc.OK, hc.last_error()
        torch.cuda.synchronize()
        got.append(float(out.item()))
    ref_out = torch.zeros(1, dtype=torch.float64, device=dev)
    hc.dot_f64(xs, ys, ref_out)
    ref = float(ref_out.item())
    for v in got:
        assert abs(v - ref) <= TOL * max(1.0, abs(ref)), (v, ref)
