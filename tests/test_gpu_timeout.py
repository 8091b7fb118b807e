"""GPU test of the timeout path of the runtime's bounded device waits.

Every device-side wait of this runtime (the mbarrier waits of the TMA kernels,
the tile-status waits of the decoupled look-back scans) gives up after a poll
limit, sets the device error word and returns, instead of hanging.  Here
hyd_cuda_selftest_timeout runs each of those two waits on a condition that
nothing satisfies (an mbarrier no thread arrives at; 32 tile flags no tile
publishes) with a short poll limit.  The test checks that hyd_cuda_check then
reports HYD_CUDA_ERR_TIMEOUT once, that the error is cleared by reading it, and
that a normal call right after gives the right result on the same context."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1])
def test_bounded_wait_times_out_and_context_stays_usable(hc, orc, dev, which):
    L = hc.lib()
    s = torch.cuda.current_stream().cuda_stream
    assert hc.device_check() == hc.OK
    assert L.hyd_cuda_selftest_timeout(which, 1 << 12, s) == hc.OK, hc.last_error()
    assert L.hyd_cuda_check(s) == hc.ERR_TIMEOUT
    assert L.hyd_cuda_check(s) == hc.OK  # read and cleared
    n = 100_003
    xs = torch.empty(n, dtype=torch.float64, device=dev)
    ys = torch.empty(n, dtype=torch.float64, device=dev)
    hc.fill_uniform_f64(xs, 31, -1.0, 1.0)
    hc.fill_uniform_f64(ys, 32, -1.0, 1.0)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    hc.dot_f64(xs, ys, out)
    assert L.hyd_cuda_check(s) == hc.OK
    ref = orc.dot_compensated(orc.uniform_f64(n, 31, -1.0, 1.0), orc.uniform_f64(n, 32, -1.0, 1.0))
    assert abs(out.item() - ref) <= 1e-12 * max(1.0, abs(ref))
    # a scan (which uses the look-back wait) still completes normally
    x = torch.arange(1 << 16, dtype=torch.int64, device=dev)
    y = torch.empty_like(x)
    hc.scan(x, y)
    assert L.hyd_cuda_check(s) == hc.OK
    assert np.array_equal(y.cpu().numpy(), orc.scan_i64(x.cpu().numpy()))


def test_selftest_timeout_rejects_bad_arguments(hc, dev):
    L = hc.lib()
    assert L.hyd_cuda_selftest_timeout(2, 16, None) == hc.ERR_INVALID
    assert L.hyd_cuda_selftest_timeout(0, 0, None) == hc.ERR_INVALID
    assert L.hyd_cuda_selftest_timeout(0, (1 << 20) + 1, None) == hc.ERR_INVALID
