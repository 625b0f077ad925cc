"""Device arithmetic helpers give the host's results bit for bit."""
import numpy as np
import pytest

from barney_gb300 import _native as N

pytestmark = pytest.mark.gpu


def test_bounded_sincos_device_equals_host(cuda):
    import torch
    from barney_gb300.device import _stream
    x = np.linspace(-np.pi / 4, 2 * np.pi + np.pi / 4, 1_000_003, dtype=np.float64).astype(np.float32)
    hs, hc = np.empty_like(x), np.empty_like(x)
    assert N.lib().gbv_selftest_sincos(x.ctypes.data, x.size, hs.ctypes.data, hc.ctypes.data, 0, None) == N.GBV_OK
    dx = torch.from_numpy(x).cuda()
    ds, dc = torch.empty_like(dx), torch.empty_like(dx)
    assert N.lib().gbv_selftest_sincos(dx.data_ptr(), x.size, ds.data_ptr(), dc.data_ptr(), 1, _stream()) == N.GBV_OK
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ds.cpu().numpy().view(np.uint32), hs.view(np.uint32))
    np.testing.assert_array_equal(dc.cpu().numpy().view(np.uint32), hc.view(np.uint32))
