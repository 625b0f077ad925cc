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


def test_bounded_angles_device_equals_host(cuda):
    import torch
    from barney_gb300.device import _stream
    rng = np.random.default_rng(13)
    v = rng.normal(size=(1_000_003, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    y, x = v[:, 1].astype(np.float32), v[:, 2].astype(np.float32)
    ha, ht = np.empty_like(x), np.empty_like(x)
    assert N.lib().gbv_selftest_angles(y.ctypes.data, x.ctypes.data, x.size, ha.ctypes.data, ht.ctypes.data, 0,
                                       None) == N.GBV_OK
    dy, dx = torch.from_numpy(y).cuda(), torch.from_numpy(x).cuda()
    da, dt = torch.empty_like(dx), torch.empty_like(dx)
    assert N.lib().gbv_selftest_angles(dy.data_ptr(), dx.data_ptr(), x.size, da.data_ptr(), dt.data_ptr(), 1,
                                       _stream()) == N.GBV_OK
    torch.cuda.synchronize()
    np.testing.assert_array_equal(da.cpu().numpy().view(np.uint32), ha.view(np.uint32))
    np.testing.assert_array_equal(dt.cpu().numpy().view(np.uint32), ht.view(np.uint32))
