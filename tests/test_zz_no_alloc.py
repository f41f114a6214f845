"""The allocation-free acor entry point, called through the C ABI.

bay_acor_noalloc serves callers that may not allocate device memory when they call
(a host whose framework allocator owns the device, a loop with a fixed memory budget):
its work space is a fixed scratch array inside the library.  It must give the same
results as bay_acor, call after call (the shared scratch keeps the last call's
contents), and must not change the context's allocation count.
"""
import ctypes as C

import numpy as np
import pytest

from tests.conftest import acor_matrix

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import __graft_entry__
    __graft_entry__.build()
    import torch
    from bayadera_gb300 import _native as N
    from bayadera_gb300.engine import GB300BayaderaFactory
    f = GB300BayaderaFactory(device=0, wgs=256)
    yield N, f, torch
    f.release()


def _acor(N, ctx, fn, series_ptr, D, n, out_dev=None):
    tau, mean, sigma = np.zeros(D), np.zeros(D), np.zeros(D)
    lag = C.c_uint32(0)
    N.call(fn, ctx, series_ptr, D, n, C.c_void_p(tau.ctypes.data), C.c_void_p(mean.ctypes.data),
           C.c_void_p(sigma.ctypes.data), C.byref(lag))
    return tau, mean, sigma, lag.value


def _series(acor_series):
    m367 = acor_matrix(acor_series, 367, "plus 1")                    # 2 x 367
    rng = np.random.default_rng(7)
    x = np.zeros((3, 6000))
    for t in range(1, 6000):                                          # AR(1), 3 dims
        x[:, t] = 0.95 * x[:, t - 1] + rng.normal(size=3)
    return [m367, x.astype(np.float32)]


def test_acor_noalloc_matches_bay_acor(setup, acor_series):
    N, f, torch = setup
    for m in _series(acor_series):
        D, n = m.shape
        host = np.ascontiguousarray(m.T)                              # dim x n column-major
        dev = torch.from_numpy(host.copy()).cuda()
        torch.cuda.synchronize()
        want = _acor(N, f.ctx, "bay_acor", C.c_void_p(host.ctypes.data), D, n)
        before = f.allocated()
        for _ in range(2):                                            # two calls in a row
            got = _acor(N, f.ctx, "bay_acor_noalloc", C.c_void_p(dev.data_ptr()), D, n)
            for g, w in zip(got[:3], want[:3]):
                np.testing.assert_allclose(g, w, rtol=1e-12, atol=1e-15)
            assert got[3] == want[3]
        assert f.allocated() == before


def test_acor_noalloc_rejects_oversize_and_host_input(setup):
    N, f, torch = setup
    big = torch.zeros(2 * 600000, device="cuda")                      # 2 x 600000 > 2^20
    with pytest.raises(N.IllegalArgument):
        _acor(N, f.ctx, "bay_acor_noalloc", C.c_void_p(big.data_ptr()), 2, 600000)
    host = np.zeros(2 * 1000, np.float32)
    with pytest.raises(N.IllegalArgument):
        _acor(N, f.ctx, "bay_acor_noalloc", C.c_void_p(host.ctypes.data), 2, 1000)


def test_acor_noalloc_first_call_on_a_fresh_context(setup, acor_series):
    """bay_acor_noalloc as the very first computation of a new context (the scratch
    array's address was looked up when the context was created), then bay_acor."""
    N, f, torch = setup
    from bayadera_gb300.engine import GB300BayaderaFactory
    m = _series(acor_series)[1]
    D, n = m.shape
    host = np.ascontiguousarray(m.T)
    dev = torch.from_numpy(host.copy()).cuda()
    torch.cuda.synchronize()
    g = GB300BayaderaFactory(device=0, wgs=256)
    try:
        got = _acor(N, g.ctx, "bay_acor_noalloc", C.c_void_p(dev.data_ptr()), D, n)
        want = _acor(N, g.ctx, "bay_acor", C.c_void_p(host.ctypes.data), D, n)
        for a, b in zip(got[:3], want[:3]):
            np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-15)
        assert got[3] == want[3]
    finally:
        g.release()


def test_acor_noalloc_refuses_another_gpus_memory(setup):
    """A series in device memory of a GPU other than the context's is refused before any
    launch (the kernel would read another GPU's memory)."""
    N, f, torch = setup
    if torch.cuda.device_count() < 2:
        pytest.skip("needs a second GPU")
    other = torch.zeros(2 * 1000, device="cuda:1")
    torch.cuda.synchronize(1)
    with pytest.raises(N.IllegalArgument):
        _acor(N, f.ctx, "bay_acor_noalloc", C.c_void_p(other.data_ptr()), 2, 1000)
    with pytest.raises(N.IllegalArgument):
        _acor(N, f.ctx, "bay_acor", C.c_void_p(other.data_ptr()), 2, 1000)
