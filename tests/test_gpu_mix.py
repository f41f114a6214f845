"""mix!'s a-adaptation loop on the device (bay_adapt_a: one CUDA graph, a conditional
WHILE node over the acc-rate! probes) against the same loop run from the host
(bayadera_gb300.mcmc.adapt_a_host, one readback per probe, mcmc.clj:84-91): the same a
sequence's end point, the same number of probes and last rate, and the same sampler
state afterwards (positions, log densities, RNG words), in the plain, resident
tensor-core and streamed forms."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def factory():
    import __graft_entry__
    __graft_entry__.build()
    from bayadera_gb300.engine import GB300BayaderaFactory
    f = GB300BayaderaFactory(device=0, wgs=256)
    yield f
    f.release()


@pytest.mark.parametrize("form", ["plain", "tensor", "streamed"])
def test_adapt_a_device_matches_host(factory, form):
    from bayadera_gb300 import mcmc
    from bayadera_gb300 import models as M
    D, W = 20, 4096
    rng = np.random.default_rng(4)
    A = rng.normal(size=(D, D))
    P = (A @ A.T / D + np.eye(D)).astype(np.float32)
    kw = {"plain": dict(form="plain"), "tensor": dict(form="gemm", tensor=True),
          "streamed": dict(form="gemm", streaming=True)}[form]
    sf = factory.mcmc_factory(M.mvn_precision_model(D), **kw)
    out, times = [], []
    for on_device in (True, False):
        s = sf.create_sampler(9, W, P.reshape(-1))
        s.init_position_normal(10, 0.0, 1.0)
        s.burn_in(20, 2.0)
        # start far from the window (a = 8: acceptance well below 0.2) so the rule runs
        t0 = time.perf_counter()
        if on_device:
            r = s.adapt_a(64, 8.0, 0.2, 0.5)
            res = (r["a"], r["acc_rate"], r["probes"])
        else:
            res = mcmc.adapt_a_host(s, 64, 8.0, 0.2, 0.5)
        times.append(time.perf_counter() - t0)
        pos, lf, rngw = s.export_state()
        out.append((res, pos, lf, rngw, s.info()["iteration_counter"]))
        s.release()
    sf.release()
    (rd, pd, ld, wd, icd), (rh, ph, lh, wh, ich) = out
    print("%s form: a %.6f after %d probes (rate %.4f); device loop %.2f ms, host loop %.2f ms"
          % (form, rd[0], rd[2], rd[1], 1e3 * times[0], 1e3 * times[1]))
    assert rd[2] >= 2
    assert rd[0] == rh[0] and rd[1] == rh[1] and rd[2] == rh[2]
    np.testing.assert_array_equal(pd, ph)
    np.testing.assert_array_equal(ld, lh)
    np.testing.assert_array_equal(wd, wh)
    assert icd == ich


def test_mix_on_device_matches_host(factory):
    """The whole mix! (anneal, adaptation, two burn-ins, two probes) both ways."""
    from bayadera_gb300 import mcmc
    from bayadera_gb300 import models as M
    D, W = 6, 2048
    P = np.diag(np.linspace(0.5, 3.0, D)).astype(np.float32)
    sf = factory.mcmc_factory(M.mvn_precision_model(D), form="plain")
    res = []
    for on_device in (True, False):
        s = sf.create_sampler(3, W, P.reshape(-1))
        s.init_position_normal(4, 0.0, 1.0)
        r = mcmc.mix(s, {"step": 16, "a": 6.0}, on_device=on_device)
        res.append((r, s.positions().copy()))
        s.release()
    sf.release()
    assert res[0][0] == res[1][0]
    np.testing.assert_array_equal(res[0][1], res[1][1])
