"""Checkpoint and resume (bay_state_export / bay_state_import): the walker positions, their
log densities and the counter-based RNG state (seeds, step counters, iteration counter, a,
beta) restart a run bit for bit in a sampler created with another seed -- plain, tiled and
resident tensor-core forms."""
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


def _case(M, form):
    rng = np.random.default_rng(11)
    if form == "tiled":
        data = rng.normal(3.0, 2.0, 500).astype(np.float32)
        params = np.concatenate([data, np.array([0.0, 10.0, 0.0, 20.0], np.float32)])
        return (M.gaussian_posterior_model(), {"form": "tiled"}, params, 1024,
                lambda s: s.init_position(9, [0.0, 6.0, 0.1, 6.0]))
    D = 6 if form == "plain" else 20
    A = rng.normal(size=(D, D))
    P = (A @ A.T / D + np.eye(D)).astype(np.float32).reshape(-1)
    kw = {"form": "plain"} if form == "plain" else {"form": "gemm", "tensor": True}
    return (M.mvn_precision_model(D), kw, P, 2048, lambda s: s.init_position_normal(4, 0.0, 1.0))


def _continue(s):
    s.burn_in(10, 2.0)
    r = s.run_sampler(12, 2.0, return_means=True)
    return s.positions().copy(), s.logfn().copy(), r["means"].copy(), r["acceptance_rate"]


@pytest.mark.parametrize("form", ["plain", "tiled", "tensor"])
def test_export_import_resumes_bit_exact(factory, form):
    from bayadera_gb300 import models as M
    model, kw, params, W, init = _case(M, form)
    sf = factory.mcmc_factory(model, **kw)
    a = sf.create_sampler(5, W, params)
    init(a)
    a.burn_in(10, 2.0)
    a.run_sampler(6, 1.7)                 # the accu seed and counters move too
    state = a.export_state()
    want = _continue(a)
    b = sf.create_sampler(99, W, params)  # another seed: everything comes from the state
    b.import_state(*state)
    got = _continue(b)
    for x, y in zip(want[:3], got[:3]):
        np.testing.assert_array_equal(x, y)
    assert want[3] == got[3]
    assert b.info()["iteration_counter"] == a.info()["iteration_counter"]
    a.release()
    b.release()
    sf.release()
