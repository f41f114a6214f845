"""Determinism (the check that stands in for a race detector, the sanitizer being closed
on this pool): the same seeds run twice in fresh samplers give identical bits.  Covered
are the forms whose reductions span many CTAs or work items -- the GEMM form streamed
through the tensor cores (row super-blocks, partials summed in a fixed order), the batched
engine (row-chunk partials per member), and the resident tensor-core form's statistics --
with CUDA-graph replay on and off."""
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


@pytest.fixture(scope="module")
def M():
    from bayadera_gb300 import models
    return models


def _twice(run):
    a, b = run(True), run(False)          # graphs on, then off
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_streamed_tensor_core_deterministic(factory, M):
    rng = np.random.default_rng(3)
    n, F, W = 20000, 64, 512
    X = rng.normal(size=(n, F)).astype(np.float32)
    y = (rng.random(n) < 0.5).astype(np.float32)
    params = np.concatenate([np.concatenate([X, y[:, None]], axis=1).reshape(-1),
                             np.array([5.0], np.float32)]).astype(np.float32)

    def run(graphs):
        sf = factory.mcmc_factory(M.logistic_model(F), form="gemm", tensor=True)
        s = sf.create_sampler(8, W, params)
        s.set_graphs(graphs)
        s.init_position_normal(9, 0.0, 0.2)
        s.burn_in(40, 2.0)
        r = s.run_sampler(40, 2.0, return_means=True)
        out = (s.positions().copy(), s.logfn().copy(), r["means"].copy())
        s.release()
        sf.release()
        return out
    _twice(run)


def test_batched_engine_deterministic(factory, M):
    rng = np.random.default_rng(4)
    members = []
    for i, J in enumerate((3, 8, 16)):
        ys = [rng.normal(j, 1.0, 30 + 5 * j) for j in range(J)]
        p, rows = M.hierarchical_rows_params(ys, np.ones(J))
        members.append({"dim": J + 2, "seed": 20 + i, "walkers": 256, "params": p, "rows": rows})

    def run(graphs):
        fam = factory.mcmc_factory(M.hierarchical_rows_batch_model(16), form="batch")
        b = fam.create_batch(members)
        b.set_graphs(graphs)
        b.init_position_normal([1, 2, 3], 0.0, 1.0)
        b.burn_in(40, 2.0)
        r = b.run_sampler(40, 2.0, return_means=True)
        out = tuple(x.copy() for x in b.positions()) + tuple(x.copy() for x in b.logfn()) + \
            tuple(m.copy() for m in r["means"]) + (r["acceptance_rates"].copy(),)
        b.release()
        fam.release()
        return out
    _twice(run)


def test_resident_tensor_core_statistics_deterministic(factory, M):
    D, W = 50, 16384
    rng = np.random.default_rng(5)
    A = rng.normal(size=(D, D))
    P = (A @ A.T / D + np.eye(D)).astype(np.float32).reshape(-1)

    def run(graphs):
        sf = factory.mcmc_factory(M.mvn_precision_model(D), form="gemm", tensor=True)
        s = sf.create_sampler(12, W, P)
        s.set_graphs(graphs)
        s.init_position_normal(13, 0.0, 1.0)
        s.burn_in(40, 2.0)
        r = s.run_sampler(70, 2.0, return_means=True)
        out = (s.positions().copy(), s.logfn().copy(), r["means"].copy(),
               np.array([r["acceptance_rate"]]))
        s.release()
        sf.release()
        return out
    _twice(run)
