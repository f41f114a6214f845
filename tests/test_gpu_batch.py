"""Batched engine (bay_batch_*): many independent hierarchical models of uneven dimension,
walkers and data advanced together, against the oracle's FP64 density, the single-model
sampler with the same seed, and an FP64 quadrature of the posterior."""
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


@pytest.fixture(scope="module")
def family(factory, M):
    sf = factory.mcmc_factory(M.hierarchical_rows_batch_model(128), form="batch")
    yield sf
    sf.release()


def _member(M, rng, J, n_lo, n_hi, walkers, seed):
    sig = np.exp(rng.uniform(np.log(0.5), np.log(2.0), J))
    mu, tau = rng.normal(0.0, 3.0), np.exp(rng.normal(0.0, 0.5))
    theta = rng.normal(mu, tau, J)
    ys = [rng.normal(theta[j], sig[j], int(rng.integers(n_lo, n_hi + 1))) for j in range(J)]
    params, rows = M.hierarchical_rows_params(ys, sig)
    return {"dim": J + 2, "seed": seed, "walkers": walkers, "params": params, "rows": rows,
            "ys": ys, "sig": sig}


def _members(M, seed=0):
    rng = np.random.default_rng(seed)
    spec = [(2, 10, 30, 4), (5, 10, 100, 256), (17, 50, 400, 258), (40, 200, 600, 512),
            (3, 3000, 9000, 1024), (128, 10, 40, 256), (9, 0, 0, 64)]
    out = []
    for i, (J, lo, hi, W) in enumerate(spec):
        m = _member(M, rng, J, lo, hi, W, 100 + 7 * i)
        out.append(m)
    return out


def test_batch_logfn_matches_fp64(family, M, oracle):
    """After init-position, every member's log densities against the oracle's FP64 density
    (relative 2e-5: fp32 row terms, Kahan chunk sums, compensated chunk combine).  Members
    span dimension 4..130, 4..1024 walkers, 0..~40000 rows (several row chunks)."""
    mem = _members(M)
    b = family.create_batch(mem)
    b.init_position_normal([11 + i for i in range(len(mem))], 0.0, 1.0)
    pos, lf = b.positions(), b.logfn()
    for m, p, l in zip(mem, pos, lf):
        idx = np.arange(0, m["walkers"], max(1, m["walkers"] // 24))
        want = np.array([oracle.logfn64("hrows", m["params"], 3 * m["rows"], m["dim"],
                                        p[i].astype(np.float64)) for i in idx])
        err = np.abs(l[idx] - want) / np.maximum(np.abs(want), 1.0)
        assert err.max() < 2e-5, (m["dim"], m["rows"], err.max())
    b.release()


def test_batch_member_matches_single_sampler(factory, family, M):
    """Member m uses the single sampler's Philox keys and counters with its seed: the same
    initial walkers bit-for-bit, and after burn-in steps the same walkers except where an
    accept decision is marginal (the two sum the density in different orders)."""
    mem = _members(M, seed=1)[:5]
    b = family.create_batch(mem)
    seeds = [21 + i for i in range(len(mem))]
    b.init_position_normal(seeds, 0.0, 0.5)
    init = [p.copy() for p in b.positions()]
    b.burn_in(6, 2.0)
    got = b.positions()
    for i, m in enumerate(mem):
        sf = factory.mcmc_factory(M.hierarchical_rows_model(m["dim"] - 2), form="plain")
        s = sf.create_sampler(m["seed"], m["walkers"], m["params"])
        s.init_position_normal(seeds[i], 0.0, 0.5)
        np.testing.assert_array_equal(s.positions().T, init[i])
        s.burn_in(6, 2.0)
        differ = np.any(s.positions().T != got[i], axis=1).sum()
        assert differ <= max(2, m["walkers"] // 20), (i, differ)
        s.release()
        sf.release()
    b.release()


def test_batch_graphs_match_direct_launches(family, M):
    """Graph replay and direct launches run the same kernels in the same order: identical
    positions and log densities."""
    mem = _members(M, seed=2)[:4]
    out = []
    for graphs in (True, False):
        b = family.create_batch(mem)
        b.set_graphs(graphs)
        b.init_position_normal([5, 6, 7, 8], 0.0, 1.0)
        b.burn_in(40, 2.0)
        out.append((np.concatenate([p.reshape(-1) for p in b.positions()]),
                    np.concatenate(b.logfn())))
        b.release()
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])


def _posterior_grid(ys, sig, h0=10.0, h1=1.0):
    """E[mu | y] and E[log tau | y] of the hierarchical model by FP64 quadrature over
    u = log tau: theta integrates out exactly (ybar_j | mu, tau ~ N(mu, s_j^2 + tau^2),
    s_j^2 = sigma_j^2 / n_j), then mu (Gaussian)."""
    yb = np.array([np.mean(np.asarray(y, np.float32).astype(np.float64)) for y in ys])
    s2 = np.array([float(np.float32(s)) ** 2 / len(y) for y, s in zip(ys, sig)])
    u = np.linspace(-12.0, 6.0, 40001)
    V = s2[None, :] + np.exp(2.0 * u)[:, None]
    lam = 1.0 / h0 ** 2 + np.sum(1.0 / V, axis=1)
    b = np.sum(yb[None, :] / V, axis=1)
    logp = (-0.5 * np.sum(np.log(V), axis=1) - 0.5 * np.sum(yb[None, :] ** 2 / V, axis=1)
            + 0.5 * b * b / lam - 0.5 * np.log(lam) - 0.5 * u * u / h1 ** 2)
    w = np.exp(logp - logp.max())
    w /= w.sum()
    return float(np.sum(w * b / lam)), float(np.sum(w * u))


def _batch_se(series, nb=16):
    n = series.size // nb * nb
    bm = series[:n].reshape(nb, -1).mean(axis=1)
    return bm.std(ddof=1) / np.sqrt(nb)


def test_batch_posterior_matches_quadrature(family, M):
    """Posterior means of mu and log tau of several members (run means over 2000 steps)
    within 4.5 batch-means standard errors of the FP64 quadrature, and acceptance counts
    per member: the per-step means' last column is the mean of the walkers."""
    rng = np.random.default_rng(7)
    mem = [_member(M, rng, J, lo, hi, W, 300 + i) for i, (J, lo, hi, W) in
           enumerate([(3, 20, 60, 512), (8, 10, 50, 1024), (12, 30, 90, 512), (6, 5, 15, 1024)])]
    b = family.create_batch(mem)
    b.init_position_normal([31, 32, 33, 34], 0.0, 0.5)
    b.burn_in(1500, 2.0)
    r = b.run_sampler(2000, 2.0, return_means=True)
    pos = b.positions()
    for i, m in enumerate(mem):
        a = r["acceptance_rates"][i]
        assert 0.05 < a < 0.95, a
        means = r["means"][i]
        np.testing.assert_allclose(means[:, -1], pos[i].mean(axis=0), rtol=1e-4, atol=1e-5)
        mu_ref, lt_ref = _posterior_grid(m["ys"], m["sig"])
        J = m["dim"] - 2
        for d, ref in ((J, mu_ref), (J + 1, lt_ref)):
            est = means[d].mean()
            se = _batch_se(means[d])
            assert abs(est - ref) <= 4.5 * se + 1e-3, (i, d, est, ref, se)
    b.release()


def test_batch_rejects_bad_members(family, M):
    from bayadera_gb300._native import BayaderaError
    rng = np.random.default_rng(3)
    m = _member(M, rng, 4, 5, 10, 64, 1)
    bad = dict(m, dim=131)
    with pytest.raises(BayaderaError, match="dim"):
        family.create_batch([m, bad])
    with pytest.raises(BayaderaError, match="walkers"):
        family.create_batch([dict(m, walkers=7)])


@pytest.mark.parametrize("shape", [None, {"rows_per_thread": 64, "walkers_per_item": 32,
                                          "walkers_per_thread": 4}])
def test_batch_persistent_matches_per_launch(family, M, shape):
    """One persistent cooperative launch per chunk of steps (every member's proposals, row
    terms and accept phases separated by bounded grid barriers) against three launches per
    half-step: identical positions, log densities, acceptance rates and per-step means (a
    40-step burn-in: a whole chunk and a partial one; a 37-step run)."""
    mem = _members(M, 4)
    out = {}
    for persist in (False, True):
        b = family.create_batch(mem, shape)
        b.set_persistent(persist)
        b.init_position_normal([31 + i for i in range(len(mem))], 0.0, 1.0)
        b.burn_in(40, 2.0)
        r = b.run_sampler(37, 2.0, return_means=True)
        out[persist] = ([p.copy() for p in b.positions()], [l.copy() for l in b.logfn()],
                        np.array(r["acceptance_rates"]), [m.copy() for m in r["means"]])
        b.release()
    a, c = out[False], out[True]
    for x, y in zip(a[0], c[0]):
        np.testing.assert_array_equal(x, y)
    for x, y in zip(a[1], c[1]):
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(a[2], c[2])
    for x, y in zip(a[3], c[3]):
        np.testing.assert_array_equal(x, y)


def test_batch_persistent_many_tiles_per_cta(family, M):
    """The persistent launch with several tiles and work items per CTA (900 small members:
    900 accept tiles against at most one CTA per SM and a few per SM by occupancy), where a
    phase's next tile reuses the CTA's shared memory: identical to three launches per
    half-step, and every log density within 2e-5 relative of FP64."""
    import bench
    rng = np.random.default_rng(9)
    mem = []
    for i in range(900):
        J = int(rng.integers(2, 6))
        mem.append(_member(M, rng, J, 5, 12, 256, 500 + i))
    out = {}
    for persist in (False, True):
        b = family.create_batch(mem, {"rows_per_thread": 32, "walkers_per_item": 64,
                                      "walkers_per_thread": 4})
        b.set_persistent(persist)
        b.init_position_normal([7 + i for i in range(len(mem))], 0.0, 1.0)
        b.burn_in(20, 2.0)
        b.run_sampler(12, 2.0)
        out[persist] = ([p.copy() for p in b.positions()], [l.copy() for l in b.logfn()])
        b.release()
    for x, y in zip(out[False][0], out[True][0]):
        np.testing.assert_array_equal(x, y)
    for x, y in zip(out[False][1], out[True][1]):
        np.testing.assert_array_equal(x, y)
    for i in range(0, 900, 97):
        m, pos, lf = mem[i], out[True][0][i], out[True][1][i]
        want = bench.fp64_hrows(m["params"], m["rows"], pos.astype(np.float64))
        assert np.all(np.abs(lf - want) <= 2e-5 * np.abs(want) + 1e-3), i


def test_batch_grid_barrier_runs_out_and_context_recovers(family, M):
    """Device failure path without a fault: armed, the persistent launch's grid barriers
    wait for one CTA more than the launch has; every CTA gives up after its bounded wait
    (2 s), raises the abort flag and the status word, and the launch ends.  The host reads
    the status (BAY_ERR_DEVICE, naming the grid barrier); a new batch on the same context
    then runs normally."""
    import time
    from bayadera_gb300._native import BayaderaError, BAY_ERR_DEVICE
    mem = _members(M, 5)
    b = family.create_batch(mem)
    b.set_persistent(True)
    b.init_position_normal([1 + i for i in range(len(mem))], 0.0, 1.0)
    b.arm_barrier_timeout(True)
    t0 = time.perf_counter()
    with pytest.raises(BayaderaError, match="grid barrier") as e:
        b.run_sampler(8, 2.0)
    assert e.value.code == BAY_ERR_DEVICE
    assert time.perf_counter() - t0 < 60.0
    b.release()
    b = family.create_batch(mem)
    b.set_persistent(True)
    b.init_position_normal([1 + i for i in range(len(mem))], 0.0, 1.0)
    r = b.run_sampler(16, 2.0)
    assert np.all((np.array(r["acceptance_rates"]) > 0.05) & (np.array(r["acceptance_rates"]) < 0.95))
    b.release()
