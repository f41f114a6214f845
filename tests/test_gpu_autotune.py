"""The autotuner (bay_autotune, bay_batch_autotune) and the shapes it chooses between.

* Shapes that do not change the order of the log-density sums give identical bits: the
  resident tensor-core form's tile groups per CTA (1 or 2), the streamed tensor-core form's
  ring stages at a fixed sub-tile count.
* Shapes that do change it stay within the stated tolerance of the FP64 density: the tiled
  form's (walkers per CTA, CTA threads) pairs (relative 2e-6: compensated sums), the
  streamed form's sub-tile counts, the batched engine's work-list shapes (2e-5).
* The tuner returns one of its candidates, its time is no worse than the default's, and a
  second call comes from the cache.
"""
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


def _c1_params(n=4000):
    rng = np.random.default_rng(0)
    data = rng.normal(3.0, 2.0, n).astype(np.float32)
    return np.concatenate([data, np.array([0.0, 10.0, 0.0, 20.0], np.float32)])


def _fp64_c1(params, pos):
    import bench
    return bench.fp64_c1(params, pos)


@pytest.mark.parametrize("n", [4000, 30001])
def test_tiled_shapes_match_fp64(factory, M, n):
    """Every tiled-form shape the tuner tries, on one chunk of staged rows (4,000) and on
    three chunks with a ragged tail (30,001 rows, not a multiple of 4): log densities of the
    initial and moved walkers within 2e-6 relative of FP64."""
    params = _c1_params(n)
    W = 1024
    for wpc, cta in ((8, 256), (2, 256), (4, 512), (16, 256), (32, 256), (32, 1024)):
        sf = factory.mcmc_factory(M.gaussian_posterior_model(), form="tiled", walkers_per_cta=wpc,
                                  cta_threads=cta)
        s = sf.create_sampler(5, W, params)
        s.init_position(6, [2.0, 4.0, 1.0, 3.0])
        for phase in range(2):
            pos = s.positions().T.astype(np.float64)
            want = _fp64_c1(params, pos)
            err = np.abs(s.logfn() - want) / np.abs(want)
            assert err.max() < 2e-6, (wpc, cta, phase, err.max())
            s.burn_in(3, 2.0)
        s.release()
        sf.release()


@pytest.mark.parametrize("n", [10000, 30001])
def test_tiled_row_slices(factory, M, n):
    """The tiled form split into row slices (each slice's CTA sums its rows, the group's
    last CTA combines them in slice order): log densities of the moved walkers within 2e-6
    relative of FP64 for 2, 4 and 8 slices (30,001 rows: ragged slices over several staged
    chunks); the same seed gives the same bits twice (the combine order does not depend
    on which CTA finishes last); the run's per-step means agree with the mean of the
    positions it ends on."""
    params = _c1_params(n)
    W = 2048
    for sl in (2, 4, 8):
        runs = []
        for rep in range(2):
            sf = factory.mcmc_factory(M.gaussian_posterior_model(), form="tiled", walkers_per_cta=8,
                                      cta_threads=128, tile_slices=sl)
            s = sf.create_sampler(9, W, params)
            s.init_position(10, [2.0, 4.0, 1.0, 3.0])
            s.burn_in(6, 2.0)
            r = s.run_sampler(5, 2.0, return_means=True)
            pos = s.positions().T.astype(np.float64)
            want = _fp64_c1(params, pos)
            err = np.abs(s.logfn() - want) / np.abs(want)
            assert err.max() < 2e-6, (sl, err.max())
            np.testing.assert_allclose(r["means"][:, -1], s.mean(), rtol=1e-5, atol=1e-6)
            assert 0.3 < r["acceptance_rate"] < 0.95
            runs.append((s.positions().copy(), s.logfn().copy()))
            s.release()
            sf.release()
        np.testing.assert_array_equal(runs[0][0], runs[1][0])
        np.testing.assert_array_equal(runs[0][1], runs[1][1])


@pytest.mark.parametrize("n", [0, 3, 257])
def test_tiled_row_slices_few_rows(factory, M, n):
    """Row slices with fewer rows than slices x 4 (empty slices; no data at all): the log
    densities are the prior (n = 0) or the few rows' sum, within 2e-6 relative of FP64,
    for 1 and 8 slices."""
    rng = np.random.default_rng(n)
    params = np.concatenate([rng.normal(3.0, 2.0, n).astype(np.float32),
                             np.array([0.0, 10.0, 0.0, 20.0], np.float32)])
    for sl in (1, 8):
        sf = factory.mcmc_factory(M.gaussian_posterior_model(), form="tiled", walkers_per_cta=8,
                                  cta_threads=256, tile_slices=sl)
        s = sf.create_sampler(5, 512, params)
        s.init_position(6, [2.0, 4.0, 1.0, 3.0])
        s.burn_in(4, 2.0)
        pos = s.positions().T.astype(np.float64)
        want = _fp64_c1(params, pos)
        err = np.abs(s.logfn() - want) / np.abs(want)
        assert err.max() < 2e-6, (n, sl, err.max())
        s.release()
        sf.release()


def test_resident_tile_groups_bit_identical(factory, M):
    """Resident tensor-core form, 50-D target: one or two tile groups per CTA give the same
    positions, log densities, per-step means and acceptance (a partial last tile)."""
    import bench
    P, _ = bench.precision_matrix()
    W = 2 * (64 * 37 + 11)
    out = []
    for groups in (1, 2):
        sf = factory.mcmc_factory(M.mvn_precision_model(50), form="gemm", tensor=True,
                                  tc_groups=groups)
        s = sf.create_sampler(3, W, P.reshape(-1))
        s.init_position_normal(4, 0.0, 1.0)
        s.burn_in(40, 2.0)
        r = s.run_sampler(37, 2.0, return_means=True)
        out.append((s.positions().copy(), s.logfn().copy(), r["means"].copy(),
                    r["acceptance_rate"]))
        s.release()
        sf.release()
    a, b = out
    for x, y in zip(a[:3], b[:3]):
        np.testing.assert_array_equal(x, y)
    assert a[3] == b[3]


def test_streamed_tc_stages_bit_identical_subtiles_within_bound(factory, M, oracle):
    """Streamed tensor-core form (logistic regression, 3,000 rows): the ring's depth does not
    change the sums (2 and 4 stages at 2 sub-tiles: identical bits); one sub-tile per CTA
    changes the row-block partition, so its log densities are checked against FP64 within
    the split-bf16 bound."""
    rng = np.random.default_rng(2)
    n, F, W = 3000, 16, 512
    X = rng.normal(size=(n, F)).astype(np.float32)
    beta = rng.normal(scale=0.25, size=F)
    y = (rng.random(n) < 1.0 / (1.0 + np.exp(-(X.astype(np.float64) @ beta)))).astype(np.float32)
    params = np.concatenate([np.concatenate([X, y[:, None]], axis=1).reshape(-1),
                             np.array([5.0], np.float32)]).astype(np.float32)
    res = {}
    for g, st in ((2, 2), (2, 4), (1, 3)):
        sf = factory.mcmc_factory(M.logistic_model(F), form="gemm", tensor=True, tc_subtiles=g,
                                  tc_stages=st)
        s = sf.create_sampler(7, W, params)
        s.init_position_normal(8, 0.0, 0.3)
        s.burn_in(4, 2.0)
        res[(g, st)] = (s.positions().copy(), s.logfn().copy())
        s.release()
        sf.release()
    np.testing.assert_array_equal(res[(2, 2)][0], res[(2, 4)][0])
    np.testing.assert_array_equal(res[(2, 2)][1], res[(2, 4)][1])
    pos, lf = res[(1, 3)][0].T.astype(np.float64), res[(1, 3)][1]
    for k in range(0, W, 37):
        want = oracle.logfn64("logistic", params, n * (F + 1), F, pos[k])
        bound = (2.0 ** -15 + 4 * F * 2.0 ** -24) * float(np.sum(np.abs(X) @ np.abs(pos[k])))
        assert abs(lf[k] - want) <= bound + 1e-5 * abs(want) + 1e-3


def test_autotune_tiled_and_cache(factory, M):
    """bay_autotune on the 2-D posterior (4,096 walkers, 10,000 rows): the chosen shape is
    one of the tiled candidates, timed no slower than the default, and compiles and runs;
    the second call returns the same shape from the cache."""
    params = _c1_params(10000)
    model = M.gaussian_posterior_model()
    r = factory.autotune(model, 4096, params, form="tiled")
    print("tiled autotune: %s, %.1f us per step (default %.1f us), %d candidates"
          % (r["shape"], r["us_per_step"], r["default_us_per_step"], r["candidates"]))
    assert r["candidates"] >= 2 and not r["from_cache"]
    assert r["us_per_step"] <= r["default_us_per_step"]
    assert r["shape"].get("tile_slices", 1) in (1, 2, 4, 8, 16)
    assert (r["shape"]["walkers_per_cta"], r["shape"]["cta_threads"]) in (
        (8, 256), (2, 256), (4, 256), (4, 512), (4, 128), (8, 128), (16, 256), (32, 256),
        (8, 512), (16, 512), (32, 512), (32, 1024))
    r2 = factory.autotune(model, 4096, params, form="tiled")
    assert r2["from_cache"] and r2["shape"] == r["shape"]
    sf = factory.mcmc_factory(model, form="tiled", **r["shape"])
    s = sf.create_sampler(1, 4096, params)
    s.init_position(2, [2.0, 4.0, 1.0, 3.0])
    s.burn_in(10, 2.0)
    pos = s.positions().T.astype(np.float64)
    err = np.abs(s.logfn() - _fp64_c1(params, pos)) / np.abs(_fp64_c1(params, pos))
    assert err.max() < 2e-6
    s.release()
    sf.release()


def test_autotune_resident_groups(factory, M):
    """bay_autotune on the resident tensor-core form picks tile groups 1 or 2."""
    import bench
    P, _ = bench.precision_matrix()
    r = factory.autotune(M.mvn_precision_model(50), 65536, P.reshape(-1), form="gemm", tensor=True)
    print("resident tensor-core autotune: %s, %.2f us per step (default %.2f us)"
          % (r["shape"], r["us_per_step"], r["default_us_per_step"]))
    assert r["shape"].get("tc_groups") in (1, 2)
    assert r["us_per_step"] <= r["default_us_per_step"]


def test_batch_shapes_and_autotune(factory, M, oracle):
    """Batched engine: two work-list shapes give log densities within 2e-5 of FP64 for every
    member; bay_batch_autotune returns a valid shape and caches it."""
    rng = np.random.default_rng(3)
    fam = factory.mcmc_factory(M.hierarchical_rows_batch_model(16), form="batch")
    members = []
    for i, J in enumerate((2, 5, 11, 16)):
        ys = [rng.normal(j, 1.0, 40 + 13 * j) for j in range(J)]
        p, rows = M.hierarchical_rows_params(ys, np.ones(J))
        members.append({"dim": J + 2, "seed": 10 + i, "walkers": 256, "params": p, "rows": rows})
    for shape in ({"rows_per_thread": 32, "walkers_per_item": 16},
                  {"rows_per_thread": 512, "walkers_per_item": 64}):
        b = fam.create_batch(members, shape)
        b.init_position_normal([1, 2, 3, 4], 0.0, 1.0)
        b.burn_in(5, 2.0)
        for m, pos, lf in zip(members, b.positions(), b.logfn()):
            for k in range(0, 256, 31):
                want = oracle.logfn64("hrows", m["params"], 3 * m["rows"], m["dim"],
                                      pos[k].astype(np.float64))
                assert abs(lf[k] - want) <= 2e-5 * abs(want) + 1e-3
        b.release()
    r = fam.autotune_batch(members)
    print("batch autotune: %s, %.1f us per step (default %.1f us), %d candidates"
          % (r["shape"], r["us_per_step"], r["default_us_per_step"], r["candidates"]))
    assert r["shape"]["walkers_per_item"] in (16, 32, 64)
    assert r["us_per_step"] <= r["default_us_per_step"]
    assert fam.autotune_batch(members)["from_cache"]
    fam.release()


def test_batch_walkers_per_thread_bit_identical(factory, M):
    """The row-term kernel with 4 walkers per thread shares each staged row between them;
    with the same row groups per walker (16 walkers per item at 1 per thread, 64 at 4 per
    thread: 16 row groups each) and the same row chunks (chunk_floats caps them at 256
    rows), every walker's sum has the same order: identical positions and log densities."""
    rng = np.random.default_rng(5)
    fam = factory.mcmc_factory(M.hierarchical_rows_batch_model(16), form="batch")
    members = []
    for i, J in enumerate((2, 7, 16)):
        ys = [rng.normal(j, 1.0, 100 + 29 * j) for j in range(J)]
        p, rows = M.hierarchical_rows_params(ys, np.ones(J))
        members.append({"dim": J + 2, "seed": 20 + i, "walkers": 256, "params": p, "rows": rows})
    out = []
    for shape in ({"rows_per_thread": 512, "walkers_per_item": 16, "chunk_floats": 1024,
                   "walkers_per_thread": 1},
                  {"rows_per_thread": 512, "walkers_per_item": 64, "chunk_floats": 1024,
                   "walkers_per_thread": 4}):
        b = fam.create_batch(members, shape)
        b.init_position_normal([5, 6, 7], 0.0, 1.0)
        b.burn_in(6, 2.0)
        out.append(([p.copy() for p in b.positions()], [l.copy() for l in b.logfn()]))
        b.release()
    fam.release()
    for pa, pb in zip(out[0][0], out[1][0]):
        np.testing.assert_array_equal(pa, pb)
    for la, lb in zip(out[0][1], out[1][1]):
        np.testing.assert_array_equal(la, lb)
