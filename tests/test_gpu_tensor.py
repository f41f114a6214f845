"""GEMM form on the tensor cores (tcgen05, split bf16, fp32 accumulation) against exact
and FP64 references.

Error model of the split form: each factor is stored as bf16 hi + lo (residual below
2^-17 relative), the products hi.hi + hi.lo + lo.hi are summed in fp32 on the tensor
cores and lo.lo (below 2^-16 relative) is dropped, so each product term x_f b_f carries a
relative error below 2^-15, plus fp32 accumulation over the F terms.  The tests bound
|logfn_tc - logfn_exact| by

    sum_r |d term_r / d eta_r| (2^-15 + 4 F 2^-24) sum_f |x_rf b_f|  +  fp32 term rounding,

and, on inputs that bf16 hi + lo represents exactly, check the kernel against the exact
split-product sum with only the accumulation term left (a dropped hi.lo or lo.hi
product, a swizzle or layout slip would be off by 2^-9 or more)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LINEAR_SRC = r"""
#include <stdint.h>
extern "C" {
inline REAL tclin_logpdf(const uint32_t data_len, const uint32_t hyper_len,
                         const REAL* params, const uint32_t dim, const REAL* x) {
    const uint32_t row = dim + 1, n = data_len / row;
    REAL res = 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        const REAL* r = params + (uint64_t)i * row;
        REAL eta = 0.0f;
        for (uint32_t f = 0; f < dim; ++f) eta = fmaf(r[f], x[f], eta);
        res += eta * r[dim];
    }
    return res;
}
inline void tclin_prep(const REAL* h, const uint32_t hl, const uint32_t dim, const REAL* x,
                       REAL* prep) {}
inline REAL tclin_term(const REAL eta, const REAL* aux, const uint64_t row, const REAL* x,
                       const REAL* prep) {
    return eta * aux[0];
}
inline REAL tclin_walker(const uint64_t rows, const REAL* h, const uint32_t hl,
                         const uint32_t dim, const REAL* x) {
    return 0.0f;
}
}
"""


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


def linear_model(M, F):
    g = {"prep": "tclin_prep", "term": "tclin_term", "walker": "tclin_walker",
         "features": F, "coef": 0, "block": "data", "ld": F + 1, "offset": 0,
         "aux_col": F, "aux_len": 1}
    return M.device_distribution_model(LINEAR_SRC, name="tclin", logpdf="tclin_logpdf",
                                       dimension=F, params_size=1, gemm=g)


def bf16_rn(v):
    """bf16 round-to-nearest-even of float32 values, returned as float64."""
    u = np.ascontiguousarray(v, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


def split(v):
    v = np.asarray(v, np.float32)
    hi = bf16_rn(v)
    lo = bf16_rn((v.astype(np.float64) - hi).astype(np.float32))
    return hi, lo


def sixteen_bit(rng, shape, scale):
    """float32 values with 16 significant bits (exact as bf16 hi + lo), mixed signs and
    exponents."""
    v = (rng.normal(size=shape) * scale * np.exp2(rng.integers(-3, 4, size=shape))).astype(np.float32)
    return (v.view(np.uint32) & np.uint32(0xFFFFFF00)).view(np.float32)


@pytest.mark.parametrize("rows,F,W", [(1000, 64, 512), (300, 7, 200), (777, 130, 260),
                                      (128, 256, 256), (200, 320, 130), (5000, 64, 1024),
                                      (50, 50, 512), (100, 7, 258), (256, 64, 130),
                                      (16, 130, 200)])
def test_tc_eta_exact_split_products(factory, M, rows, F, W):
    """Linear row term (term = eta_r w_r): with every factor exact in bf16 hi + lo the
    kernel must equal sum_r w_r sum_f (xh bh + xh bl + xl bh) up to fp32 accumulation.
    Streamed form (rows > 256 or a large operand): rows and walkers not multiples of the
    128 tiles, features padded to 64, one and two walker sub-tiles per CTA, 1..5 feature
    chunks.  Resident form (the last four: rows <= 256, one launch per half-step): N =
    rows padded to 16, 1..3 feature atoms, partial walker tiles."""
    rng = np.random.default_rng(rows + F)
    X = sixteen_bit(rng, (rows, F), 1.0)
    w = sixteen_bit(rng, rows, 1.0)
    pos = sixteen_bit(rng, (W, F), 0.5)
    params = np.concatenate([np.concatenate([X, w[:, None]], axis=1).reshape(-1),
                             np.zeros(1, np.float32)]).astype(np.float32)
    sf = factory.mcmc_factory(linear_model(M, F), form="gemm", tensor=True)
    s = sf.create_sampler(3, W, params)
    s.init_position(pos)
    got = s.logfn().astype(np.float64)
    xh, xl = split(X)
    bh, bl = split(pos)
    eta = bh @ xh.T + bl @ xh.T + bh @ xl.T                      # (W, rows), exact in fp64
    want = eta @ w.astype(np.float64)
    mag = (np.abs(pos).astype(np.float64) @ np.abs(X).T.astype(np.float64)) @ np.abs(w).astype(np.float64)
    tol = 4 * F * 2.0 ** -24 * mag + 2.0 ** -22 * (np.abs(eta) @ np.abs(w).astype(np.float64)) + 1e-30
    err = np.abs(got - want)
    assert np.all(err <= tol), (err / tol).max()
    # and the split-product sum is itself within the 2^-15 model of the exact sum
    exact = (pos.astype(np.float64) @ X.T.astype(np.float64)) @ w.astype(np.float64)
    assert np.all(np.abs(want - exact) <= 2.0 ** -15 * mag)
    s.release()
    sf.release()


LINEAR_OFS_SRC = r"""
#include <stdint.h>
extern "C" {
inline REAL NAME_logpdf(const uint32_t data_len, const uint32_t hyper_len,
                        const REAL* params, const uint32_t dim, const REAL* x) {
    const uint32_t nf = dim - COEF, row = nf + 1, n = data_len / row;
    REAL res = 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        const REAL* r = params + (uint64_t)i * row;
        REAL eta = 0.0f;
        for (uint32_t f = 0; f < nf; ++f) eta = fmaf(r[f], x[COEF + f], eta);
        res += eta * r[nf];
    }
    return res;
}
inline void NAME_prep(const REAL* h, const uint32_t hl, const uint32_t dim, const REAL* x,
                      REAL* prep) {}
inline REAL NAME_term(const REAL eta, const REAL* aux, const uint64_t row, const REAL* x,
                      const REAL* prep) {
    return eta * aux[0];
}
inline REAL NAME_walker(const uint64_t rows, const REAL* h, const uint32_t hl,
                        const uint32_t dim, const REAL* x) {
    return 0.0f;
}
}
"""


@pytest.mark.parametrize("rows,F,coef,W", [(100, 20, 1, 300), (64, 64, 3, 130)])
def test_tcr_exact_split_products_coefficient_offset(factory, M, rows, F, coef, W):
    """Resident form with the coefficients at walker dims coef .. coef + F - 1 (the A
    operand taken from the staged rows, not from the gather): the exact split-product sum
    as in the test above."""
    name = "tclo%d" % coef
    src = LINEAR_OFS_SRC.replace("NAME", name).replace("COEF", str(coef))
    g = {"prep": name + "_prep", "term": name + "_term", "walker": name + "_walker",
         "features": F, "coef": coef, "block": "data", "ld": F + 1, "offset": 0,
         "aux_col": F, "aux_len": 1}
    model = M.device_distribution_model(src, name=name, logpdf=name + "_logpdf",
                                        dimension=F + coef, params_size=1, gemm=g)
    rng = np.random.default_rng(rows + F + coef)
    X = sixteen_bit(rng, (rows, F), 1.0)
    w = sixteen_bit(rng, rows, 1.0)
    pos = sixteen_bit(rng, (W, F + coef), 0.5)
    params = np.concatenate([np.concatenate([X, w[:, None]], axis=1).reshape(-1),
                             np.zeros(1, np.float32)]).astype(np.float32)
    sf = factory.mcmc_factory(model, form="gemm", tensor=True)
    s = sf.create_sampler(3, W, params)
    s.init_position(pos)
    got = s.logfn().astype(np.float64)
    xh, xl = split(X)
    bh, bl = split(pos[:, coef:])
    eta = bh @ xh.T + bl @ xh.T + bh @ xl.T
    want = eta @ w.astype(np.float64)
    mag = (np.abs(pos[:, coef:]).astype(np.float64) @ np.abs(X).T.astype(np.float64)) @ \
        np.abs(w).astype(np.float64)
    tol = 4 * F * 2.0 ** -24 * mag + 2.0 ** -22 * (np.abs(eta) @ np.abs(w).astype(np.float64)) + 1e-30
    err = np.abs(got - want)
    assert np.all(err <= tol), (err / tol).max()
    s.release()
    sf.release()


def _regression(rng, n, F, kind):
    X = rng.normal(size=(n, F)).astype(np.float32)
    beta = rng.normal(scale=1.0 / np.sqrt(F), size=F)
    eta = X.astype(np.float64) @ beta
    if kind == "logistic":
        y = (rng.random(n) < 1.0 / (1.0 + np.exp(-eta))).astype(np.float32)
        hyper = np.array([5.0], np.float32)
    else:
        y = (eta + 0.5 * rng.standard_t(4, n)).astype(np.float32)
        hyper = np.array([4.0, 10.0, 1.0], np.float32)
    rows = np.concatenate([X, y[:, None]], axis=1).astype(np.float32)
    return np.concatenate([rows.reshape(-1), hyper]), rows.size, X, hyper


def _bound(kind, X, hyper, pos, F, lf64):
    """Per-walker bound on |logfn_tc - logfn_fp64| (module docstring)."""
    b = pos[:, :F].astype(np.float64)
    mag_rows = np.abs(b) @ np.abs(X.astype(np.float64)).T       # (W, rows)
    if kind == "logistic":
        sens = np.ones(len(pos))
    else:
        nu = float(hyper[0])
        sens = (nu + 1.0) / (2.0 * np.sqrt(nu)) * np.exp(-pos[:, F].astype(np.float64))
    eta_err = (2.0 ** -15 + 4 * F * 2.0 ** -24) * mag_rows.sum(axis=1)
    rows = X.shape[0]
    return sens * eta_err + 1e-6 * rows + 1e-5 * np.abs(lf64)


@pytest.mark.parametrize("kind,rows,F,W", [("logistic", 3000, 64, 512),
                                           ("logistic", 1000, 7, 1000),
                                           ("robust_t", 700, 255, 300),
                                           ("robust_t", 2000, 64, 258)])
def test_tc_logfn_within_bound_of_fp64(factory, M, oracle, kind, rows, F, W):
    """Model log densities (logistic softplus terms, Student-t terms) of the initial and of
    moved walkers against the oracle's FP64 density, within the split-bf16 bound."""
    rng = np.random.default_rng(11)
    params, dl, X, hyper = _regression(rng, rows, F, kind)
    model = M.logistic_model(F) if kind == "logistic" else M.robust_t_model(F)
    D = model.dimension
    sf = factory.mcmc_factory(model, form="gemm", tensor=True)
    s = sf.create_sampler(5, W, params)
    s.init_position_normal(6, 0.0, 0.3)
    for phase in range(2):
        pos = s.positions().T.astype(np.float64)
        lf = s.logfn().astype(np.float64)
        idx = np.arange(0, W, max(1, W // 64))
        want = np.array([oracle.logfn64(kind, params, dl, D, pos[i]) for i in idx])
        tol = _bound(kind, X, hyper, pos[idx].astype(np.float32), F, want)
        err = np.abs(lf[idx] - want)
        assert np.all(err <= tol), (phase, (err / tol).max())
        s.burn_in(2, 2.0)
    s.release()
    sf.release()


def test_tc_matches_simt_streaming(factory, M):
    """Same seeds, tensor-core and fp32 SIMT streamed forms: log densities at the same
    positions agree within the split-bf16 bound, and the first moves make the same
    accept decisions except for marginal ones."""
    rng = np.random.default_rng(21)
    F, rows, W = 64, 20000, 2048
    params, dl, X, hyper = _regression(rng, rows, F, "logistic")
    out = []
    for tensor in (False, True):
        sf = factory.mcmc_factory(M.logistic_model(F), form="gemm", streaming=True,
                                  tensor=tensor)
        s = sf.create_sampler(7, W, params)
        s.init_position_normal(8, 0.0, 0.05)
        lf0 = s.logfn().copy()
        s.burn_in(3, 2.0)
        out.append((lf0, s.positions().copy()))
        s.release()
        sf.release()
    d = np.abs(out[0][0].astype(np.float64) - out[1][0])
    assert np.median(d) < 0.05, np.median(d)
    walkers_differ = np.any(out[0][1] != out[1][1], axis=0).sum()
    assert walkers_differ <= W // 50, walkers_differ


def test_tc_run_sampler_statistics(factory, M):
    """Accu path on the tensor cores: acceptance count, per-step means (last = mean of the
    walkers), and posterior means within max(5 MC standard errors, 0.1 posterior sd) of
    the fp32 SIMT form (same seeds, so the two chains share their Philox draws until a
    marginal accept decision differs)."""
    rng = np.random.default_rng(4)
    F = 8
    params, dl, X, hyper = _regression(rng, 5000, F, "robust_t")
    res = {}
    for tensor in (False, True):
        sf = factory.mcmc_factory(M.robust_t_model(F), form="gemm", streaming=True,
                                  tensor=tensor)
        s = sf.create_sampler(8, 2048, params)
        s.init_position_normal(9, 0.0, 0.2)
        s.burn_in(1000, 2.0)
        r = s.run_sampler(512, 2.0, return_means=True)
        assert 0.1 < r["acceptance_rate"] < 0.9
        np.testing.assert_allclose(r["means"][:, -1], s.mean(), rtol=1e-5, atol=1e-6)
        m = r["means"].mean(axis=1)
        ac = r["autocorrelation"]
        # MC s.e. of the run mean, sqrt(var tau / (W n)), with tau at least 50 (acor on a
        # 512-step run can under- or misestimate it, even return a negative D)
        tau = np.asarray(ac.tau, np.float64) if ac is not None else np.full(F + 1, np.nan)
        tau = np.where(np.isfinite(tau), np.maximum(tau, 50.0), 50.0)
        se = np.sqrt(s.variance() * tau / (2048 * 512))
        res[tensor] = (m, se, r["acceptance_rate"], np.sqrt(s.variance()))
        s.release()
        sf.release()
    (m0, se0, a0, sd0), (m1, se1, a1, sd1) = res[False], res[True]
    se = np.sqrt(se0 ** 2 + se1 ** 2)
    d = np.abs(m0 - m1)
    assert np.all(d <= np.maximum(5 * se, 0.1 * np.minimum(sd0, sd1))), (d / se, d / sd0)
    n = 2048 * 512
    assert abs(a0 - a1) <= 3 * np.sqrt(2 * a0 * (1 - a0) / n) + 0.01


def test_tc_rejects_too_many_features(factory, M):
    from bayadera_gb300._native import BayaderaError
    with pytest.raises(BayaderaError, match="320 features"):
        factory.mcmc_factory(M.logistic_model(384), form="gemm", tensor=True)


def test_tcr_mvn_logfn_and_moves(factory, M, oracle):
    """Resident tensor-core form on a 50-D Gaussian (precision matrix as the MMA's B
    operand): log densities of the initial and moved walkers against the oracle's FP64
    density within the split-bf16 bound (term = -x_r eta_r / 2), and the same moves as
    the fp32 SIMT resident form except for marginal accept decisions."""
    D, W = 50, 2048
    rng = np.random.default_rng(5)
    A = rng.normal(size=(D, D))
    P = (A @ A.T / D + np.eye(D)).astype(np.float32)
    out = []
    for tensor in (True, False):
        sf = factory.mcmc_factory(M.mvn_precision_model(D), form="gemm", tensor=tensor)
        s = sf.create_sampler(11, W, P.reshape(-1))
        s.init_position_normal(3, 0.0, 1.0)
        for phase in range(2):
            if tensor:
                pos = s.positions().T.astype(np.float64)
                lf = s.logfn().astype(np.float64)
                idx = np.arange(0, W, 32)
                want = np.array([oracle.logfn64("mvn_precision", P.reshape(-1), 0, D, pos[i])
                                 for i in idx])
                x = pos[idx]
                mag = 0.5 * np.sum(np.abs(x) * (np.abs(x) @ np.abs(P.astype(np.float64)).T), axis=1)
                tol = (2.0 ** -15 + 4 * D * 2.0 ** -24) * mag + 1e-5 * np.abs(want) + 1e-5
                err = np.abs(lf[idx] - want)
                assert np.all(err <= tol), (phase, (err / tol).max())
            s.burn_in(2, 2.0)
        out.append(s.positions().copy())
        s.release()
        sf.release()
    differ = np.any(out[0] != out[1], axis=0).sum()
    assert differ <= W // 25, differ


def test_tcr_c2_matrix_logfn_error(factory, M, oracle):
    """The 50-D benchmark's own target: the AR(1) rho = 0.9 precision matrix with scales
    log-uniform in [0.1, 10] (entries from 0.1 to 929, strong cancellation in x'Px), 4,096
    walkers after 300 burn-in steps (near the posterior).  The resident tensor-core form's
    log densities against the oracle's FP64 density: every walker within the split-bf16
    bound (2^-15 + 4 D 2^-24) sum_r |x_r| sum_c |P_rc x_c| / 2; the measured error, and the
    fp32 SIMT form's beside it, are printed."""
    import bench
    D, W = 50, 4096
    P, _ = bench.precision_matrix()
    P64 = P.astype(np.float64)
    for tensor in (True, False):
        sf = factory.mcmc_factory(M.mvn_precision_model(D), form="gemm", tensor=tensor)
        s = sf.create_sampler(13, W, P.reshape(-1))
        s.init_position_normal(3, 0.0, 1.0)
        s.burn_in(300, 2.0)
        pos = s.positions().T.astype(np.float64)
        lf = s.logfn().astype(np.float64)
        want = -0.5 * np.einsum("wi,ij,wj->w", pos, P64, pos)
        mag = 0.5 * np.einsum("wi,ij,wj->w", np.abs(pos), np.abs(P64), np.abs(pos))
        err = np.abs(lf - want)
        print("%s form: |logfn - FP64| max %.3g, median %.3g; relative max %.3g; "
              "bound median %.3g" % ("tensor-core" if tensor else "fp32 SIMT", err.max(),
                                     np.median(err), (err / np.abs(want)).max(),
                                     np.median((2.0 ** -15 + 4 * D * 2.0 ** -24) * mag)))
        if tensor:
            tol = (2.0 ** -15 + 4 * D * 2.0 ** -24) * mag + 1e-6 * np.abs(want) + 1e-6
        else:
            tol = 4 * D * 2.0 ** -24 * mag + 1e-6 * np.abs(want) + 1e-6
        assert np.all(err <= tol), (err / tol).max()
        s.release()
        sf.release()


@pytest.mark.parametrize("D", [10, 63, 64, 80])
def test_tcr_run_sampler_matches_simt(factory, M, D):
    """Resident tensor-core accu path: acceptance rate within 3 binomial s.e. of the SIMT
    form's, per-step means (last = mean of the walkers).  The per-dim sums run in 256 / D
    walker groups: 8 groups for D = 10, 4 for D = 63 and 64, 3 for D = 80."""
    W = 4096
    P = np.diag(np.linspace(0.5, 2.0, D)).astype(np.float32)
    rates = {}
    for tensor in (True, False):
        sf = factory.mcmc_factory(M.mvn_precision_model(D), form="gemm", tensor=tensor)
        s = sf.create_sampler(17, W, P.reshape(-1))
        s.init_position_normal(2, 0.0, 1.0)
        s.burn_in(100, 2.0)
        r = s.run_sampler(200, 2.0, return_means=True)
        np.testing.assert_allclose(r["means"][:, -1], s.mean(), rtol=1e-5, atol=1e-6)
        rates[tensor] = r["acceptance_rate"]
        s.release()
        sf.release()
    a = rates[False]
    assert abs(rates[True] - a) <= 3 * np.sqrt(2 * a * (1 - a) / (W * 200)) + 0.005


@pytest.mark.parametrize("D,W", [(50, 4096), (10, 89600), (64, 2 * (64 * 5 + 17))])
def test_tcr_persistent_matches_per_launch(factory, M, D, W):
    """Resident tensor-core form: the persistent cooperative launch (a chunk of steps per
    launch, grid barriers between half-steps, several tiles per CTA when the tiles
    outnumber the resident CTAs: 700 tiles for 89,600 walkers) and one launch per
    half-step give bit-identical positions, log densities, per-step means and acceptance
    (a partial last tile in the third case)."""
    rng = np.random.default_rng(D)
    A = rng.normal(size=(D, D))
    P = (A @ A.T / D + np.eye(D)).astype(np.float32)
    out = {}
    for persist in (True, False):
        sf = factory.mcmc_factory(M.mvn_precision_model(D), form="gemm", tensor=True)
        s = sf.create_sampler(23, W, P.reshape(-1))
        s.set_persistent(persist)
        s.init_position_normal(4, 0.0, 1.0)
        s.burn_in(40, 2.0)
        r = s.run_sampler(37, 2.0, return_means=True)
        out[persist] = (s.positions().copy(), s.logfn().copy(), r["means"].copy(),
                        r["acceptance_rate"])
        s.release()
        sf.release()
    a, b = out[True], out[False]
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(a[2], b[2])
    assert a[3] == b[3]


def test_tcr_grid_barrier_runs_out_and_context_recovers(factory, M):
    """Device failure path without a fault: armed, the persistent form's grid barriers wait
    for one CTA more than the launch has; every CTA gives up after its bounded wait (2 s),
    raises the abort flag and the status word, and the launch ends.  The host reads the
    status (BAY_ERR_DEVICE, naming the grid barrier); a new sampler on the same context
    then runs normally."""
    import time
    from bayadera_gb300._native import BayaderaError, BAY_ERR_DEVICE
    D, W = 10, 4096
    P = np.diag(np.linspace(0.5, 2.0, D)).astype(np.float32)
    sf = factory.mcmc_factory(M.mvn_precision_model(D), form="gemm", tensor=True)
    s = sf.create_sampler(31, W, P.reshape(-1))
    s.set_persistent(True)
    s.init_position_normal(2, 0.0, 1.0)
    s.arm_barrier_timeout(True)
    t0 = time.perf_counter()
    with pytest.raises(BayaderaError, match="grid barrier") as e:
        s.run_sampler(8, 2.0)
    assert e.value.code == BAY_ERR_DEVICE
    assert time.perf_counter() - t0 < 60.0
    s.release()
    s = sf.create_sampler(31, W, P.reshape(-1))
    s.set_persistent(True)
    s.init_position_normal(2, 0.0, 1.0)
    r = s.run_sampler(40, 2.0, return_means=True)
    assert 0.2 < r["acceptance_rate"] < 0.9
    np.testing.assert_allclose(r["means"][:, -1], s.mean(), rtol=1e-5, atol=1e-6)
    s.release()
    sf.release()
