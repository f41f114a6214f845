"""The models the benchmark configs run, as the oracle states them (FP64 and fp32), against
independent numpy formulas of the same densities; the host-side parameter encodings
(hierarchical rows) and the cooling schedules of anneal! / mix! (mcmc.clj:43-53).  CPU."""
import math

import numpy as np
import pytest


def _rel(a, b):
    return abs(a - b) / max(1.0, abs(b))


def test_mvn_precision(oracle):
    rng = np.random.default_rng(1)
    D = 12
    A = rng.normal(size=(D, D))
    P = (A @ A.T / D + np.eye(D)).astype(np.float32)
    for _ in range(5):
        x = rng.normal(size=D)
        want = -0.5 * x @ P.astype(np.float64) @ x
        assert _rel(oracle.logfn64("mvn_precision", P.reshape(-1), 0, D, x), want) < 1e-12
        assert _rel(oracle.logfn32("mvn_precision", P.reshape(-1), 0, D, x.astype(np.float32)),
                    want) < 1e-5


def test_logistic(oracle):
    rng = np.random.default_rng(2)
    n, F = 300, 7
    X = rng.normal(size=(n, F)).astype(np.float32)
    y = (rng.random(n) < 0.5).astype(np.float32)
    h0 = 5.0
    params = np.concatenate([np.concatenate([X, y[:, None]], axis=1).reshape(-1),
                             np.array([h0], np.float32)])
    for _ in range(5):
        b = rng.normal(scale=0.5, size=F)
        eta = X.astype(np.float64) @ b
        want = np.sum(y * eta - np.logaddexp(0.0, eta)) - b @ b / (2 * h0 * h0)
        assert _rel(oracle.logfn64("logistic", params, n * (F + 1), F, b), want) < 1e-12
        assert _rel(oracle.logfn32("logistic", params, n * (F + 1), F, b.astype(np.float32)),
                    want) < 1e-4


def test_robust_t(oracle):
    rng = np.random.default_rng(3)
    n, F = 200, 5
    X = rng.normal(size=(n, F)).astype(np.float32)
    y = (X @ rng.normal(size=F) + 0.5 * rng.standard_t(4, n)).astype(np.float32)
    nu, bsd, lsd = 4.0, 10.0, 1.0
    params = np.concatenate([np.concatenate([X, y[:, None]], axis=1).reshape(-1),
                             np.array([nu, bsd, lsd], np.float32)])
    for _ in range(5):
        x = np.concatenate([rng.normal(size=F), [rng.normal(scale=0.3)]])
        b, ls = x[:F], x[F]
        r = (y - X.astype(np.float64) @ b) / math.exp(ls)
        want = (np.sum(-0.5 * (nu + 1) * np.log1p(r * r / nu)) - n * ls
                - b @ b / (2 * bsd * bsd) - ls * ls / (2 * lsd * lsd))
        assert _rel(oracle.logfn64("robust_t", params, n * (F + 1), F + 1, x), want) < 1e-12
        assert _rel(oracle.logfn32("robust_t", params, n * (F + 1), F + 1, x.astype(np.float32)),
                    want) < 1e-4


def test_gaussian_posterior(oracle):
    rng = np.random.default_rng(4)
    data = rng.normal(3.0, 2.0, 400).astype(np.float32)
    h = np.array([0.0, 10.0, 0.0, 20.0], np.float32)
    params = np.concatenate([data, h])
    d = data.astype(np.float64)
    for mu, sg in ((2.5, 1.7), (3.1, 2.2), (-1.0, 0.5)):
        lik = np.sum(-(d - mu) ** 2 / (2 * sg * sg)) - d.size * (math.log(sg) + 0.5 * math.log(2 * math.pi))
        prior = (-(mu - 0.0) ** 2 / (2 * 100.0) - math.log(10.0) - 0.5 * math.log(2 * math.pi)
                 - math.log(20.0))
        want = lik + prior
        assert _rel(oracle.logfn64("gaussian_posterior", params, d.size, 2, np.array([mu, sg])),
                    want) < 1e-11
    # sigma outside the uniform prior's support: log density -inf (or NaN for sigma <= 0)
    assert oracle.logfn64("gaussian_posterior", params, d.size, 2, np.array([1.0, 25.0])) == -math.inf


def test_hierarchical_rows_encoding(oracle):
    """models.hierarchical_rows_params + the hrows density against the hierarchical model
    written out group by group."""
    from bayadera_gb300 import models as M
    rng = np.random.default_rng(5)
    J = 6
    ys = [rng.normal(j, 1.0, 10 + 4 * j) for j in range(J)]
    sig = rng.uniform(0.5, 2.0, J)
    h0, h1 = 10.0, 1.0
    params, rows = M.hierarchical_rows_params(ys, sig, h0, h1)
    assert rows == sum(len(y) for y in ys) and params.size == 3 * rows + 2
    for _ in range(5):
        theta = rng.normal(size=J)
        mu, lt = rng.normal(), rng.normal(scale=0.3)
        x = np.concatenate([theta, [mu, lt]])
        want = 0.0
        for j in range(J):
            yj = np.asarray(ys[j], np.float32).astype(np.float64)
            s2 = float(np.float32(-0.5 / (float(sig[j]) ** 2)))     # the encoded coefficient
            want += s2 * np.sum((yj - theta[j]) ** 2)
        tau2 = math.exp(2 * lt)
        want += np.sum(-(theta - mu) ** 2 / (2 * tau2)) - J * lt - mu * mu / (2 * h0 * h0) \
            - lt * lt / (2 * h1 * h1)
        assert _rel(oracle.logfn64("hrows", params, 3 * rows, J + 2, x), want) < 1e-11


def test_cooling_schedules():
    """mcmc.clj:43-53: sqrt-n, pow-n and minus-n of a temperature at step i."""
    from bayadera_gb300 import mcmc
    assert mcmc.minus_n(10)(3) == 7
    assert mcmc.sqrt_n(10)(1) == pytest.approx(3.0)
    assert mcmc.pow_n(2.0)(10)(4) == pytest.approx(36.0)


def test_oracle_stretch_samples_a_correlated_gaussian(oracle):
    """The oracle's stretch move at D > 1 (where the reference has no golden vectors): a 3-D
    Gaussian with correlations 0.8 and scales 0.5..4 from N(0, I) starts; after burn-in the
    ensemble's covariance matches the target within 10 % per entry and the per-step means
    average to 0 within 5 MC standard errors (their spread over steps, inflated for
    autocorrelation)."""
    D, W = 3, 4096
    s = np.array([0.5, 1.5, 4.0])
    R = np.array([[1.0, 0.8, 0.64], [0.8, 1.0, 0.8], [0.64, 0.8, 1.0]])
    Sigma = R * np.outer(s, s)
    P = np.linalg.inv(Sigma).astype(np.float32).reshape(-1)
    st = oracle.Stretch("mvn_precision", D, W, P, data_len=0, seed=7, wgs=256)
    st.init(7)
    st.init_position_normal(8, 0.0, 1.0)
    st.burn_in(300, 2.0)
    rate, means = st.run_sampler(400, 2.0)
    assert 0.3 < rate < 0.9
    xs = st.xs.reshape(W, D).astype(np.float64)
    C = np.cov(xs.T)
    assert np.all(np.abs(C - Sigma) <= 0.1 * np.sqrt(np.outer(np.diag(Sigma), np.diag(Sigma))))
    m = means.astype(np.float64)                    # (D, steps) ensemble means
    se = m.std(axis=1) * np.sqrt(50.0 / m.shape[1])  # tau <= 50 steps for this target
    assert np.all(np.abs(m.mean(axis=1)) <= 5 * se + 1e-3 * s)


def test_core_host_wrappers_without_gpu():
    """core.py's reference-shaped wrappers, checked with stand-in engines: dataset rejects
    an empty matrix, sample! fills a contiguous matrix and rejects a strided one, and
    evidence(lik, data, prior_sample) evaluates through the likelihood's engine for the
    prior sample's dimension."""
    from bayadera_gb300 import core as c

    with pytest.raises(ValueError, match="can not support"):
        c.Dataset(object(), np.zeros((0, 3)))

    class FakeSampler:
        def sample(self, n):
            return np.arange(2 * n, dtype=np.float32).reshape(2, n)

    out = np.zeros((2, 4), np.float32)
    c.sample_(FakeSampler(), out)
    assert out.tolist() == [[0, 1, 2, 3], [4, 5, 6, 7]]
    with pytest.raises(ValueError, match="contiguous"):
        c.sample_(FakeSampler(), np.zeros((2, 8), np.float32)[:, ::2])

    class FakeEngine:
        def __init__(self, dim):
            self.dim = dim

        def evidence(self, data, x):
            return float(self.dim * 100 + len(data) + x.shape[0])

        def release(self):
            pass

    class FakeFactory:
        def likelihood_engine(self, model, dim):
            return FakeEngine(dim)

    lik = c.Likelihood(FakeFactory(), "model")
    assert c.evidence(lik, [1.0, 2.0, 3.0], np.zeros((5, 2))) == 2 * 100 + 3 + 5
    assert set(lik._engines) == {2}
    lik.release()


def test_library_parameters_and_moments():
    """library.py: the parameter vectors' log-normalising constants (the densities' log
    normaliser read by the device models) and the closed-form moments against scipy."""
    st = pytest.importorskip("scipy.stats")
    from bayadera_gb300 import library as L
    t = L.student_t(None, 5.0, 1.0, 2.0)
    x = 0.7
    unscaled = -0.5 * (5.0 + 1.0) * math.log1p(((x - 1.0) / 2.0) ** 2 / 5.0)
    assert unscaled + float(np.float64(t.params[3])) == pytest.approx(st.t.logpdf(x, 5.0, 1.0, 2.0), rel=1e-6)
    assert (t.mean(), t.variance()) == pytest.approx((st.t.mean(5.0, 1.0, 2.0), st.t.var(5.0, 1.0, 2.0)))
    b = L.beta(None, 2.0, 3.0)
    assert (1.0 * math.log(0.4) + 2.0 * math.log(0.6) + b.params[2]) == pytest.approx(
        st.beta.logpdf(0.4, 2.0, 3.0), rel=1e-6)
    assert b.mean() == pytest.approx(st.beta.mean(2.0, 3.0))
    assert b.variance() == pytest.approx(st.beta.var(2.0, 3.0))
    assert b.median() == pytest.approx(st.beta.median(2.0, 3.0), rel=1e-12)    # exact case
    assert L.beta(None, 3.0, 2.0).median() == pytest.approx(st.beta.median(3.0, 2.0), rel=1e-12)
    g = L.gamma(None, 1.5, 3.0)
    assert (2.0 * math.log(2.0) - 2.0 / 1.5 + g.params[2]) == pytest.approx(
        st.gamma.logpdf(2.0, 3.0, scale=1.5), rel=1e-6)
    assert (g.mean(), g.variance(), g.mode()) == pytest.approx((4.5, 6.75, 3.0))
    e = L.erlang(None, 2.0, 4)
    assert (3.0 * math.log(1.3) - 2.0 * 1.3 + e.params[2]) == pytest.approx(
        st.gamma.logpdf(1.3, 4, scale=0.5), rel=1e-6)
    x = L.exponential(None, 2.5)
    assert (x.mean(), x.variance(), x.median()) == pytest.approx((0.4, 0.16, math.log(2) / 2.5))
    assert L.uniform(None, -1.0, 3.0).variance() == pytest.approx(16.0 / 12.0)
    for bad in (lambda: L.uniform(None, 1.0, 1.0), lambda: L.gaussian(None, 0.0, 0.0),
                lambda: L.student_t(None, -1.0), lambda: L.beta(None, 0.0, 1.0),
                lambda: L.gamma(None, 1.0, 0.0), lambda: L.exponential(None, 0.0),
                lambda: L.erlang(None, 1.0, 0)):
        with pytest.raises(ValueError, match="illegal"):
            bad()
