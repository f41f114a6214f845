"""Direct samplers and density / likelihood / evidence engines against the reference's
golden vectors (nvidia_gtx_test.clj direct samplers), the oracle, and FP64 numpy."""
import math

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


def test_direct_uniform_bit_exact(factory, golden, oracle):
    """Uniform samples: the golden first/last four, extrema and mean, and every sample
    equal to the oracle's (no transcendental on the path)."""
    g = golden["direct_samplers"]["uniform"]
    s = factory.direct_sample("uniform", g["seed"], g["params"], g["n"])
    assert s[:4].tolist() == g["first4"]
    assert s[-4:].tolist() == g["last4"]
    assert float(s.max()) == g["max"] and float(s.min()) == g["min"]
    assert abs(s.astype(np.float64).mean() - g["mean"]) < 1e-5
    np.testing.assert_array_equal(s, oracle.sample_direct("uniform", g["n"], g["params"], g["seed"]))


@pytest.mark.parametrize("kind", ["gaussian", "exponential", "erlang"])
def test_direct_transcendental_samplers(factory, golden, oracle, kind):
    """Gaussian (Box-Muller), exponential and erlang samples: the reference's golden values
    within 2e-5 (fast-math sin/cos/log/sqrt as the reference compiles them), and the
    oracle's libm samples within 5e-5 relative."""
    g = golden["direct_samplers"][kind]
    s = factory.direct_sample(kind, g["seed"], g["params"], g["n"])
    np.testing.assert_allclose(s[:4], g["first4"], rtol=2e-5, atol=2e-5)
    np.testing.assert_allclose(s[-4:], g["last4"], rtol=2e-5, atol=2e-5)
    assert abs(float(s.max()) - g["max"]) <= 2e-5 * abs(g["max"])
    assert abs(s.astype(np.float64).mean() - g["mean"]) <= 1e-5 * abs(g["mean"])
    o = oracle.sample_direct(kind, g["n"], g["params"], g["seed"])
    np.testing.assert_allclose(s, o, rtol=5e-5, atol=5e-5 * float(np.abs(o).max()))


def test_direct_sampler_rejects_ragged(factory):
    from bayadera_gb300._native import BayaderaError
    with pytest.raises(BayaderaError, match="multiple of 4"):
        factory.direct_sample("uniform", 1, [0.0, 1.0], 10)


def test_distribution_engine_gaussian(factory, M):
    """log-density / density of the gaussian distribution (its normalised logpdf) at 1000
    points against FP64 numpy."""
    eng = factory.distribution_engine(M.distribution_models()["gaussian"])
    rng = np.random.default_rng(0)
    x = rng.normal(1.5, 3.0, size=(1000, 1)).astype(np.float32)
    params = np.array([1.5, 3.0], np.float32)
    want = -0.5 * ((x[:, 0].astype(np.float64) - 1.5) / 3.0) ** 2 - np.log(3.0) - 0.5 * np.log(2 * np.pi)
    np.testing.assert_allclose(eng.log_density(params, x), want, rtol=2e-6, atol=2e-6)
    np.testing.assert_allclose(eng.density(params, x), np.exp(want), rtol=1e-5, atol=1e-9)
    eng.release()


def test_distribution_engine_posterior_vs_oracle(factory, M, oracle):
    """A posterior's logpdf (likelihood + prior over 500 data) at points of (mu, sigma)
    against the oracle's FP64 density."""
    rng = np.random.default_rng(1)
    data = rng.normal(3.0, 2.0, 500).astype(np.float32)
    params = np.concatenate([data, np.array([0.0, 10.0, 0.0, 20.0], np.float32)])
    eng = factory.distribution_engine(M.gaussian_posterior_model(tiled=False))
    pts = np.stack([rng.uniform(1.0, 5.0, 300), rng.uniform(0.5, 4.0, 300)], axis=1).astype(np.float32)
    got = eng.log_density(params, pts)
    want = np.array([oracle.logfn64("gaussian_posterior", params, data.size, 2, p.astype(np.float64))
                     for p in pts])
    np.testing.assert_allclose(got, want, rtol=2e-5)
    eng.release()


def test_likelihood_engine_and_evidence(factory, M):
    """The gaussian likelihood (loglik through the 5-argument adapter) at points (mu, sigma)
    against FP64 numpy; evidence = mean of exp(loglik) over the points in FP64."""
    rng = np.random.default_rng(2)
    y = rng.normal(0.5, 1.0, 20).astype(np.float32)
    eng = factory.likelihood_engine(M.likelihood_models()["gaussian"], 2)
    pts = np.stack([rng.normal(0.5, 0.5, 2000), rng.uniform(0.6, 1.6, 2000)], axis=1).astype(np.float32)
    yd = y.astype(np.float64)[None, :]
    mu, sg = pts[:, :1].astype(np.float64), pts[:, 1:].astype(np.float64)
    want = np.sum(-0.5 * ((yd - mu) / sg) ** 2 - np.log(sg) - 0.5 * np.log(2 * np.pi), axis=1)
    got = eng.log_density(y, pts)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-4)
    ev = eng.evidence(y, pts)
    assert abs(ev - np.mean(np.exp(want))) <= 1e-4 * np.mean(np.exp(want))
    eng.release()


def test_density_engine_needs_plain_form(factory, M):
    from bayadera_gb300._native import BayaderaError
    sf = factory.mcmc_factory(M.gaussian_posterior_model(), form="tiled")
    import ctypes as C
    from bayadera_gb300 import _native as N
    p = np.zeros(5, np.float32)
    x = np.zeros(2, np.float32)
    out = np.zeros(1, np.float32)
    with pytest.raises(BayaderaError, match="plain form"):
        N.call("bay_log_density", sf.handle, C.c_void_p(p.ctypes.data), 5,
               C.c_void_p(x.ctypes.data), 1, C.c_void_p(out.ctypes.data))
    sf.release()


def test_dataset_moments_and_histogram(factory, oracle):
    """Dataset engine on a 3 x 50,000 data matrix: FP64 moments against the oracle's FP64
    mean and variance, and the histogram (limits, pdf, bin ranks; counts from 0) bit-exact
    against the oracle's."""
    rng = np.random.default_rng(4)
    x = np.stack([rng.normal(2.0, 1.0, 50000), rng.exponential(1.5, 50000),
                  rng.uniform(-3.0, 5.0, 50000)], axis=1).astype(np.float32)
    mean, var = factory.data_moments(x)
    np.testing.assert_allclose(mean, oracle.mean64(x.reshape(-1), 3), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(var, oracle.variance64(x.reshape(-1), 3), rtol=1e-12)
    h = factory.data_histogram(x, 256)
    ol, opdf, orank, _ = oracle.histogram([x.reshape(-1)], 3, 256, wgs=256)
    np.testing.assert_array_equal(h.limits.T.reshape(-1), ol)
    np.testing.assert_array_equal(h.pdf.T.reshape(-1), opdf)
    np.testing.assert_array_equal(h.bin_ranks.T.reshape(-1), orank)


def test_core_dataset_likelihood_evidence(factory, M):
    """The reference-shaped core API over the engines: dataset(...) moments and histogram
    equal the dataset engine's; evidence(likelihood(model), data, prior_sample) equals the
    likelihood engine's evidence."""
    from bayadera_gb300 import core
    rng = np.random.default_rng(6)
    x = np.stack([rng.normal(1.0, 2.0, 20000), rng.exponential(1.0, 20000)], axis=1).astype(np.float32)
    ds = core.dataset(factory, x)
    m, v = factory.data_moments(x)
    np.testing.assert_array_equal(core.mean(ds), m)
    np.testing.assert_array_equal(core.variance(ds), v)
    np.testing.assert_allclose(core.sd(ds), np.sqrt(v))
    h = core.histogram(ds, 1, 128)
    h2 = factory.data_histogram(x, 128)
    np.testing.assert_array_equal(h.pdf, h2.pdf)
    y = rng.normal(0.5, 1.0, 20).astype(np.float32)
    pts = np.stack([rng.normal(0.5, 0.5, 1000), rng.uniform(0.6, 1.6, 1000)], axis=1).astype(np.float32)
    lik = core.likelihood(factory, M.likelihood_models()["gaussian"])
    ev = core.evidence(lik, y, pts)
    eng = factory.likelihood_engine(M.likelihood_models()["gaussian"], 2)
    assert ev == eng.evidence(y, pts)
    eng.release()
    lik.release()


def test_library_distributions_sample_and_density(factory):
    """library.py on the GPU: log densities at points against scipy (rtol 2e-5); direct
    samplers (uniform, Gaussian, exponential, Erlang) and the MCMC samplers the reference
    warms up (Student's t, beta, gamma) give sample means and variances near the closed
    forms (5 sigma of the sample-mean error, 10 % on the variance)."""
    st = pytest.importorskip("scipy.stats")
    from bayadera_gb300 import core, library as L
    cases = [
        (L.uniform(factory, -1.0, 3.0), lambda x: st.uniform.logpdf(x, -1.0, 4.0), [-0.5, 0.0, 2.9]),
        (L.gaussian(factory, 1.0, 2.0), lambda x: st.norm.logpdf(x, 1.0, 2.0), [-1.0, 0.5, 4.0]),
        (L.exponential(factory, 2.5), lambda x: st.expon.logpdf(x, scale=0.4), [0.1, 0.7, 2.0]),
        (L.erlang(factory, 2.0, 3), lambda x: st.gamma.logpdf(x, 3, scale=0.5), [0.3, 1.5, 4.0]),
        (L.student_t(factory, 5.0, 1.0, 2.0), lambda x: st.t.logpdf(x, 5.0, 1.0, 2.0), [-3.0, 1.2, 6.0]),
        (L.beta(factory, 2.0, 3.0), lambda x: st.beta.logpdf(x, 2.0, 3.0), [0.1, 0.4, 0.9]),
        (L.gamma(factory, 1.5, 3.0), lambda x: st.gamma.logpdf(x, 3.0, scale=1.5), [0.5, 2.0, 9.0]),
    ]
    for d, ref, pts in cases:
        got = d.log_density(pts)
        np.testing.assert_allclose(got, ref(np.array(pts)), rtol=2e-5, atol=2e-5)
        if d.direct is not None:
            x = core.sample(d.sampler({"seed": 3}), 1 << 18)[0].astype(np.float64)
        else:
            s = d.sampler({"seed": 3, "walkers": 1 << 15, "warm_up": 256})
            x = core.sample(s, 1 << 15)[0].astype(np.float64)
            s.release()
        n_eff = x.size if d.direct is not None else x.size / 8.0
        assert abs(x.mean() - d.mean()) <= 5.0 * d.sd() / math.sqrt(n_eff), (d.name, x.mean())
        assert abs(x.var() - d.variance()) <= 0.1 * d.variance(), (d.name, x.var())
        d.release()
