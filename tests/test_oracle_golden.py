"""Pins the CPU oracle to the reference's own golden vectors
(test/clojure/uncomplicate/bayadera/internal/nvidia_gtx_test.clj), CPU only."""
import numpy as np
import pytest

from tests.conftest import acor_matrix


def test_philox_known_answers(oracle):
    # Random123 known-answer vectors for philox4x32-10 (kat_vectors).
    assert [hex(x) for x in oracle.philox([0, 0, 0, 0], [0, 0])] == \
        ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(x) for x in oracle.philox([0xffffffff] * 4, [0xffffffff] * 2)] == \
        ["0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(x) for x in oracle.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                                          [0xa4093822, 0x299f31d0])] == \
        ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_u01_open_interval(oracle):
    assert oracle.u01(0) == np.float32(0.5 * 2.0 ** -23)
    assert oracle.u01(0xffffffff) == np.float32(1.0 - 2.0 ** -24)


def test_direct_uniform_bit_exact(oracle, golden):
    g = golden["direct_samplers"]["uniform"]
    s = oracle.sample_direct("uniform", g["n"], g["params"], g["seed"])
    assert s[:4].tolist() == g["first4"]
    assert s[-4:].tolist() == g["last4"]
    assert float(s.max()) == g["max"]
    assert float(s.min()) == g["min"]
    assert abs(s.astype(np.float64).mean() - g["mean"]) < 1e-5


@pytest.mark.parametrize("kind", ["gaussian", "erlang", "exponential"])
def test_direct_transcendental_samplers(oracle, golden, kind):
    # The reference uses fast-math sin/cos/log/sqrt; libm differs in the last bits.
    g = golden["direct_samplers"][kind]
    s = oracle.sample_direct(kind, g["n"], g["params"], g["seed"])
    np.testing.assert_allclose(s[:4], g["first4"], rtol=2e-5, atol=2e-5)
    np.testing.assert_allclose(s[-4:], g["last4"], rtol=2e-5, atol=2e-5)
    assert abs(float(s.max()) - g["max"]) <= 2e-5 * abs(g["max"])
    assert abs(float(s.min()) - g["min"]) <= 1e-3 * abs(g["min"]) + 1e-7
    assert abs(s.astype(np.float64).mean() - g["mean"]) <= 1e-5 * abs(g["mean"])


def _uniform_sampler(oracle, g):
    s = oracle.Stretch("uniform", 1, g["walkers"], g["params"], data_len=0, seed=g["seed"],
                       wgs=g["wgs"])
    s.init(g["seed"])
    s.init_position(g["seed"], g["limits"])
    return s


def test_stretch_uniform_trajectory_bit_exact(oracle, golden):
    g = golden["stretch_uniform"]
    s = _uniform_sampler(oracle, g)
    for want in g["sample_steps_first4"]:
        assert s.sample()[:4, 0].tolist() == want


def test_stretch_uniform_relaunch(oracle, golden):
    # nvidia_gtx_test.clj:214-235: bare kernels launched by hand for steps 0 and 1.
    g = golden["stretch_uniform"]
    s = _uniform_sampler(oracle, g)
    for step, want in enumerate(g["relaunch_first4"]):
        s.half(0, g["seed"], 3333, step, g["a"], 1.0)
        s.half(1, g["seed"] + 1, 4444, step, g["a"], 1.0)
        assert s.xs[:4].tolist() == want


def test_stretch_accu_statistics(oracle, golden):
    # nvidia_gtx_test.clj:237-258: one stretch_move_accu step after two bare steps.
    g = golden["stretch_uniform"]
    s = _uniform_sampler(oracle, g)
    s.move_bare()
    s.move_bare()
    G = s.K // g["wgs"]
    accept = np.zeros(G, np.uint32)
    means = np.zeros(G, np.float32)
    s.move_accu(g["seed"], 0, g["a"], accept, means)
    assert s.xs[:4].tolist() == g["accu_first4"]
    assert means[:10].tolist() == [float(np.float32(v)) for v in g["accu_means_blocks_first10"]]
    assert accept[:10].tolist() == g["accu_accept_blocks_first10"]
    total = np.zeros(1, np.float32)
    oracle.lib().bo_sum_means_vertical(1, G, g["wgs"], means, total)
    assert total[0] == np.float32(g["accu_means_total"])


def test_stretch_gaussian_trajectory(oracle, golden):
    # Gaussian target: q passes through exp; libm expf and the GPU's fast exp give
    # the same accept decisions on these walkers, so the values match exactly.
    g = golden["stretch_gaussian"]
    s = oracle.Stretch("gaussian", 1, g["walkers"], g["params"], seed=g["seed"], wgs=g["wgs"])
    s.init(g["seed"])
    s.init_position(g["seed"], g["limits"])
    for want in g["sample_steps_first4"]:
        np.testing.assert_array_max_ulp(s.sample()[:4, 0], np.array(want, np.float32), maxulp=1)


@pytest.mark.parametrize("flags", [0, 2])
def test_burn_in_gaussian(oracle, golden, flags):
    g = golden["burn_in_gaussian"]
    s = oracle.Stretch("gaussian", 1, g["walkers"], g["params"], seed=g["init_seed"],
                       wgs=g["wgs"], flags=flags)
    s.init_position(g["init_seed"], g["limits"])
    s.init(g["seed"])
    s.burn_in(g["steps"], g["a"])
    m = s.sample().astype(np.float64).mean()
    assert abs(m - g["mean"]) < 1e-5
    assert s.sample()[::1500, 0].tolist() == g["take_nth_1500"]
    assert abs(s.sample().astype(np.float64).std() - g["sd"]) < 1e-5


@pytest.mark.parametrize("n", [67, 367])
def test_acor_short_series_bit_exact(oracle, golden, acor_series, n):
    a = golden["acor"][str(n)]
    m = acor_matrix(acor_series, n, a["row1"])
    tau, mean, sigma, lag = oracle.acor_ref(m, golden["acor"]["wgs"])
    assert tau.tolist() == a["tau"]
    assert float(sigma[0]) == pytest.approx(a["sigma0"], abs=0, rel=1e-7)
    tau64, _, sigma64, _ = oracle.acor64(m, golden["acor"]["wgs"])
    np.testing.assert_allclose(tau64, a["tau"], rtol=1e-5)
    np.testing.assert_allclose(sigma64[0], a["sigma0"], rtol=1e-5)


def test_acor_long_series(oracle, golden, acor_series):
    a = golden["acor"]["112640"]
    m = acor_matrix(acor_series, 112640, a["row1"])
    for fn in (oracle.acor_ref, oracle.acor64):
        tau, _, sigma, _ = fn(m, golden["acor"]["wgs"])
        assert abs(tau[1] - a["tau1"]) <= a["tau1_tol"]
        assert abs(sigma[0] - a["sigma0"]) <= a["sigma0_tol"]


def test_acor_too_short_raises(oracle):
    with pytest.raises(ValueError):
        oracle.acor_ref(np.ones((1, 40), np.float32))


def test_bitonic_ranks_descending(oracle):
    rng = np.random.default_rng(0)
    pdf = rng.integers(0, 5, size=256).astype(np.float32)
    ranks = np.zeros(256, np.float32)
    oracle.lib().bo_bitonic_ranks(1, 256, pdf, ranks)
    order = ranks.astype(int)
    assert sorted(order.tolist()) == list(range(256))
    assert np.all(np.diff(pdf[order]) <= 0)


def test_histogram_normalised(oracle):
    rng = np.random.default_rng(1)
    xs = rng.random(3 * 4096).astype(np.float32)
    limits, pdf, ranks, counts = oracle.histogram([xs], 3, 256)
    pdf = pdf.reshape(3, 256)
    width = (limits[1::2] - limits[0::2]) / 256
    np.testing.assert_allclose((pdf * width[:, None]).sum(axis=1), 1.0, rtol=1e-5)
    assert counts.sum() == 3 * 4096


def test_beta_binomial_posterior_and_evidence(golden):
    """nvidia_gtx_test.clj:133-159 as the device models state it: the beta-binomial
    posterior's log density (binomial loglik of (n, z) without the coefficient + the beta
    prior with library.py's parameter vector) minus the conjugate Beta(a + z, b + n - z)'s
    is the golden constant at every point, and the likelihood engine's evidence (the mean of
    exp(loglik) over the points) is the golden value."""
    import math
    from bayadera_gb300 import library as L
    g = golden["beta_binomial"]
    n, z, a, b = g["n"], g["z"], g["a"], g["b"]
    x = (g["start"] + g["step"] * np.arange(g["points"])).astype(np.float32).astype(np.float64)
    prior = L.beta(None, a, b).params.astype(np.float64)
    conj = L.beta(None, a + z, b + n - z).params.astype(np.float64)

    def beta_log(p, t):
        return (p[0] - 1.0) * np.log(t) + (p[1] - 1.0) * np.log1p(-t) + p[2]

    loglik = z * np.log(x) + (n - z) * np.log1p(-x)
    post = loglik + beta_log(prior, x)
    diff = post - beta_log(conj, x)
    assert np.linalg.norm(diff - g["log_ratio"]) / math.sqrt(x.size) <= g["log_ratio_tol"]
    assert np.mean(np.exp(loglik)) == pytest.approx(g["evidence"], rel=1e-5)


def test_log_det_accuracy(oracle):
    """The accept test's fp32 logarithm (the kernels' bay_log_det, restated by the oracle
    with the same operations): within 2 ulp of the correctly rounded log on the accept
    test's domain -- uniforms (0.5 + i) 2^-23 and stretch factors in [1/8, 8]."""
    import numpy as np
    rng = np.random.default_rng(1)
    xs = np.concatenate([(0.5 + rng.integers(0, 1 << 23, 20000)) * 2.0 ** -23,
                         np.exp(rng.uniform(np.log(0.125), np.log(8.0), 20000)),
                         [2.0 ** -24, 0.5, 1.0, 1.41421354, 1.4142137, 2.0, 8.0]]).astype(np.float32)
    got = np.array([oracle.log_det(x) for x in xs], np.float32)
    want = np.log(xs.astype(np.float64))
    ulp = np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)
    err = np.abs(got.astype(np.float64) - want)
    assert np.all(err <= 2 * ulp + 1e-45), float(np.max(err / ulp))
    assert oracle.log_det(1.0) == 0.0
