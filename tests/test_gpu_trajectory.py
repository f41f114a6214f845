"""Free-running walker trajectories of the plain form (the reference's kernel structure,
one thread per walker) against the oracle, step by step for 64 steps and more, and the
reference-compatibility modes (fast-math stretch factor, element-offset partner, fast
division in the histogram).

Bars, stated per test:
* Where the model's density uses no fast-math operation (the 50-D Gaussian: products and
  sums), the oracle runs its own restatement of the model.  Positions and log densities
  are bit-identical (0 ulp) for every walker that made the same accept decisions.
* Where the model uses fast-math operations (division, log; compiled with -use_fast_math
  like the reference), the oracle draws, proposes and decides, and the proposals' log
  densities come from the same model compiled for the device (bay_log_density).  Again 0
  ulp for walkers with the same decisions.
* The accept decision is the fp32 test log u <= (D-1) log z + beta (ly - lx) with the
  kernels' own logarithm (bay_log_det: explicitly rounded operations only), which the
  oracle restates operation for operation (bo_log_det), so the decisions are the same
  bits on both sides and no walker may diverge.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 64
DIVERGED_CEILING = 0


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
def N():
    from bayadera_gb300 import _native
    return _native


def _device_density(N, sf, params):
    """log densities of points Y (n x dim) through the sampler module's own density kernel
    (bay_log_density): the model code the stretch kernel runs, compiled the same way."""
    p = np.ascontiguousarray(params, np.float32).reshape(-1)

    def dens(Y):
        Y = np.ascontiguousarray(Y, np.float32)
        out = np.zeros(Y.shape[0], np.float32)
        N.call("bay_log_density", sf.handle, C.c_void_p(p.ctypes.data), p.size,
               C.c_void_p(Y.ctypes.data), Y.shape[0], C.c_void_p(out.ctypes.data))
        return out
    return dens


def _run(s, r, steps, move, W, dim):
    """Both sides `steps` bare steps from the same state; per step, the walkers whose
    positions differ.  Returns the counts per step."""
    counts = []
    for t in range(steps):
        got = s.sample().T.reshape(W, dim)
        move()
        want = r.xs.reshape(W, dim)
        counts.append(int(np.any(got != want, axis=1).sum()))
    return counts


def _check(s, r, counts, W, name):
    print("%s: walkers differing after each step: max %d, final %d of %d"
          % (name, max(counts), counts[-1], W))
    assert max(counts) <= DIVERGED_CEILING * W, counts
    same = np.all(s.positions().T.reshape(W, -1) == r.xs.reshape(W, -1), axis=1)
    lf_gpu, lf_ref = s.logfn(), r.logfn
    # walkers with the same decisions: log densities bit-identical (0 ulp)
    np.testing.assert_array_equal(lf_gpu[same], lf_ref[same])


def test_free_running_mvn50_c2_matrix(factory, M, oracle):
    """The 50-D benchmark target (the AR(1) rho = 0.9 precision matrix with scales
    log-uniform in [0.1, 10]) in the plain form, 2,048 walkers from N(0, I), 64 steps
    against the oracle's own fp32 density (same fma order): bit-identical."""
    import bench
    D, W = 50, 2048
    P, _ = bench.precision_matrix()
    sf = factory.mcmc_factory(M.mvn_precision_model(D), form="plain")
    s = sf.create_sampler(21, W, P.reshape(-1))
    r = oracle.Stretch("mvn_precision", D, W, P.reshape(-1), seed=21,
                       flags=oracle.ACCEPT_LOG)
    r.init_position_normal(22, 0.0, 1.0)
    s.init_position(r.xs.reshape(W, D))
    np.testing.assert_array_equal(s.logfn(), r.logfn)
    counts = _run(s, r, STEPS, r.move_bare, W, D)
    _check(s, r, counts, W, "mvn50")
    s.release()
    sf.release()


def test_free_running_gaussian_d1_golden_config(factory, M, N, oracle, golden):
    """The reference's Gaussian stretch case (nvidia_gtx_test.clj:260-277: 11,264
    walkers, seed 123) for 64 steps; the model's fast-math density on both sides."""
    g = golden["stretch_gaussian"]
    W = g["walkers"]
    params = np.array(g["params"], np.float32)
    sf = factory.mcmc_factory(M.distribution_models()["gaussian"])
    s = sf.create_sampler(g["seed"], W, params)
    s.init(g["seed"])
    s.init_position(g["seed"], g["limits"])
    r = oracle.Stretch("gaussian", 1, W, params, seed=g["seed"], flags=oracle.ACCEPT_LOG)
    r.init(g["seed"])
    r.xs[:] = s.positions().T.reshape(-1)
    r.logfn[:] = s.logfn()
    dens = _device_density(N, sf, params)
    counts = _run(s, r, STEPS, lambda: r.move_bare_with_density(dens, a=2.0), W, 1)
    _check(s, r, counts, W, "gaussian d=1")
    s.release()
    sf.release()


def test_free_running_c1_posterior(factory, M, N, oracle):
    """The 2-D (mu, sigma) posterior of 10,000 N(3, 2^2) data with the N(0, 10^2) x
    U(0, 20) prior, 4,096 walkers, 64 steps, the model's fast-math density on both
    sides."""
    rng = np.random.default_rng(0)
    data = rng.normal(3.0, 2.0, 10000).astype(np.float32)
    params = np.concatenate([data, np.array([0.0, 10.0, 0.0, 20.0], np.float32)])
    W = 4096
    sf = factory.mcmc_factory(M.gaussian_posterior_model(), form="plain")
    s = sf.create_sampler(31, W, params)
    s.init_position(32, [2.0, 4.0, 1.0, 3.0])
    r = oracle.Stretch("gaussian_posterior", 2, W, params, data_len=data.size, seed=31,
                       flags=oracle.ACCEPT_LOG)
    r.xs[:] = s.positions().T.reshape(-1)
    r.logfn[:] = s.logfn()
    dens = _device_density(N, sf, params)
    counts = _run(s, r, STEPS, lambda: r.move_bare_with_density(dens, a=2.0), W, 2)
    _check(s, r, counts, W, "c1 posterior")
    s.release()
    sf.release()


# ------------------------------------------------------------------ reference compat modes
def _u0(oracle, seed, stream, step, k):
    return float(oracle.u01(int(oracle.philox([k, step, stream, 0xbeeff00d],
                                              [seed & 0xffffffff, 0xdecafbad])[0])))


@pytest.mark.parametrize("dim", [2, 3])
def test_partner_element_matches_oracle(factory, M, N, oracle, dim):
    """Quirk Q1 on the GPU: the element-offset partner (uint)(u0 K dim), elements past the
    half's end read as 0, against the oracle's PARTNER_ELEMENT mode: 16 free-running steps
    of the uniform model at dim 2 and 3, bit-identical positions.  Partners that straddle
    the half's end occur in the run (counted from the oracle's draws)."""
    W, seed = 4096, 77
    K = W // 2
    params = np.array([-1.0, 2.0], np.float32)
    uni = M.device_distribution_model(M.get_source("uniform"), name="uniform", dimension=dim,
                                      params_size=2)
    sf = factory.mcmc_factory(uni, partner_element=True)
    s = sf.create_sampler(seed, W, params)
    s.init(seed)
    s.init_position(seed, [-1.0, 2.0] * dim)
    r = oracle.Stretch("uniform", dim, W, params, seed=seed,
                       flags=oracle.ACCEPT_LOG | oracle.PARTNER_ELEMENT)
    r.init(seed)
    r.xs[:] = s.positions().T.reshape(-1)
    r.logfn[:] = s.logfn()
    dens = _device_density(N, sf, params)
    steps = 16
    counts = _run(s, r, steps, lambda: r.move_bare_with_density(dens, a=2.0), W, dim)
    print("partner element dim %d: differing walkers per step %s" % (dim, counts))
    assert max(counts) == 0
    straddle = 0
    for t in range(steps):
        for half, stream in ((0, 3333), (1, 4444)):
            for k in range(K):
                j0 = int(np.float32(np.float32(_u0(oracle, seed + half, stream, t, k))
                                    * np.float32(K)) * np.float32(dim))
                straddle += j0 + dim - 1 >= K * dim
    print("partners past the half's end: %d" % straddle)
    assert straddle >= 1
    s.release()
    sf.release()


@pytest.mark.parametrize("accept_ref", [False, True])
def test_stretch_ref_golden_uniform(factory, M, oracle, golden, accept_ref):
    """The stretch factor with the reference build's fast division for 1/a gives the
    golden uniform trajectories bit for bit (a = 2, where 1/a is exact either way).  (The
    reference's own spelling of the expression, compiled by today's NVRTC, contracts
    differently and misses the golden vector by 1 ulp: the operation order is kept.)"""
    g = golden["stretch_uniform"]
    sf = factory.mcmc_factory(M.distribution_models()["uniform"], accept_ref=accept_ref,
                              stretch_ref=True)
    s = sf.create_sampler(g["seed"], g["walkers"], np.array(g["params"], np.float32))
    s.init(g["seed"])
    s.init_position(g["seed"], g["limits"])
    for want in g["sample_steps_first4"]:
        assert s.sample()[0][:4].tolist() == want
    s.release()
    sf.release()


@pytest.mark.parametrize("a", [1.5, 1.7, 2.5, 3.3])
def test_stretch_ref_vs_ieee(factory, M, a):
    """At a != 2 the fast division moves 1/a, and so z, by a few ulp: one step of the
    uniform model (every in-range proposal accepted) from the same positions, compat vs
    default, differs by at most 2^-20 a (|X| + |S|) per walker, and only where a proposal
    sits on the support's edge do the decisions differ."""
    W, seed = 8192, 5
    params = np.array([-1.0, 2.0], np.float32)
    out = []
    for ref in (False, True):
        sf = factory.mcmc_factory(M.distribution_models()["uniform"], stretch_ref=ref)
        s = sf.create_sampler(seed, W, params)
        s.init(seed)
        s.init_position(seed, [-1.0, 2.0])
        s.burn_in(1, a)
        out.append(s.positions()[0].astype(np.float64))
        s.release()
        sf.release()
    d = np.abs(out[0] - out[1])
    bound = 2.0 ** -20 * a * 4.0
    edge = np.zeros(W, bool)
    for o in out:
        edge |= np.minimum(np.abs(o + 1.0), np.abs(o - 2.0)) < 4 * bound
    print("a = %g: %d of %d walkers differ, largest difference %.3g"
          % (a, int((d > 0).sum()), W, d.max()))
    assert np.all((d <= bound) | edge)


def _ar1_samples(n, seed=0):
    import bench
    _, sigma = bench.precision_matrix()
    L = np.linalg.cholesky(sigma)
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((n, sigma.shape[0])) @ L.T).astype(np.float32)


def test_histogram_fastdiv_moves_only_edge_values(factory, oracle):
    """The reference's fast division in the bin index (BAY_HIST_COMPAT_FASTDIV) on data
    shaped like the 50-D benchmark's (65,536 draws of the AR(1) Gaussian, 128 bins): the
    IEEE counts are bit-exact with the oracle; the fast-division counts equal them except
    for values within 4 ulp of a bin edge (the net count crossing each edge is at most the
    number of such values there).  Prints how many values moved."""
    from bayadera_gb300 import _native as N
    x = _ar1_samples(65536)
    n, D = x.shape
    bins = 128
    h_ieee = factory.data_histogram(x, bins)
    h_fast = factory.data_histogram(x, bins, N.HIST_COMPAT_FASTDIV)
    lim, pdf, ranks, counts = oracle.histogram([x.reshape(-1)], D, bins)
    np.testing.assert_array_equal(h_ieee.limits.T.reshape(-1), lim)
    np.testing.assert_array_equal(h_ieee.pdf.T.reshape(-1), pdf)
    np.testing.assert_array_equal(h_fast.limits, h_ieee.limits)
    alpha = np.float32(bins / n)
    moved = cand_total = 0
    for d in range(D):
        lo, hi = lim[2 * d], lim[2 * d + 1]
        c = np.float64(np.float32(alpha / np.float32(hi - lo)))
        cf = np.rint(h_fast.pdf[:, d].astype(np.float64) / c).astype(np.int64)
        ci = counts[d * bins:(d + 1) * bins].astype(np.int64)
        assert cf.sum() == n
        v = (x[:, d] - lo) / np.float32(hi - lo) * np.float32(bins)      # IEEE fp32 as the oracle
        near = np.abs(v - np.rint(v)) <= 4 * np.spacing(np.maximum(v, 1.0))
        edges = np.rint(v[near]).astype(np.int64)
        flow = np.cumsum(cf - ci)[:-1]              # net values moved below edge k + 1
        cand = np.bincount(edges, minlength=bins + 1)[1:bins]
        assert np.all(np.abs(flow) <= cand), d
        moved += int(np.abs(cf - ci).sum() // 2)
        cand_total += int(cand.sum())
    print("fast division: %d of %d values changed bin; %d values lie within 4 ulp of an edge"
          % (moved, n * D, cand_total))


def test_sampler_histogram_fastdiv(factory, M, oracle):
    """The sampler path's histogram with the fast division: limits equal the IEEE run's and
    the counts total walkers x cycles."""
    from bayadera_gb300 import _native as N
    W = 4096
    rng = np.random.default_rng(2)
    A = rng.normal(size=(8, 8))
    P = (A @ A.T / 8 + np.eye(8)).astype(np.float32)
    sf = factory.mcmc_factory(M.mvn_precision_model(8), form="plain")
    hs = []
    for flags in (0, N.HIST_COMPAT_FASTDIV):
        s = sf.create_sampler(3, W, P.reshape(-1))
        s.init_position_normal(4, 0.0, 1.0)
        s.burn_in(10, 2.0)
        hs.append(s.histogram(2, 64, flags))
        s.release()
    sf.release()
    np.testing.assert_array_equal(hs[0].limits, hs[1].limits)
    for h in hs:
        lo, hi = h.limits[0], h.limits[1]
        tot = (h.pdf * (hi - lo)[None, :] / 64 * (2 * W)).sum(axis=0)
        np.testing.assert_allclose(tot, 2 * W, rtol=1e-4)
