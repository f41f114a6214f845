"""Device models and their C sources (mirrors internal/device/models.clj).

A distribution model carries its C source, the name of its log density (and the
MCMC variant without the normalising constant), its dimension, the number of
hyperparameters and default limits; a likelihood model carries a source and the
name of its loglik.  device_posterior_model composes a prior and a likelihood into
a new distribution model by generating the posterior's C function
(models.clj:102-115; the template is cuda/distributions/posterior.cu:5-10):

    post(data_len, hyper_len, params, dim, x) =
        loglik(data_len, params, dim, x)
      + prior_logpdf(data_len, hyper_len, &params[data_len], dim, x)

so the posterior's params are data || prior hyperparameters.
"""
import itertools
import os

import numpy as np

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "library")

_counter = itertools.count()

FLOAT_MAX = float(np.finfo(np.float32).max)
FLOAT_MIN = float(np.finfo(np.float32).tiny)


def _gensym(prefix):
    return "%s%d" % (prefix, next(_counter))


def source_library():
    """name -> C source of the built-in model library (csrc/library/*.h)."""
    out = {}
    for fn in sorted(os.listdir(LIB_DIR)):
        if fn.endswith(".h"):
            with open(os.path.join(LIB_DIR, fn)) as f:
                out[fn[:-2]] = f.read()
    return out


_SOURCES = None


def get_source(name):
    global _SOURCES
    if _SOURCES is None:
        _SOURCES = source_library()
    return _SOURCES[name]


class DeviceLikelihoodModel:
    """DeviceLikelihoodModel (models.clj:25-51)."""

    def __init__(self, name, loglik, source, dialect="c99"):
        self.name = name
        self.loglik = loglik
        self.sources = list(source) if isinstance(source, (list, tuple)) else [source]
        self.dialect = dialect

    def source(self):
        return self.sources


class DeviceDistributionModel:
    """DeviceDistributionModel (models.clj:57-100).

    tiled: optional dict with keys prep, term, walker, row_len, prep_len
    (the data-tiled form of the same density, see include/bayadera_gb300.h).
    gemm: optional dict with keys prep, term, walker, prep_len, features, coef, block
    ("data" | "hyper"), ld, offset, rows, aux_col, aux_len (the linear-predictor form).
    """

    def __init__(self, name, logpdf, mcmc_logpdf, dimension, params_size, limits, source,
                 dialect="c99", tiled=None, gemm=None, batch=None):
        self.name = name
        self.logpdf = logpdf
        self.mcmc_logpdf = mcmc_logpdf
        self.dimension = int(dimension)
        self.params_size = int(params_size)
        self.limits = None if limits is None else np.asarray(limits, np.float32).reshape(-1)
        self.sources = list(source) if isinstance(source, (list, tuple)) else [source]
        self.dialect = dialect
        self.tiled = tiled
        self.gemm = gemm
        self.batch = batch

    def source(self):
        return self.sources

    def full_source(self):
        seen, out = set(), []
        for s in self.sources:
            if s not in seen:
                seen.add(s)
                out.append(s)
        return "\n".join(out)

    def posterior_model(self, name, likelihood):
        return device_posterior_model(self, name, likelihood)


def device_distribution_model(source, name=None, logpdf=None, mcmc_logpdf=None, dimension=1,
                              params_size=1, limits=None, dialect="c99", tiled=None, gemm=None,
                              batch=None):
    """device-distribution-model (models.clj:84-89) with the same defaults."""
    name = name or _gensym("distribution")
    logpdf = logpdf or "%s_logpdf" % name
    return DeviceDistributionModel(name, logpdf, mcmc_logpdf or logpdf, dimension, params_size,
                                   limits, source, dialect, tiled, gemm, batch)


def device_likelihood_model(source, name=None, loglik=None, dialect="c99"):
    """device-likelihood-model (models.clj:46-51)."""
    name = name or _gensym("likelihood")
    return DeviceLikelihoodModel(name, loglik or "%s_loglik" % name, source, dialect)


_POSTERIOR = """
extern "C" {
inline REAL %(post)s(const uint32_t data_len, const uint32_t hyperparams_len,
                    const REAL* params, const uint32_t dim, const REAL* x) {
    return %(loglik)s(data_len, params, dim, x)
        + %(prior)s(data_len, hyperparams_len, &params[data_len], dim, x);
}
}
"""


def device_posterior_model(prior, name, lik):
    """device-posterior-model (models.clj:102-115)."""
    if prior.dialect != lik.dialect:
        raise ValueError("Incompatible types of likelihood and prior models.")
    post = _gensym(name)
    post_logpdf = "%s_logpdf" % post
    post_mcmc = "%s_mcmc_logpdf" % post
    srcs = []
    for s in prior.sources + lik.sources:
        if s not in srcs:
            srcs.append(s)
    srcs.append(_POSTERIOR % {"post": post_logpdf, "loglik": lik.loglik, "prior": prior.logpdf}
                + _POSTERIOR % {"post": post_mcmc, "loglik": lik.loglik, "prior": prior.logpdf})
    return DeviceDistributionModel(post, post_logpdf, post_mcmc, prior.dimension,
                                   prior.params_size, prior.limits, srcs, prior.dialect)


# ----------------------------------------------------------------- built-in models
def _lim(lo, hi):
    return [lo, hi]


def distribution_models():
    """distribution-models (models.clj:183-201): name -> model."""
    g = get_source
    return {
        "uniform": device_distribution_model(g("uniform"), name="uniform", params_size=2,
                                             limits=_lim(-FLOAT_MAX, FLOAT_MAX)),
        "gaussian": device_distribution_model(g("gaussian"), name="gaussian",
                                              mcmc_logpdf="gaussian_mcmc_logpdf", params_size=2,
                                              limits=_lim(-FLOAT_MAX, FLOAT_MAX)),
        "student_t": device_distribution_model(g("student_t"), name="student_t",
                                               mcmc_logpdf="student_t_mcmc_logpdf", params_size=4,
                                               limits=_lim(-FLOAT_MAX, FLOAT_MAX)),
        "beta": device_distribution_model(g("beta"), name="beta", mcmc_logpdf="beta_mcmc_logpdf",
                                          params_size=3, limits=_lim(0.0, 1.0)),
        "exponential": device_distribution_model(g("exponential"), name="exponential",
                                                 mcmc_logpdf="exponential_mcmc_logpdf",
                                                 params_size=2,
                                                 limits=_lim(FLOAT_MIN, FLOAT_MAX)),
        "erlang": device_distribution_model(g("erlang"), name="erlang",
                                            mcmc_logpdf="erlang_mcmc_logpdf", params_size=3,
                                            limits=_lim(0.0, FLOAT_MAX)),
        "gamma": device_distribution_model(g("gamma"), name="gamma",
                                           mcmc_logpdf="gamma_mcmc_logpdf", params_size=2,
                                           limits=_lim(0.0, FLOAT_MAX)),
        "binomial": device_distribution_model(g("binomial"), name="binomial",
                                              mcmc_logpdf="binomial_mcmc_logpdf", params_size=3,
                                              limits=_lim(0.0, FLOAT_MAX)),
    }


def likelihood_models():
    """likelihood-models (models.clj:203-206)."""
    g = get_source
    return {
        "gaussian": device_likelihood_model(g("gaussian"), name="gaussian"),
        "student_t": device_likelihood_model(g("student_t"), name="student_t"),
        "binomial": device_likelihood_model(g("binomial"), name="binomial"),
    }


# ----------------------------------------------------------------- benchmark models
def gaussian_posterior_model(tiled=True):
    """(mu, sigma) of Gaussian data with prior N(mu | h0, h1^2) Uniform(sigma | h2, h3);
    params = data || (h0, h1, h2, h3)."""
    src = [get_source("gaussian"), get_source("uniform"), get_source("gaussian_posterior")]
    t = None
    if tiled:
        t = {"prep": "gaussian_posterior_prep", "term": "gaussian_posterior_term",
             "walker": "gaussian_posterior_walker", "row_len": 1, "prep_len": 2}
    return device_distribution_model(src, name="gaussian_posterior", dimension=2, params_size=4,
                                     logpdf="gaussian_posterior_logpdf", tiled=t)


def mvn_precision_model(dim):
    """Zero-mean Gaussian with a dim x dim precision matrix as hyperparameters; GEMM form
    A = P (rows of the hyperparameter block), term -x_r eta_r / 2."""
    g = {"prep": "mvn_precision_prep", "term": "mvn_precision_term",
         "walker": "mvn_precision_walker", "features": dim, "coef": 0, "block": "hyper",
         "ld": dim, "offset": 0, "rows": dim}
    return device_distribution_model(get_source("mvn_precision"), name="mvn_precision",
                                     dimension=dim, params_size=dim * dim,
                                     logpdf="mvn_precision_logpdf", gemm=g)


def logistic_model(features):
    """Logistic regression on data rows (x_1..x_F, y); GEMM form A = the rows' features."""
    g = {"prep": "logistic_prep", "term": "logistic_term", "walker": "logistic_walker",
         "features": features, "coef": 0, "block": "data", "ld": features + 1, "offset": 0,
         "aux_col": features, "aux_len": 1}
    return device_distribution_model(get_source("logistic"), name="logistic",
                                     dimension=features, params_size=1, logpdf="logistic_logpdf",
                                     gemm=g)


def robust_t_model(features):
    """Student-t regression on data rows (x_1..x_F, y), x = (beta, log sigma)."""
    g = {"prep": "robust_t_prep", "term": "robust_t_term", "walker": "robust_t_walker",
         "prep_len": 3, "features": features, "coef": 0, "block": "data", "ld": features + 1,
         "offset": 0, "aux_col": features, "aux_len": 1}
    return device_distribution_model(get_source("robust_t"), name="robust_t",
                                     dimension=features + 1, params_size=3,
                                     logpdf="robust_t_logpdf", gemm=g)


def hierarchical_model(groups):
    return device_distribution_model(get_source("hierarchical"), name="hierarchical",
                                     dimension=groups + 2, params_size=2,
                                     logpdf="hierarchical_logpdf")


HROWS_BATCH = {"prep": "hrows_prep", "term": "hrows_term", "walker": "hrows_walker",
               "row_len": 3, "prep_len": 1}


def hierarchical_rows_model(groups):
    """Gaussian hierarchical model on observation rows (y, group, -1/(2 sigma^2)), plain
    single-model form, D = groups + 2; also the batch family member of that dimension."""
    return device_distribution_model(get_source("hierarchical_rows"), name="hrows",
                                     dimension=groups + 2, params_size=2,
                                     logpdf="hrows_logpdf", batch=HROWS_BATCH)


def hierarchical_rows_batch_model(max_groups=128):
    """The batch family of the row-encoded hierarchical model (runtime dimension up to
    max_groups + 2): many independent models advanced by one bay_batch."""
    return device_distribution_model(get_source("hierarchical_rows"), name="hrows",
                                     dimension=max_groups + 2, params_size=2,
                                     logpdf="hrows_logpdf", batch=HROWS_BATCH)


def hierarchical_rows_params(groups_y, sigmas, h0=10.0, h1=1.0):
    """params of the row-encoded hierarchical model: one row (y, j, -1/(2 sigma_j^2)) per
    observation of group j, then (h0, h1).  Returns (params float32, rows)."""
    rows = []
    for j, (y, s) in enumerate(zip(groups_y, sigmas)):
        y = np.asarray(y, np.float32)
        r = np.empty((y.size, 3), np.float32)
        r[:, 0] = y
        r[:, 1] = j
        r[:, 2] = -0.5 / (float(s) * float(s))
        rows.append(r)
    rows = np.concatenate(rows) if rows else np.zeros((0, 3), np.float32)
    return np.concatenate([rows.reshape(-1), np.array([h0, h1], np.float32)]), rows.shape[0]
