"""User-level distributions, mirroring uncomplicate.bayadera.library (library.clj:76-175) and
the distribution types of internal/distribution_library.clj.

Each distribution holds its parameters in the layout the device models read (the
reference's distributions.clj `*-params`: the parameters, then a log-normalising constant
where the density needs one), samples through the direct sampler engine (uniform,
Gaussian, exponential, Erlang) or through an MCMC sampler set up and warmed up as the
reference does (Student's t, beta, gamma: distribution_library.clj:97-106 and the beta /
gamma types), evaluates its density and log density through the distribution engine, and
gives the closed-form mean, mode, median and variance.

    with core.with_bayadera() as f:
        d = library.student_t(f, 4.0, 1.0, 2.0)
        s = d.sampler({"walkers": 8192})
        x = core.sample(s, 8192)
"""
import math
import random

import numpy as np

from . import models as M


def _log_beta(a, b):
    return math.lgamma(a) + math.lgamma(b) - math.lgamma(a + b)


def _beta_median(a, b):
    """beta-median (distributions.clj:559-569): closed forms where they exist, the exact
    medians of Beta(3, 2) and Beta(2, 3) (the root of 4x^3 - 3x^4 = 1/2), the
    (a - 1/3) / (a + b - 2/3) approximation for a, b > 1, NaN otherwise."""
    if a == b:
        return 0.5
    if a == 1.0 and b > 0.0:
        return 1.0 - 2.0 ** (-1.0 / b)
    if b == 1.0 and a > 0.0:
        return 2.0 ** (-1.0 / a)
    if (a, b) in ((3.0, 2.0), (2.0, 3.0)):
        lo, hi = 0.0, 1.0                          # Beta(3, 2) CDF 4x^3 - 3x^4, increasing
        for _ in range(200):
            mid = 0.5 * (lo + hi)
            if 4.0 * mid ** 3 - 3.0 * mid ** 4 < 0.5:
                lo = mid
            else:
                hi = mid
        m = 0.5 * (lo + hi)
        return m if a == 3.0 else 1.0 - m
    if a > 1.0 and b > 1.0:
        return (a - 1.0 / 3.0) / (a + b - 2.0 / 3.0)
    return math.nan


class DirectSampler:
    """DirectSampler (impl.clj:49-68): each sample call advances the seed by one, then draws
    n values with the direct sampler engine (n defaults to the factory's processing
    elements)."""

    def __init__(self, factory, kind, params, sample_count, seed):
        self.factory = factory
        self.kind = kind
        self.params = params
        self.sample_count = int(sample_count)
        self.seed = int(seed)

    def sample(self, n=None):
        n = self.sample_count if n is None else int(n)
        self.seed = (self.seed + 1) & 0xffffffff
        n4 = (n + 3) // 4 * 4                      # the engine draws four values a Philox call
        return self.factory.direct_sample(self.kind, self.seed, self.params, n4)[:n].reshape(1, n)

    def release(self):
        pass


class LibraryDistribution:
    """A distribution of the library with concrete parameters."""

    direct = None            # direct sampler kind, or None for an MCMC sampler

    def __init__(self, factory, name, params):
        self.factory = factory
        self.name = name
        self.params = np.asarray(params, np.float32)
        self.model = M.distribution_models()[name]
        self._engine = None
        self._mcmc = None

    # the distribution engine (density, log density)
    def _eng(self):
        if self._engine is None:
            self._engine = self.factory.distribution_engine(self.model)
        return self._engine

    def log_density(self, x):
        return self._eng().log_density(self.params, np.asarray(x, np.float32).reshape(-1, 1))

    def density(self, x):
        return self._eng().density(self.params, np.asarray(x, np.float32).reshape(-1, 1))

    def sd(self):
        return math.sqrt(self.variance())

    def _seed(self, options):
        if options and options.get("seed") is not None:
            return int(options["seed"])
        return random.SystemRandom().getrandbits(31)

    def sampler(self, options=None):
        o = options or {}
        if self.direct is not None:
            return DirectSampler(self.factory, self.direct, self.params,
                                 self.factory.processing_elements(), self._seed(o))
        # MCMC: walkers, limits and a burn-in at a = 8 as distribution_library.clj sets them
        walkers = o.get("walkers") or self.factory.processing_elements() * 256
        seed = self._seed(o)
        if self._mcmc is None:
            self._mcmc = self.factory.mcmc_factory(self.model, form="plain")
        samp = self._mcmc.create_sampler(seed, walkers, self.params)
        samp.init_position(seed + 1, list(self.mcmc_limits()))
        samp.burn_in(max(0, int(o.get("warm_up", 128))), 8.0)
        return samp

    def release(self):
        if self._engine is not None:
            self._engine.release()
            self._engine = None
        if self._mcmc is not None:
            self._mcmc.release()
            self._mcmc = None


class Uniform(LibraryDistribution):
    direct = "uniform"

    def __init__(self, factory, a, b):
        if not a < b:
            raise ValueError("Uniform distribution parameters are illegal: a is not less than b.")
        super().__init__(factory, "uniform", [a, b])
        self.a, self.b = float(a), float(b)

    def mean(self):
        return 0.5 * (self.a + self.b)

    mode = median = mean

    def variance(self):
        return (self.b - self.a) ** 2 / 12.0


class Gaussian(LibraryDistribution):
    direct = "gaussian"

    def __init__(self, factory, mu, sigma):
        if not sigma > 0.0:
            raise ValueError("Gaussian distribution parameters are illegal: sigma is not positive.")
        super().__init__(factory, "gaussian", [mu, sigma])
        self.mu, self.sigma = float(mu), float(sigma)

    def mean(self):
        return self.mu

    mode = median = mean

    def variance(self):
        return self.sigma ** 2


class StudentT(LibraryDistribution):
    def __init__(self, factory, nu, mu=0.0, sigma=1.0):
        if not (nu > 0.0 and sigma > 0.0):
            raise ValueError("Student's t distribution parameters are illegal: "
                             "nu and sigma must be positive.")
        log_scale = (math.lgamma(0.5 * (nu + 1.0)) - math.lgamma(0.5 * nu)
                     - 0.5 * math.log(nu * math.pi) - math.log(sigma))
        super().__init__(factory, "student_t", [nu, mu, sigma, log_scale])
        self.nu, self.mu, self.s = float(nu), float(mu), float(sigma)

    def mean(self):
        return self.mu if self.nu > 1.0 else math.nan

    mode = median = mean

    def variance(self):
        if self.nu > 2.0:
            return self.s * self.s * self.nu / (self.nu - 2.0)
        return math.inf if self.nu > 1.0 else math.nan

    def mcmc_limits(self):
        m, sd = self.mean(), math.sqrt(self.variance())
        return m - 10.0 * sd, m + 10.0 * sd


class Beta(LibraryDistribution):
    def __init__(self, factory, a, b):
        if not (a > 0.0 and b > 0.0):
            raise ValueError("Beta distribution parameters are illegal: a and b must be positive.")
        super().__init__(factory, "beta", [a, b, -_log_beta(a, b)])
        self.a, self.b = float(a), float(b)

    def mean(self):
        return self.a / (self.a + self.b)

    def mode(self):
        if self.a > 1.0 and self.b > 1.0:
            return (self.a - 1.0) / (self.a + self.b - 2.0)
        return math.nan

    def median(self):
        return _beta_median(self.a, self.b)

    def variance(self):
        s = self.a + self.b
        return self.a * self.b / (s * s * (s + 1.0))

    def mcmc_limits(self):
        return 0.0, 1.0


class Gamma(LibraryDistribution):
    def __init__(self, factory, theta, k):
        if not (theta > 0.0 and k > 0.0):
            raise ValueError("Gamma distribution parameters are illegal: theta and k must be positive.")
        super().__init__(factory, "gamma", [theta, k, -(math.lgamma(k) + k * math.log(theta))])
        self.theta, self.k = float(theta), float(k)

    def mean(self):
        return self.k * self.theta

    def mode(self):
        return (self.k - 1.0) * self.theta if self.k >= 1.0 else None

    def median(self):
        raise NotImplementedError("No closed form for gamma median.")

    def variance(self):
        return self.k * self.theta * self.theta

    def mcmc_limits(self):
        return 0.0, self.mean() + 2.0 * math.sqrt(self.variance())


class Exponential(LibraryDistribution):
    direct = "exponential"

    def __init__(self, factory, lam):
        if not lam > 0.0:
            raise ValueError("Exponential distribution parameters are illegal: lambda is not positive.")
        super().__init__(factory, "exponential", [lam, math.log(lam)])
        self.lam = float(lam)

    def mean(self):
        return 1.0 / self.lam

    def mode(self):
        return 0.0

    def median(self):
        return math.log(2.0) / self.lam

    def variance(self):
        return 1.0 / (self.lam * self.lam)


class Erlang(LibraryDistribution):
    direct = "erlang"

    def __init__(self, factory, lam, k):
        k = int(k)
        if not (lam > 0.0 and k > 0):
            raise ValueError("Erlang distribution parameters are illegal: lambda and k must be positive.")
        super().__init__(factory, "erlang", [lam, k, k * math.log(lam) - math.lgamma(k)])
        self.lam, self.k = float(lam), k

    def mean(self):
        return self.k / self.lam

    def mode(self):
        return (self.k - 1) / self.lam

    def median(self):
        return (self.k / self.lam) / (1.0 - 1.0 / (3.0 * self.k + 0.2))

    def variance(self):
        return self.k / (self.lam * self.lam)


def uniform(factory, a, b):
    return Uniform(factory, a, b)


def gaussian(factory, mu, sigma):
    return Gaussian(factory, mu, sigma)


def student_t(factory, nu, mu=0.0, sigma=1.0):
    return StudentT(factory, nu, mu, sigma)


def beta(factory, a, b):
    return Beta(factory, a, b)


def gamma(factory, theta, k):
    return Gamma(factory, theta, k)


def exponential(factory, lam):
    return Exponential(factory, lam)


def erlang(factory, lam, k):
    return Erlang(factory, lam, k)
