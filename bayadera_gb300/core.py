"""Public API, mirroring uncomplicate.bayadera.core (src/clojure/uncomplicate/bayadera/core.clj).

    with with_bayadera() as f:
        post = distribution(f, likelihood_model, prior_model)      # posterior creator
        d = post(data)                                             # params = data || hyper
        s = sampler(d, {"walkers": 4096, "limits": [...]})
        burn_in(s, 512, 2.0); run_sampler(s, 1024, 2.0)
        mean(s), variance(s), histogram(s)
"""
import contextlib
import os
import random

import numpy as np

from . import models as M
from .engine import GB300BayaderaFactory

_default_factory = []


@contextlib.contextmanager
def with_bayadera(device=0, wgs=1024, stream=None, mem_limit=0):
    """with-bayadera / with-default-bayadera (core.clj:24-27, cuda.clj:27-31)."""
    f = GB300BayaderaFactory(device, wgs, stream, mem_limit)
    _default_factory.append(f)
    try:
        yield f
    finally:
        _default_factory.pop()
        f.release()


def _factory(f):
    if f is not None:
        return f
    if not _default_factory:
        raise RuntimeError("no bayadera factory: use `with with_bayadera():`")
    return _default_factory[-1]


def generate_seed():
    return random.SystemRandom().getrandbits(31)


class DistributionImpl:
    """DistributionImpl (impl.clj:84-116): a model with concrete params."""

    def __init__(self, factory, sampler_factory, params):
        self.factory = factory
        self.sampler_factory = sampler_factory
        self.params = params

    @property
    def model(self):
        return self.sampler_factory.model

    def sampler(self, options=None):
        o = options or {}
        walkers = o.get("walkers") or 2 * self.factory.processing_elements()
        samp = self.sampler_factory.create_sampler(o.get("seed", generate_seed()), walkers,
                                                   self.params)
        lim = o.get("limits")
        if lim is None:
            lim = self.model.limits
        if lim is not None:
            samp.init_position(generate_seed() if o.get("position_seed") is None
                               else o["position_seed"], lim)
        if o.get("positions") is not None:
            samp.init_position(o["positions"])
        return samp


class DistributionCreator:
    """DistributionCreator / PosteriorCreator (impl.clj:124-163)."""

    def __init__(self, factory, model, hyperparams=None, **compile_opts):
        self.factory = factory
        self.model = model
        self.hyperparams = None if hyperparams is None else np.asarray(hyperparams, np.float32)
        self.sampler_factory = factory.mcmc_factory(model, **compile_opts)

    def __call__(self, data_or_params, hyperparams=None):
        h = self.hyperparams if hyperparams is None else np.asarray(hyperparams, np.float32)
        if h is not None:
            if h.size != self.model.params_size:
                raise ValueError("Dimension of params must match the distribution.")
            params = np.concatenate([np.asarray(data_or_params, np.float32).reshape(-1), h])
        else:
            params = data_or_params
            if getattr(params, "size", None) is not None and params.size != self.model.params_size:
                raise ValueError("Dimension of params must match the distribution.")
        return DistributionImpl(self.factory, self.sampler_factory, params)

    def release(self):
        self.sampler_factory.release()


class Dataset:
    """DatasetImpl (impl.clj:25-45): a data matrix (n points x dim) whose mean, variance,
    sd and histogram come from the dataset engine (nvidia_gtx.clj:145-228)."""

    def __init__(self, factory, data):
        x = np.ascontiguousarray(data, np.float32)
        if x.ndim == 1:
            x = x[:, None]
        if x.ndim != 2 or x.size == 0:
            raise ValueError("The engine can not support this data: a non-empty n x dim matrix.")
        self.factory = factory
        self.data = x

    def mean(self):
        return self.factory.data_moments(self.data)[0]

    def variance(self):
        return self.factory.data_moments(self.data)[1]

    def sd(self):
        return np.sqrt(self.variance())

    def histogram(self, cycles=1, bins=0, flags=0):
        return self.factory.data_histogram(self.data, bins, flags)


def dataset(*args):
    """dataset (core.clj:31-45): dataset(data) or dataset(factory, data)."""
    if len(args) == 2:
        return Dataset(_factory(args[0]), args[1])
    return Dataset(_factory(None), args[0])


class Likelihood:
    """LikelihoodImpl (impl.clj): a likelihood model with its engine; the engine is compiled
    for the dimension of the points it is evaluated at (the prior sample's)."""

    def __init__(self, factory, model):
        self.factory = factory
        self.model = model
        self._engines = {}

    def engine(self, dim):
        if dim not in self._engines:
            self._engines[dim] = self.factory.likelihood_engine(self.model, dim)
        return self._engines[dim]

    def release(self):
        for e in self._engines.values():
            e.release()
        self._engines.clear()


def likelihood(*args):
    """likelihood (core.clj:58-66): likelihood(model) or likelihood(factory, model)."""
    if len(args) == 2:
        return Likelihood(_factory(args[0]), args[1])
    return Likelihood(_factory(None), args[0])


def posterior_model(likelihood, prior, name=None):
    """posterior-model (core.clj:49-56)."""
    return M.device_posterior_model(prior, name or "posterior", likelihood)


def distribution(*args, **compile_opts):
    """distribution (core.clj:68-86):
       distribution(model) / distribution(factory, model)
       distribution(factory, likelihood, prior[, hyperparams]) -> a posterior creator."""
    args = list(args)
    factory = args.pop(0) if args and isinstance(args[0], GB300BayaderaFactory) else None
    factory = _factory(factory)
    if len(args) == 1:
        return DistributionCreator(factory, args[0], **compile_opts)
    lik, prior = args[0], args[1]
    hyper = args[2] if len(args) > 2 else None
    return DistributionCreator(factory, posterior_model(lik, prior), hyper, **compile_opts)


def sampler(dist, options=None):
    return dist.sampler(options)


def sample(samp, n=None):
    return samp.sample(n)


def sample_(samp, out):
    """sample! (core.clj:131-137): fill a contiguous dim x n matrix with n samples."""
    if not (isinstance(out, np.ndarray) and out.ndim == 2 and out.flags.c_contiguous):
        raise ValueError("Data has to be a contiguous matrix.")
    out[...] = samp.sample(out.shape[1])
    return out


def mean(x):
    return x.mean()


def variance(x):
    return x.variance()


def sd(x):
    return x.sd()


def histogram(x, cycles=1, bins=0, flags=0):
    return x.histogram(cycles, bins, flags)


def histogram_(x, n):
    """histogram! (core.clj:145-147)."""
    return x.histogram(n)


def log_density(dist, x):
    """log-density (core.clj:105-113): the distribution's logpdf at the points x (n x dim)."""
    eng = dist.factory.distribution_engine(dist.model)
    try:
        return eng.log_density(dist.params, x)
    finally:
        eng.release()


def density(dist, x):
    """density (core.clj:105-113)."""
    eng = dist.factory.distribution_engine(dist.model)
    try:
        return eng.density(dist.params, x)
    finally:
        eng.release()


def evidence(*args):
    """evidence (core.clj:115-121): the mean likelihood of data over the points of a prior
    sample (n x dim).  evidence(lik, data, prior_sample) with lik from likelihood(...), as
    the reference; or evidence(factory, likelihood_model, data, prior_sample)."""
    if len(args) == 3:
        lik, data, x = args
        x = np.asarray(x, np.float32)
        return lik.engine(x.shape[-1]).evidence(data, x)
    factory, model, data, x = args
    x = np.asarray(x, np.float32)
    eng = _factory(factory).likelihood_engine(model, x.shape[-1])
    try:
        return eng.evidence(data, x)
    finally:
        eng.release()
