"""MCMC driver functions, mirroring uncomplicate.bayadera.mcmc
(src/clojure/uncomplicate/bayadera/mcmc.clj)."""
import math


def init_position(samp, seed_or_position, limits=None):
    return samp.init_position(seed_or_position, limits)


def acc_rate(samp, a=2.0):
    """acc-rate! (mcmc.clj:21-25)."""
    return float(samp.acc_rate(a))


def burn_in(samp, steps=None, a=2.0):
    """burn-in! (mcmc.clj:27-33): default 256 * dim steps."""
    return samp.burn_in(256 * samp.dim if steps is None else steps, a)


def run_sampler(samp, steps=None, a=2.0, **kw):
    """run-sampler! (mcmc.clj:35-41): default 64 * dim steps."""
    return samp.run_sampler(64 * samp.dim if steps is None else steps, a, **kw)


def sqrt_n(temp):
    return lambda i: math.sqrt(temp - i)


def pow_n(power):
    return lambda temp: (lambda i: math.pow(temp - i, power))


def minus_n(temp):
    return lambda i: temp - i


def anneal(samp, steps=None, a=2.0, schedule=minus_n):
    """anneal! (mcmc.clj:43-64): temperature schedule(steps)(i) at step i."""
    steps = 256 * samp.dim if steps is None else int(steps)
    return samp.anneal(schedule(steps), steps, a)


def adapt_a_host(samp, step, a, min_acc, max_acc):
    """mix!'s a-adaptation loop (mcmc.clj:84-91) run from the host, one acc-rate! probe
    (and one readback) per iteration; returns (a, the last probe's rate, probes)."""
    target = (max_acc + min_acc) / 2.0
    i = probes = 0
    while True:
        r = samp.acc_rate(a)
        probes += 1
        if step < i:
            break
        if r < min_acc:
            a = 1.0 + (a - 1.0) * (r / target)
        elif max_acc < r:
            a = a * (r / target)
        else:
            break
        i += 1
    return a, r, probes


def mix(samp, options=None, on_device=True):
    """mix! (mcmc.clj:66-101): anneal, adapt a toward the acceptance window, burn in.
    on_device: the adaptation loop runs inside one CUDA graph (bay_adapt_a); else from
    the host (adapt_a_host).  Both give the same a and the same sampler state."""
    o = options or {}
    step = int(o.get("step", 64))
    dim_pow = float(o.get("dimension_power", 0.8))
    schedule = o.get("cooling_schedule", minus_n)
    a = float(o.get("a", 2.0))
    min_acc = float(o.get("min_acc_rate", 0.2))
    max_acc = float(o.get("max_acc_rate", 0.5))
    nf = step * math.pow(samp.dim, dim_pow)  # the reference keeps the fractional count
    n = int(nf)                              # as the temperature and runs floor(nf) steps
    samp.anneal(schedule(nf), n, a)
    if on_device:
        a = samp.adapt_a(step, a, min_acc, max_acc)["a"]
    else:
        a = adapt_a_host(samp, step, a, min_acc, max_acc)[0]
    samp.burn_in(n, a)
    samp.burn_in(step, 2.0)
    return {"a": a, "acc_rate": samp.acc_rate(a), "acc_rate_2": samp.acc_rate(2.0)}
