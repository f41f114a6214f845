"""GB300 engine objects over the C ABI (mirrors internal/device/nvidia_gtx.clj).

GB300BayaderaFactory  <- GTXBayaderaFactory (nvidia_gtx.clj:761-807)
GB300StretchFactory   <- GTXStretchFactory  (nvidia_gtx.clj:543-610)
GB300Stretch          <- GTXStretch         (nvidia_gtx.clj:282-541)
GB300AcorEngine       <- GTXAcorEngine      (nvidia_gtx.clj:230-278)

Host arrays are numpy; positions are dim x walkers (column-major in memory, i.e.
a (walkers, dim) C-contiguous numpy array viewed transposed), as in the reference.
"""
import ctypes as C
from collections import namedtuple

import numpy as np

from . import _native as N

Histogram = namedtuple("Histogram", ["limits", "pdf", "bin_ranks"])
Autocorrelation = namedtuple("Autocorrelation", ["tau", "mean", "sigma", "steps", "lag"])


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


def _dev_ptr(t):
    """Device pointer of an object with data_ptr() (a CUDA tensor), else None."""
    dp = getattr(t, "data_ptr", None)
    if dp is not None and getattr(getattr(t, "device", None), "type", "cpu") == "cuda":
        return C.c_void_p(dp())
    return None


class GB300AcorEngine:
    def __init__(self, factory):
        self.factory = factory

    def acor(self, data_matrix):
        """AcorEngine/acor on a dim x n matrix (numpy (dim, n) array)."""
        m = np.asarray(data_matrix, np.float32)
        if m.ndim == 1:
            m = m[None, :]
        dim, n = m.shape
        series = np.ascontiguousarray(m.T)  # column-major dim x n
        tau = np.zeros(dim)
        mean = np.zeros(dim)
        sigma = np.zeros(dim)
        lag = C.c_uint32(0)
        N.call("bay_acor", self.factory.ctx, _ptr(series), dim, n, _ptr(tau), _ptr(mean),
               _ptr(sigma), C.byref(lag))
        return Autocorrelation(tau, mean, sigma, n, lag.value)


class GB300BayaderaFactory:
    """Context: one device, one stream, the reference's WGS."""

    def __init__(self, device=0, wgs=1024, stream=None, mem_limit=0):
        opts = N.CtxOpts(device, wgs, stream, mem_limit)
        h = C.c_void_p()
        N.call("bay_ctx_create", C.byref(opts), C.byref(h))
        self.ctx = h
        self.wgs = wgs
        self.acor_engine = GB300AcorEngine(self)

    def release(self):
        if self.ctx:
            N.call("bay_ctx_release", self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.release()

    def processing_elements(self):
        v = C.c_uint64()
        N.call("bay_ctx_processing_elements", self.ctx, C.byref(v))
        return v.value

    def stream(self):
        s = C.c_void_p()
        N.call("bay_ctx_stream", self.ctx, C.byref(s))
        return s.value

    def synchronize(self):
        N.call("bay_ctx_synchronize", self.ctx)

    def allocated(self):
        v = C.c_uint64()
        N.call("bay_ctx_allocated", self.ctx, C.byref(v))
        return v.value

    def autotune(self, model, walkers, params, form=None, tensor=False, positions=None):
        """bay_autotune: the fastest kernel shape of the model's form on this workload (the
        tiled form's walkers per CTA, CTA threads and row slices, the streamed tensor-core
        form's sub-tiles and stages, the resident one's tile groups), timed on the device;
        pass the result's shape keys to mcmc_factory."""
        d, keep = model_desc(model, form, tensor=tensor)
        r = N.TuneResult()
        dp = _dev_ptr(params)
        if dp is not None:
            pp, n = dp, int(params.numel())
        else:
            p = np.ascontiguousarray(params, np.float32).reshape(-1)
            keep.append(p)
            pp, n = _ptr(p), p.size
        pos = None
        if positions is not None:
            pos = np.ascontiguousarray(positions, np.float32)
        N.call("bay_autotune", self.ctx, C.byref(d), int(walkers), pp, n,
               _ptr(pos) if pos is not None else None, C.byref(r))
        shape = {}
        if r.walkers_per_cta:
            shape.update(walkers_per_cta=r.walkers_per_cta, cta_threads=r.cta_threads)
        if r.tile_slices > 1:
            shape.update(tile_slices=r.tile_slices)
        if r.tc_subtiles:
            shape.update(tc_subtiles=r.tc_subtiles, tc_stages=r.tc_stages)
        if r.tc_groups:
            shape.update(tc_groups=r.tc_groups)
        return {"shape": shape, "candidates": r.candidates, "from_cache": bool(r.from_cache),
                "us_per_step": r.us_per_step, "default_us_per_step": r.default_us_per_step}

    def mcmc_factory(self, model, form=None, accept_ref=False, walkers_per_cta=0,
                     cta_threads=0, streaming=False, tensor=False, stretch_ref=False,
                     partner_element=False, tc_subtiles=0, tc_stages=0, tc_groups=0,
                     tile_slices=0):
        """EngineFactory/mcmc-factory: compile the model's fused stretch kernels.  GEMM form:
        streaming=True streams the matrix even when it fits in shared memory; tensor=True
        streams it through the tensor cores (split bf16, fp32 accumulation).  Reference
        compatibility: accept_ref (fp32 accept formula), stretch_ref (the stretch factor's
        fast-math expression), partner_element (the element-offset partner, quirk Q1).
        Kernel shapes (0: the library's choice): walkers_per_cta, cta_threads, tile_slices
        (tiled form); tc_subtiles, tc_stages, tc_groups (tensor-core GEMM form)."""
        return GB300StretchFactory(self, model, form, accept_ref, walkers_per_cta, cta_threads,
                                   streaming, tensor, stretch_ref, partner_element, tc_subtiles,
                                   tc_stages, tc_groups, tile_slices)

    def acor(self, data_matrix):
        return self.acor_engine.acor(data_matrix)

    # ------------------------------------------------------------ engines (EngineFactory)
    def distribution_engine(self, model):
        """distribution-engine (protocols.clj:132-138): log-density / density of the model's
        logpdf at points."""
        return GB300DensityEngine(self, model)

    def likelihood_engine(self, likelihood, dim):
        """likelihood-engine: log-density / density / evidence of a likelihood model at
        points of dimension dim (data = the params)."""
        return GB300DensityEngine(self, likelihood, dim=dim)

    # ------------------------------------------------------------ dataset engine
    def data_moments(self, x):
        """data-mean and data-variance of a data matrix x (n points x dim) in FP64."""
        x = np.ascontiguousarray(x, np.float32)
        if x.ndim == 1:
            x = x[:, None]
        n, dim = x.shape
        mean = np.zeros(dim)
        var = np.zeros(dim)
        N.call("bay_data_moments", self.ctx, _ptr(x), dim, n, _ptr(mean), _ptr(var))
        return mean, var

    def data_histogram(self, x, bins=0, flags=0):
        """histogram of a data matrix x (n points x dim): Histogram(limits 2 x dim, pdf and
        bin ranks bins x dim)."""
        x = np.ascontiguousarray(x, np.float32)
        if x.ndim == 1:
            x = x[:, None]
        n, dim = x.shape
        bins = bins or self.wgs
        lim = np.zeros((dim, 2), np.float32)
        pdf = np.zeros((dim, bins), np.float32)
        ranks = np.zeros((dim, bins), np.float32)
        N.call("bay_data_histogram", self.ctx, _ptr(x), dim, n, bins, flags, _ptr(lim),
               _ptr(pdf), _ptr(ranks))
        return Histogram(lim.T, pdf.T, ranks.T)

    def direct_sample(self, kind, seed, params, n):
        """direct-sampler-engine sample: n samples (a multiple of 4) of uniform, gaussian,
        exponential or erlang with the given parameters."""
        kinds = {"uniform": N.DIRECT_UNIFORM, "gaussian": N.DIRECT_GAUSSIAN,
                 "exponential": N.DIRECT_EXPONENTIAL, "erlang": N.DIRECT_ERLANG}
        p = np.ascontiguousarray(params, np.float32)
        out = np.zeros(int(n), np.float32)
        N.call("bay_sample_direct", self.ctx, kinds[kind], _ptr(p), int(seed) & 0xffffffff,
               int(n), _ptr(out))
        return out


def model_desc(model, form=None, accept_ref=False, walkers_per_cta=0, cta_threads=0,
               streaming=False, tensor=False, stretch_ref=False, partner_element=False,
               tc_subtiles=0, tc_stages=0, tc_groups=0, tile_slices=0):
    """bay_model_desc of a DeviceDistributionModel; form 'plain' | 'tiled' | None (tiled
    when the model has a tiled form)."""
    if form is None:
        form = "gemm" if model.gemm else ("tiled" if model.tiled else "plain")
    keep = []

    def b(s):
        v = s.encode() if s is not None else None
        keep.append(v)
        return v

    d = N.ModelDesc()
    d.source = b(model.full_source())
    d.logfn = b(model.mcmc_logpdf)
    d.dim = model.dimension
    d.params_size = model.params_size
    d.flags = ((N.MODEL_ACCEPT_REF if accept_ref else 0) |
               (N.MODEL_GEMM_STREAMING if streaming else 0) |
               (N.MODEL_GEMM_TENSOR if tensor else 0) |
               (N.MODEL_STRETCH_REF if stretch_ref else 0) |
               (N.MODEL_PARTNER_ELEMENT if partner_element else 0))
    d.cta_threads = cta_threads
    d.tc_subtiles = tc_subtiles
    d.tc_stages = tc_stages
    d.tc_groups = tc_groups
    if form == "tiled":
        t = model.tiled
        if not t:
            raise ValueError("model %s has no tiled form" % model.name)
        d.form = N.FORM_TILED
        d.tile_prep = b(t["prep"])
        d.tile_term = b(t["term"])
        d.tile_walker = b(t["walker"])
        d.row_len = t["row_len"]
        d.prep_len = t["prep_len"]
        d.walkers_per_cta = walkers_per_cta
        d.tile_slices = tile_slices
    elif form == "batch":
        bt = model.batch
        if not bt:
            raise ValueError("model %s has no batch form" % model.name)
        d.form = N.FORM_BATCH
        d.tile_prep = b(bt["prep"])
        d.tile_term = b(bt["term"])
        d.tile_walker = b(bt["walker"])
        d.row_len = bt["row_len"]
        d.prep_len = bt.get("prep_len", 1)
    elif form == "gemm":
        gm = model.gemm
        if not gm:
            raise ValueError("model %s has no GEMM form" % model.name)
        d.form = N.FORM_GEMM
        d.tile_prep = b(gm["prep"])
        d.tile_term = b(gm["term"])
        d.tile_walker = b(gm["walker"])
        d.prep_len = gm.get("prep_len", 1)
        d.gemm_features = gm["features"]
        d.gemm_coef = gm.get("coef", 0)
        d.gemm_block = 1 if gm.get("block", "data") == "hyper" else 0
        d.gemm_ld = gm["ld"]
        d.gemm_offset = gm.get("offset", 0)
        d.gemm_rows = gm.get("rows", 0)
        d.gemm_aux_col = gm.get("aux_col", 0)
        d.gemm_aux_len = gm.get("aux_len", 0)
    else:
        d.form = N.FORM_PLAIN
    return d, keep


_LIK_ADAPTER = """
extern "C" {
inline REAL %(name)s(const uint32_t data_len, const uint32_t params_len, const REAL* params,
                     const uint32_t dim, const REAL* x) {
    return %(loglik)s(data_len, params, dim, x);
}
}
"""


class GB300DensityEngine:
    """DensityEngine / LikelihoodEngine (protocols.clj:59-72) of a distribution model (its
    logpdf) or of a likelihood model (its loglik through a 5-argument adapter, points of
    dimension dim), compiled in the plain form."""

    def __init__(self, factory, model, dim=None):
        from bayadera_gb300 import models as Mo
        if isinstance(model, Mo.DeviceLikelihoodModel):
            if dim is None:
                raise ValueError("a likelihood engine needs the points' dimension")
            name = "%s_bay_points" % model.loglik
            src = model.sources + [_LIK_ADAPTER % {"name": name, "loglik": model.loglik}]
            dm = Mo.device_distribution_model(src, name=name, logpdf=name, dimension=dim,
                                              params_size=0)
        else:
            dm = Mo.device_distribution_model(model.sources, name=model.name,
                                              logpdf=model.logpdf, dimension=model.dimension,
                                              params_size=model.params_size)
        self.model = model
        self.dim = dm.dimension
        self.sf = GB300StretchFactory(factory, dm, form="plain")

    def release(self):
        self.sf.release()

    def _pts(self, x):
        x = np.ascontiguousarray(x, np.float32)
        if x.ndim == 1:
            x = x.reshape(-1, self.dim)
        if x.shape[-1] != self.dim:
            raise ValueError("points must be n x %d" % self.dim)
        return x

    def _call(self, fn, params, x):
        p = np.ascontiguousarray(params, np.float32).reshape(-1)
        x = self._pts(x)
        out = np.zeros(x.shape[0], np.float32)
        N.call(fn, self.sf.handle, _ptr(p), p.size, _ptr(x), x.shape[0], _ptr(out))
        return out

    def log_density(self, params, x):
        return self._call("bay_log_density", params, x)

    def density(self, params, x):
        return self._call("bay_density", params, x)

    def evidence(self, params, x):
        p = np.ascontiguousarray(params, np.float32).reshape(-1)
        x = self._pts(x)
        r = C.c_double()
        N.call("bay_evidence", self.sf.handle, _ptr(p), p.size, _ptr(x), x.shape[0], C.byref(r))
        return r.value


def check_model(model, form=None, wgs=1024, accept_ref=False, tensor=False, stretch_ref=False,
                partner_element=False, walkers_per_cta=0, cta_threads=0, tc_subtiles=0,
                tc_stages=0, tc_groups=0, tile_slices=0):
    """Compile-check a model's fused kernels with NVRTC (no device needed)."""
    d, keep = model_desc(model, form, accept_ref, walkers_per_cta, cta_threads, tensor=tensor,
                         stretch_ref=stretch_ref, partner_element=partner_element,
                         tc_subtiles=tc_subtiles, tc_stages=tc_stages, tc_groups=tc_groups,
                         tile_slices=tile_slices)
    N.call("bay_model_check", C.byref(d), wgs)


class GB300StretchFactory:
    def __init__(self, factory, model, form=None, accept_ref=False, walkers_per_cta=0,
                 cta_threads=0, streaming=False, tensor=False, stretch_ref=False,
                 partner_element=False, tc_subtiles=0, tc_stages=0, tc_groups=0,
                 tile_slices=0):
        self.factory = factory
        self.model = model
        d, keep = model_desc(model, form, accept_ref, walkers_per_cta, cta_threads, streaming,
                             tensor, stretch_ref, partner_element, tc_subtiles, tc_stages,
                             tc_groups, tile_slices)
        h = C.c_void_p()
        N.call("bay_model_compile", factory.ctx, C.byref(d), C.byref(h))
        self.handle = h

    def release(self):
        if self.handle:
            N.call("bay_model_release", self.handle)
            self.handle = None

    def create_sampler(self, seed, walkers, params):
        """SamplerFactory/create-sampler: params = data || hyperparameters (numpy, or a
        CUDA tensor that stays resident and must outlive the sampler)."""
        return GB300Stretch(self, seed, walkers, params)

    def create_batch(self, members, shape=None):
        """A batch of independent models of this (batch-form) family; members is a list of
        dicts {dim, seed, walkers, params (numpy float32: rows || hyperparameters), rows};
        shape: the work lists' {rows_per_thread, walkers_per_item, chunk_floats} (e.g. from
        autotune_batch), None = the library's."""
        return GB300Batch(self, members, shape)

    def autotune_batch(self, members):
        """bay_batch_autotune: the fastest work-list shape for these members."""
        arr, keep = _batch_members(members)
        r = N.BatchTuneResult()
        N.call("bay_batch_autotune", self.handle, arr, len(members), C.byref(r))
        return {"shape": {"rows_per_thread": r.shape.rows_per_thread,
                          "walkers_per_item": r.shape.walkers_per_item,
                          "chunk_floats": r.shape.chunk_floats,
                          "walkers_per_thread": r.shape.walkers_per_thread},
                "candidates": r.candidates, "from_cache": bool(r.from_cache),
                "us_per_step": r.us_per_step, "default_us_per_step": r.default_us_per_step}


def _batch_members(members):
    arr = (N.BatchMember * len(members))()
    keep = []
    for i, m in enumerate(members):
        p = np.ascontiguousarray(m["params"], np.float32)
        keep.append(p)
        arr[i].dim = int(m["dim"])
        arr[i].seed = int(m["seed"]) & 0xffffffff
        arr[i].walkers = int(m["walkers"])
        arr[i].params = p.ctypes.data
        arr[i].n_params = p.size
        arr[i].rows = int(m["rows"])
    return arr, keep


class GB300Batch:
    """Many independent models of one family advanced together (bay_batch_*): member m
    behaves as GB300Stretch(seed_m, walkers_m, params_m) of dimension dim_m."""

    def __init__(self, sfactory, members, shape=None):
        self.sfactory = sfactory
        self.members = [dict(m) for m in members]
        arr, keep = _batch_members(self.members)
        h = C.c_void_p()
        if shape:
            sh = N.BatchShape(int(shape.get("rows_per_thread", 0)),
                              int(shape.get("walkers_per_item", 0)),
                              int(shape.get("chunk_floats", 0)),
                              int(shape.get("walkers_per_thread", 0)))
            N.call("bay_batch_create_shaped", sfactory.handle, arr, len(members), C.byref(sh),
                   C.byref(h))
        else:
            N.call("bay_batch_create", sfactory.handle, arr, len(members), C.byref(h))
        self.handle = h
        self.dims = np.array([m["dim"] for m in self.members], np.int64)
        self.walkers = np.array([m["walkers"] for m in self.members], np.int64)

    def release(self):
        if self.handle:
            N.call("bay_batch_release", self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.release()

    def info(self):
        w, f, it = C.c_uint64(), C.c_uint64(), C.c_uint64()
        N.call("bay_batch_info", self.handle, C.byref(w), C.byref(f), C.byref(it))
        return {"walkers": w.value, "floats": f.value, "items": it.value}

    def set_graphs(self, enabled):
        N.call("bay_batch_set_graphs", self.handle, 1 if enabled else 0)

    def set_persistent(self, enabled):
        """One persistent cooperative launch per chunk of steps for every member, or three
        launches per half-step (default); both give the same results."""
        N.call("bay_batch_set_persistent", self.handle, 1 if enabled else 0)

    def arm_barrier_timeout(self, enabled):
        """Testing the device failure path: the persistent launch's grid barriers wait for
        one CTA more than the launch has and run out after their bounded wait."""
        N.call("bay_batch_test_barrier_timeout", self.handle, 1 if enabled else 0)

    def init_position_normal(self, seeds, mean=0.0, sd=1.0):
        sd_ = np.ascontiguousarray(seeds, np.uint32)
        if sd_.size != len(self.members):
            raise ValueError("one seed per member")
        N.call("bay_batch_init_position_normal", self.handle, _ptr(sd_), mean, sd)
        return self

    def init_position(self, positions):
        """positions: a list of (walkers_m, dim_m) arrays."""
        flat = np.concatenate([np.ascontiguousarray(p, np.float32).reshape(-1)
                               for p in positions])
        if flat.size != int(np.sum(self.dims * self.walkers)):
            raise ValueError("positions must hold walkers_m x dim_m values per member")
        N.call("bay_batch_init_position_host", self.handle, _ptr(flat))
        return self

    def burn_in(self, n, a):
        N.call("bay_batch_burn_in", self.handle, int(n), float(a))
        return self

    def run_sampler(self, n, a, return_means=False):
        rates = np.zeros(len(self.members))
        flat = np.zeros(int(np.sum(self.dims)) * int(n), np.float32) if return_means else None
        N.call("bay_batch_run_sampler", self.handle, int(n), float(a), _ptr(rates),
               _ptr(flat) if flat is not None else None)
        out = {"acceptance_rates": rates}
        if flat is not None:
            means, o = [], 0
            for d in self.dims:
                means.append(flat[o:o + n * d].reshape(n, d).T)
                o += n * d
            out["means"] = means
        return out

    def _split(self, flat, per):
        out, o = [], 0
        for p in per:
            out.append(flat[o:o + p])
            o += p
        return out

    def positions(self):
        """list of (walkers_m, dim_m) arrays"""
        flat = np.zeros(int(np.sum(self.dims * self.walkers)), np.float32)
        N.call("bay_batch_state_export", self.handle, _ptr(flat), None)
        return [f.reshape(w, d) for f, w, d in
                zip(self._split(flat, self.dims * self.walkers), self.walkers, self.dims)]

    def logfn(self):
        flat = np.zeros(int(np.sum(self.walkers)), np.float32)
        N.call("bay_batch_state_export", self.handle, None, _ptr(flat))
        return self._split(flat, self.walkers)


class GB300Stretch:
    def __init__(self, sfactory, seed, walkers, params):
        self.sfactory = sfactory
        self.model = sfactory.model
        self.dim = self.model.dimension
        self.walkers = int(walkers)
        h = C.c_void_p()
        dp = _dev_ptr(params)
        if dp is not None:
            self._params_ref = params
            N.call("bay_sampler_create_device", sfactory.handle, seed & 0xffffffff, self.walkers,
                   dp, int(params.numel()), C.byref(h))
        else:
            p = np.ascontiguousarray(params, np.float32).reshape(-1)
            N.call("bay_sampler_create", sfactory.handle, seed & 0xffffffff, self.walkers, _ptr(p),
                   p.size, C.byref(h))
        self.handle = h

    def release(self):
        if self.handle:
            N.call("bay_sampler_release", self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.release()

    def info(self):
        i = N.SamplerInfo()
        N.call("bay_sampler_info_get", self.handle, C.byref(i))
        return {"walker_count": i.walkers, "iteration_counter": i.iteration_counter,
                "dimension": i.dim, "data_len": i.data_len}

    def set_graphs(self, enabled):
        N.call("bay_sampler_set_graphs", self.handle, 1 if enabled else 0)

    def set_persistent(self, enabled):
        """Resident tensor-core GEMM form: one persistent cooperative launch per chunk of
        steps, or one launch per half-step (default); both give the same results."""
        N.call("bay_sampler_set_persistent", self.handle, 1 if enabled else 0)

    def arm_barrier_timeout(self, enabled):
        """Testing the device failure path: the persistent form's grid barriers wait for one
        CTA more than the launch has, run out after their bounded wait and set the status
        word (the next status check raises)."""
        N.call("bay_sampler_test_barrier_timeout", self.handle, 1 if enabled else 0)

    # ---------------------------------------------------------------- MCMC
    def init(self, seed):
        N.call("bay_init", self.handle, seed & 0xffffffff)
        return self

    def init_position(self, seed_or_position, limits=None):
        if isinstance(seed_or_position, GB300Stretch):
            N.call("bay_init_position_copy", self.handle, seed_or_position.handle)
        elif limits is None:
            pos = np.ascontiguousarray(seed_or_position, np.float32)
            if pos.shape != (self.walkers, self.dim) and pos.size != self.walkers * self.dim:
                raise ValueError("positions must hold walkers x dim values")
            N.call("bay_init_position_host", self.handle, _ptr(pos))
        else:
            lim = np.ascontiguousarray(limits, np.float32).reshape(-1)
            if lim.size != 2 * self.dim:
                raise ValueError("limits must be a 2 x dim matrix")
            N.call("bay_init_position_limits", self.handle, seed_or_position & 0xffffffff,
                   _ptr(lim))
        return self

    def init_position_normal(self, seed, mean=0.0, sd=1.0):
        N.call("bay_init_position_normal", self.handle, seed & 0xffffffff, mean, sd)
        return self

    def burn_in(self, n, a):
        N.call("bay_burn_in", self.handle, int(n), float(a))
        return self

    def anneal(self, schedule, n, a):
        temps = np.array([schedule(i) for i in range(int(n))], np.float32)
        N.call("bay_anneal", self.handle, _ptr(temps), int(n), float(a))
        return self

    def acc_rate(self, a):
        r = C.c_double()
        N.call("bay_acc_rate", self.handle, float(a), C.byref(r))
        return r.value

    def adapt_a(self, step, a, min_acc, max_acc):
        """mix!'s a-adaptation loop (mcmc.clj:84-91) on the device (bay_adapt_a): returns
        {a, acc_rate (the last probe's), probes}."""
        r = N.AdaptResult()
        N.call("bay_adapt_a", self.handle, int(step), float(a), float(min_acc), float(max_acc),
               C.byref(r))
        return {"a": r.a, "acc_rate": r.acc_rate, "probes": r.probes}

    def run_sampler(self, n, a, return_means=False):
        res = N.RunResult()
        tau = np.zeros(self.dim)
        mean = np.zeros(self.dim)
        sigma = np.zeros(self.dim)
        means = np.zeros((int(n), self.dim), np.float32) if return_means else None
        N.call("bay_run_sampler", self.handle, int(n), float(a), C.byref(res), _ptr(tau),
               _ptr(mean), _ptr(sigma), _ptr(means) if means is not None else None)
        out = {"acceptance_rate": res.acceptance_rate, "a": res.a}
        if res.acor_status == N.BAY_OK:
            out["autocorrelation"] = Autocorrelation(tau, mean, sigma, int(n), res.lag)
        else:
            out["autocorrelation"] = None
            out["autocorrelation_error"] = N.last_error()
        if means is not None:
            out["means"] = means.T
        return out

    # ---------------------------------------------------------------- sampling
    def sample(self, n=None):
        """sample!: dim x n matrix of positions (numpy (dim, n) view of (n, dim))."""
        n = self.walkers if n is None else int(n)
        out = np.zeros((n, self.dim), np.float32)
        N.call("bay_sample", self.handle, n, _ptr(out))
        return out.T

    def sample_into(self, out):
        """sample! into a CUDA tensor of shape (n, dim) (device-resident output)."""
        N.call("bay_sample", self.handle, out.shape[0], C.c_void_p(out.data_ptr()))
        return out

    def positions(self):
        out = np.zeros((self.walkers, self.dim), np.float32)
        N.call("bay_state_export", self.handle, _ptr(out), None, None)
        return out.T

    def logfn(self):
        out = np.zeros(self.walkers, np.float32)
        N.call("bay_logfn_values", self.handle, _ptr(out))
        return out

    def export_state(self):
        pos = np.zeros((self.walkers, self.dim), np.float32)
        lf = np.zeros(self.walkers, np.float32)
        rng = np.zeros(8, np.uint32)
        N.call("bay_state_export", self.handle, _ptr(pos), _ptr(lf), _ptr(rng))
        return pos, lf, rng

    def import_state(self, pos, lf, rng):
        pos = np.ascontiguousarray(pos, np.float32)
        lf = np.ascontiguousarray(lf, np.float32)
        rng = np.ascontiguousarray(rng, np.uint32)
        N.call("bay_state_import", self.handle, _ptr(pos), _ptr(lf), _ptr(rng))
        return self

    # ---------------------------------------------------------------- estimates
    def mean(self):
        out = np.zeros(self.dim)
        N.call("bay_mean", self.handle, _ptr(out))
        return out

    def variance(self):
        out = np.zeros(self.dim)
        N.call("bay_variance", self.handle, _ptr(out))
        return out

    def sd(self):
        out = np.zeros(self.dim)
        N.call("bay_sd", self.handle, _ptr(out))
        return out

    def histogram(self, cycles=1, bins=0, flags=0):
        bins = bins or self.sfactory.factory.wgs
        limits = np.zeros((self.dim, 2), np.float32)
        pdf = np.zeros((self.dim, bins), np.float32)
        ranks = np.zeros((self.dim, bins), np.float32)
        N.call("bay_histogram", self.handle, int(cycles), int(bins), int(flags), _ptr(limits),
               _ptr(pdf), _ptr(ranks))
        return Histogram(limits.T, pdf.T, ranks.T)
