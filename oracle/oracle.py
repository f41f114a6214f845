"""ctypes wrapper for the CPU oracle (bay_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference arm of bench.py, as the checker.  The product
(bayadera_gb300) never imports this module.

Layouts follow the reference: walker positions are AoS (xs[k*dim + d], i.e. a
dim x walkers column-major matrix), histogram pdf/ranks are bins x dim
column-major, acor series are dim x n column-major.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "bay_oracle.c")
LIB = os.path.join(HERE, "libbay_oracle.so")

CFLAGS = ["-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11"]
# The same source built for speed, for the timed CPU baseline only (never for parity):
# optimised, vectorised, fast-math arithmetic, OpenMP.  Portable flags only (the library
# is built on x86-64 here and on the GPU hosts' Arm cores), so no -march=native.
LIB_FAST = os.path.join(HERE, "libbay_oracle_fast.so")
CFLAGS_FAST = ["-O3", "-ffast-math", "-funroll-loops", "-fopenmp", "-fPIC", "-shared",
               "-std=c11", "-DBO_SPEED", "-fno-finite-math-only"]

PARTNER_ELEMENT = 1
ACCEPT_LOG = 2
HIST_START1 = 1
HIST_ZERO_LIMITS = 2


def _build_one(lib, flags, force):
    if (not force and os.path.exists(lib)
            and os.path.getmtime(lib) >= max(os.path.getmtime(SRC),
                                             os.path.getmtime(os.path.join(HERE, "bay_oracle.h")))):
        return lib
    cmd = ["gcc"] + flags + [SRC, "-o", lib + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(lib + ".tmp", lib)
    return lib


def build(force=False):
    """Compile libbay_oracle.so (the exact build, -ffp-contract=off, for parity) and
    libbay_oracle_fast.so (the speed build, for the timed CPU baseline) next to the
    source with gcc."""
    _build_one(LIB_FAST, CFLAGS_FAST, force)
    return _build_one(LIB, CFLAGS, force)


_lib = None
_speed = False


def use_speed_build(enabled=True):
    """Route this module's calls to the speed build (for timing the CPU baseline; its
    fast-math arithmetic is not the oracle's).  Call before the first use."""
    global _speed, _lib
    if _lib is not None and _speed != enabled:
        raise RuntimeError("the oracle library is already loaded")
    _speed = enabled

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


class StretchArgs(C.Structure):
    _fields_ = [("K", C.c_uint32), ("dim", C.c_uint32), ("seed", C.c_uint32),
                ("stream", C.c_uint32), ("step", C.c_uint32), ("a", C.c_float),
                ("beta", C.c_float), ("data_len", C.c_uint32), ("params_len", C.c_uint32),
                ("params", C.c_void_p), ("model", C.c_char_p), ("S", C.c_void_p),
                ("X", C.c_void_p), ("logfn_X", C.c_void_p), ("flags", C.c_uint32),
                ("accepted", C.c_void_p), ("threads", C.c_int)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_FAST if _speed else LIB)
        L.bo_philox4x32_10.argtypes = [u32p, u32p, u32p]
        L.bo_u01_oo_32_24.argtypes = [C.c_uint32]
        L.bo_u01_oo_32_24.restype = C.c_float
        for nm in ("bo_sample_uniform",):
            getattr(L, nm).argtypes = [C.c_uint32, C.c_float, C.c_float, C.c_uint32, f32p]
        L.bo_sample_gaussian.argtypes = [C.c_uint32, C.c_float, C.c_float, C.c_uint32, f32p]
        L.bo_sample_exponential.argtypes = [C.c_uint32, C.c_float, C.c_uint32, f32p]
        L.bo_sample_erlang.argtypes = [C.c_uint32, C.c_float, C.c_float, C.c_uint32, f32p]
        L.bo_init_walkers.argtypes = [C.c_uint32, C.c_uint64, C.c_uint32, f32p, f32p]
        L.bo_init_walkers_normal.argtypes = [C.c_uint32, C.c_uint64, C.c_uint32, C.c_float,
                                             C.c_float, f32p]
        L.bo_model_exists.argtypes = [C.c_char_p]
        L.bo_logfn32.argtypes = [C.c_char_p, C.c_uint32, C.c_uint32, f32p, C.c_uint32, f32p]
        L.bo_logfn32.restype = C.c_float
        L.bo_logfn64.argtypes = [C.c_char_p, C.c_uint32, C.c_uint32, f32p, C.c_uint32, f64p]
        L.bo_logfn64.restype = C.c_double
        L.bo_logfn_all.argtypes = [C.c_char_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                   f32p, f32p, f32p, C.c_int]
        L.bo_stretch_half.argtypes = [C.POINTER(StretchArgs)]
        L.bo_log_det.argtypes = [C.c_float]
        L.bo_log_det.restype = C.c_float
        L.bo_stretch_propose.argtypes = [C.POINTER(StretchArgs), f32p, f32p, f32p]
        L.bo_stretch_accept.argtypes = [C.POINTER(StretchArgs), f32p, f32p, f32p, f32p]
        L.bo_accu_stats.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, f32p, u8p,
                                    u32p, f32p]
        L.bo_tree_sum_f32.argtypes = [f32p, C.c_uint32]
        L.bo_tree_sum_f32.restype = C.c_float
        L.bo_launch_reduce_f32.argtypes = [f32p, C.c_uint64, C.c_uint32]
        L.bo_launch_reduce_f32.restype = C.c_float
        L.bo_sum_means_vertical.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, f32p, f32p]
        L.bo_mean_ref.argtypes = [C.c_uint32, C.c_uint64, C.c_uint32, f32p, f32p]
        L.bo_variance_ref.argtypes = [C.c_uint32, C.c_uint64, C.c_uint32, f32p, f32p]
        L.bo_mean64.argtypes = [C.c_uint32, C.c_uint64, f32p, f64p]
        L.bo_variance64.argtypes = [C.c_uint32, C.c_uint64, f32p, f64p]
        L.bo_limits.argtypes = [C.c_uint32, C.c_uint64, C.c_uint32, f32p, C.c_uint32, f32p]
        L.bo_histogram_counts.argtypes = [C.c_uint32, C.c_uint64, C.c_uint32, f32p, f32p, u32p]
        L.bo_uint_to_real.argtypes = [C.c_uint32, C.c_uint32, C.c_uint64, f32p, u32p, f32p]
        L.bo_bitonic_ranks.argtypes = [C.c_uint32, C.c_uint32, f32p, f32p]
        L.bo_acor_ref.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, f32p, f32p, f32p, f32p,
                                  C.POINTER(C.c_uint32)]
        L.bo_acor_ref.restype = C.c_int
        L.bo_acor64.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, f32p, f64p, f64p, f64p,
                                C.POINTER(C.c_uint32)]
        L.bo_acor64.restype = C.c_int
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


# ------------------------------------------------------------------ RNG
def philox(ctr, key):
    out = np.zeros(4, np.uint32)
    lib().bo_philox4x32_10(np.asarray(ctr, np.uint32), np.asarray(key, np.uint32), out)
    return out


def u01(i):
    return lib().bo_u01_oo_32_24(int(i))


def sample_direct(kind, n, params, seed):
    out = np.zeros(n, np.float32)
    L = lib()
    if kind == "uniform":
        L.bo_sample_uniform(n, params[0], params[1], seed, out)
    elif kind == "gaussian":
        L.bo_sample_gaussian(n, params[0], params[1], seed, out)
    elif kind == "exponential":
        L.bo_sample_exponential(n, params[0], seed, out)
    elif kind == "erlang":
        L.bo_sample_erlang(n, params[0], params[1], seed, out)
    else:
        raise ValueError(kind)
    return out


def log_det(x):
    """The library kernels' fp32 logarithm (bay_log_det), as the oracle restates it."""
    return float(lib().bo_log_det(float(x)))


# ------------------------------------------------------------------ models
def logfn32(model, params, data_len, dim, x):
    p = _f32(params)
    return float(lib().bo_logfn32(model.encode(), data_len, len(p) - data_len, p, dim, _f32(x)))


def logfn64(model, params, data_len, dim, x):
    p = _f32(params)
    return float(lib().bo_logfn64(model.encode(), data_len, len(p) - data_len, p, dim,
                                  np.ascontiguousarray(x, np.float64)))


def logfn_all(model, params, data_len, dim, xs, threads=1):
    p = _f32(params)
    xs = _f32(xs)
    W = xs.size // dim
    res = np.zeros(W, np.float32)
    lib().bo_logfn_all(model.encode(), W, dim, data_len, len(p) - data_len, p, xs, res, threads)
    return res


# ------------------------------------------------------------------ sampler
class Stretch:
    """The reference's GTXStretch state machine (nvidia_gtx.clj:282-541) on the CPU.

    xs is AoS (walkers x dim row-major == dim x walkers column-major); halves
    s0 = walkers [0, K), s1 = [K, W).  logfn is contiguous per walker.
    """

    def __init__(self, model, dim, walkers, params, data_len=0, seed=0, wgs=256, flags=0,
                 threads=1):
        assert walkers % 2 == 0
        self.model, self.dim, self.W = model, dim, walkers
        self.K = walkers // 2
        self.params = _f32(params)
        self.data_len = data_len
        self.wgs, self.flags, self.threads = wgs, flags, threads
        self.xs = np.zeros(walkers * dim, np.float32)
        self.logfn = np.zeros(walkers, np.float32)
        self.init(seed)

    # init! (nvidia_gtx.clj:391-400)
    def init(self, seed):
        self.seed = seed & 0xffffffff
        self.move_seed = seed & 0xffffffff
        self.a = 2.0
        self.beta = 1.0
        self.bare_counter = 0

    def logfn_all(self):
        self.logfn[:] = logfn_all(self.model, self.params, self.data_len, self.dim, self.xs,
                                  self.threads)

    # init-position! with limits (nvidia_gtx.clj:409-418)
    def init_position(self, seed, limits):
        lib().bo_init_walkers(self.dim, self.W, seed & 0xffffffff, _f32(limits), self.xs)
        self.logfn_all()

    def init_position_normal(self, seed, mean=0.0, sd=1.0):
        lib().bo_init_walkers_normal(self.dim, self.W, seed & 0xffffffff, mean, sd, self.xs)
        self.logfn_all()

    def set_position(self, xs):
        self.xs[:] = _f32(xs).ravel()
        self.logfn_all()

    def _args(self, which, seed, stream, step, a, beta, accepted=None):
        D, K = self.dim, self.K
        X = self.xs[which * K * D:(which + 1) * K * D]
        S = self.xs[(1 - which) * K * D:(2 - which) * K * D]
        lf = self.logfn[which * K:(which + 1) * K]
        assert X.base is self.xs or X.ctypes.data >= self.xs.ctypes.data
        return StretchArgs(K, D, seed & 0xffffffff, stream, step & 0xffffffff, a, beta,
                           self.data_len, len(self.params) - self.data_len,
                           self.params.ctypes.data, self.model.encode(), S.ctypes.data,
                           X.ctypes.data, lf.ctypes.data, self.flags,
                           accepted.ctypes.data if accepted is not None else None, self.threads)

    def half(self, which, seed, stream, step, a, beta, accepted=None):
        lib().bo_stretch_half(C.byref(self._args(which, seed, stream, step, a, beta, accepted)))

    def half_with_density(self, which, seed, stream, step, a, beta, density):
        """One half-step whose proposals' log densities come from density(Y) (Y: K x dim
        float32 -> K float32), e.g. the model compiled for the device, instead of the
        oracle's own restatement of the model; Philox draws, partner, proposal and the
        accept test are the oracle's."""
        D, K = self.dim, self.K
        args = self._args(which, seed, stream, step, a, beta)
        Y = np.zeros(K * D, np.float32)
        zs = np.zeros(K, np.float32)
        u2 = np.zeros(K, np.float32)
        lib().bo_stretch_propose(C.byref(args), Y, zs, u2)
        ly = np.ascontiguousarray(density(Y.reshape(K, D)), np.float32).ravel()
        assert ly.size == K
        lib().bo_stretch_accept(C.byref(args), Y, zs, u2, ly)

    def move_bare_with_density(self, density, a=None, beta=None):
        """move-bare! with the proposals' log densities from density (half_with_density)."""
        a = self.a if a is None else a
        beta = self.beta if beta is None else beta
        self.half_with_density(0, self.seed, 3333, self.bare_counter, a, beta, density)
        self.half_with_density(1, self.seed + 1, 4444, self.bare_counter, a, beta, density)
        self.bare_counter += 1

    # move-bare! (nvidia_gtx.clj:358-364): odd half (s0) then even half (s1)
    def move_bare(self, a=None, beta=None):
        a = self.a if a is None else a
        beta = self.beta if beta is None else beta
        self.half(0, self.seed, 3333, self.bare_counter, a, beta)
        self.half(1, self.seed + 1, 4444, self.bare_counter, a, beta)
        self.bare_counter += 1

    def burn_in(self, n, a):
        self.a = a
        self.beta = 1.0
        for _ in range(n):
            self.move_bare()

    def sample(self):
        """sample! with n = walkers: one move-bare! then the positions."""
        self.beta = 1.0
        self.move_bare()
        return self.xs.reshape(self.W, self.dim).copy()

    # move! (stretch_move_accu, nvidia_gtx.clj:351-357) with its statistics
    def move_accu(self, seed, step, a, accept_blocks, means_blocks):
        D, K, wgs = self.dim, self.K, self.wgs
        for which, stream in ((0, 1111), (1, 2222)):
            acc = np.zeros(K, np.uint8)
            self.half(which, seed + which, stream, step, a, 1.0, accepted=acc)
            X = self.xs[which * K * D:(which + 1) * K * D]
            lib().bo_accu_stats(K, D, wgs, step, X, acc, accept_blocks, means_blocks)

    def run_sampler(self, n, a, accept_start=0):
        """run-sampler! (nvidia_gtx.clj:441-465) with the accept counters starting at
        accept_start (0 here and on OpenCL; the CUDA build memsets them to 1)."""
        D, K, wgs = self.dim, self.K, self.wgs
        G = (K + wgs - 1) // wgs
        self.move_seed = (self.move_seed + 2) & 0xffffffff
        accept_blocks = np.full(G, accept_start, np.uint32)
        means_blocks = np.zeros(G * D * n, np.float32)
        for step in range(n):
            self.move_accu(self.move_seed, step, a, accept_blocks, means_blocks)
        acc = np.zeros(D * n, np.float32)
        # launch-reduce! with blocks (WGS/local_m, local_m), local_m = min(G, WGS)
        lib().bo_sum_means_vertical(D * n, G, min(G, wgs), means_blocks, acc)
        means = acc.reshape(n, D).T * np.float32(0.5 / (wgs * G))
        rate = float(accept_blocks.astype(np.uint64).sum()) / (self.W * n)
        return rate, np.ascontiguousarray(means.astype(np.float32))


# ------------------------------------------------------------------ estimates
def mean_ref(xs, dim, wgs):
    xs = _f32(xs)
    out = np.zeros(dim, np.float32)
    lib().bo_mean_ref(dim, xs.size // dim, wgs, xs, out)
    return out


def variance_ref(xs, dim, wgs):
    xs = _f32(xs)
    out = np.zeros(dim, np.float32)
    lib().bo_variance_ref(dim, xs.size // dim, wgs, xs, out)
    return out


def mean64(xs, dim):
    xs = _f32(xs)
    out = np.zeros(dim, np.float64)
    lib().bo_mean64(dim, xs.size // dim, xs, out)
    return out


def variance64(xs, dim):
    xs = _f32(xs)
    out = np.zeros(dim, np.float64)
    lib().bo_variance64(dim, xs.size // dim, xs, out)
    return out


def histogram(xs_list, dim, bins, wgs=256, flags=0):
    """histogram! over one or more position snapshots (AoS each): limits from the
    first snapshot, counts accumulated over all.  Returns (limits 2 x dim,
    pdf bins x dim, ranks bins x dim), column-major arrays as (dim, 2)/(dim, bins)."""
    L = lib()
    first = _f32(xs_list[0])
    W = first.size // dim
    limits = np.zeros(2 * dim, np.float32)
    L.bo_limits(dim, W, wgs, first, flags, limits)
    counts = np.full(bins * dim, 1 if flags & HIST_START1 else 0, np.uint32)
    for xs in xs_list:
        L.bo_histogram_counts(dim, W, bins, limits, _f32(xs), counts)
    pdf = np.zeros(bins * dim, np.float32)
    L.bo_uint_to_real(dim, bins, W * len(xs_list), limits, counts, pdf)
    ranks = np.zeros(bins * dim, np.float32)
    L.bo_bitonic_ranks(dim, bins, pdf, ranks)
    return limits, pdf, ranks, counts


def acor_ref(series, wgs=256):
    """series: (dim, n) array; returns (tau, mean, sigma, lag) as float32 arrays."""
    s = np.asarray(series, np.float32)
    D, n = s.shape
    flat = _f32(s.T.ravel())
    tau = np.zeros(D, np.float32)
    mean = np.zeros(D, np.float32)
    sigma = np.zeros(D, np.float32)
    lag = C.c_uint32(0)
    rc = lib().bo_acor_ref(D, n, wgs, flat, tau, mean, sigma, C.byref(lag))
    if rc != 0:
        raise ValueError("number of steps (%d) must not be less than %d" % (n, 5 * lag.value))
    return tau, mean, sigma, lag.value


def acor64(series, wgs=256):
    s = np.asarray(series, np.float32)
    D, n = s.shape
    flat = _f32(s.T.ravel())
    tau = np.zeros(D, np.float64)
    mean = np.zeros(D, np.float64)
    sigma = np.zeros(D, np.float64)
    lag = C.c_uint32(0)
    rc = lib().bo_acor64(D, n, wgs, flat, tau, mean, sigma, C.byref(lag))
    if rc != 0:
        raise ValueError("number of steps (%d) must not be less than %d" % (n, 5 * lag.value))
    return tau, mean, sigma, lag.value
