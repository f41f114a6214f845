"""ctypes binding of libbayadera_gb300.so (include/bayadera_gb300.h).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libbayadera_gb300.so")

BAY_OK = 0
BAY_ERR_ARG = 1
BAY_ERR_CUDA = 2
BAY_ERR_COMPILE = 3
BAY_ERR_ALLOC = 4
BAY_ERR_STATE = 5
BAY_ERR_DEVICE = 6

FORM_PLAIN = 0
FORM_TILED = 1
FORM_GEMM = 2
FORM_BATCH = 3
MODEL_ACCEPT_REF = 1
MODEL_GEMM_STREAMING = 2
MODEL_GEMM_TENSOR = 4
MODEL_STRETCH_REF = 8
MODEL_PARTNER_ELEMENT = 16
DIRECT_UNIFORM = 0
DIRECT_GAUSSIAN = 1
DIRECT_EXPONENTIAL = 2
DIRECT_ERLANG = 3
HIST_COMPAT_START1 = 1
HIST_COMPAT_ZERO_LIMITS = 2
HIST_COMPAT_FASTDIV = 4


class BayaderaError(RuntimeError):
    """A failed library call; .code is the bay_status."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class IllegalArgument(BayaderaError, ValueError):
    pass


class CompileError(BayaderaError):
    pass


class CtxOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("wgs", C.c_uint32), ("stream", C.c_void_p),
                ("mem_limit", C.c_uint64)]


class ModelDesc(C.Structure):
    _fields_ = [("source", C.c_char_p), ("logfn", C.c_char_p), ("dim", C.c_uint32),
                ("params_size", C.c_uint32), ("form", C.c_uint32), ("tile_prep", C.c_char_p),
                ("tile_term", C.c_char_p), ("tile_walker", C.c_char_p), ("row_len", C.c_uint32),
                ("prep_len", C.c_uint32), ("walkers_per_cta", C.c_uint32),
                ("cta_threads", C.c_uint32), ("flags", C.c_uint32),
                ("gemm_features", C.c_uint32), ("gemm_coef", C.c_uint32),
                ("gemm_block", C.c_uint32), ("gemm_ld", C.c_uint32),
                ("gemm_offset", C.c_uint64), ("gemm_rows", C.c_uint64),
                ("gemm_aux_col", C.c_uint32), ("gemm_aux_len", C.c_uint32),
                ("tc_subtiles", C.c_uint32), ("tc_stages", C.c_uint32),
                ("tc_groups", C.c_uint32), ("tile_slices", C.c_uint32)]


class SamplerInfo(C.Structure):
    _fields_ = [("walkers", C.c_uint64), ("dim", C.c_uint32), ("wgs", C.c_uint32),
                ("iteration_counter", C.c_uint64), ("data_len", C.c_uint64)]


class BatchMember(C.Structure):
    _fields_ = [("dim", C.c_uint32), ("seed", C.c_uint32), ("walkers", C.c_uint64),
                ("params", C.c_void_p), ("n_params", C.c_uint64), ("rows", C.c_uint64)]


class TuneResult(C.Structure):
    _fields_ = [("walkers_per_cta", C.c_uint32), ("cta_threads", C.c_uint32),
                ("tc_subtiles", C.c_uint32), ("tc_stages", C.c_uint32),
                ("tc_groups", C.c_uint32), ("tile_slices", C.c_uint32),
                ("candidates", C.c_uint32), ("from_cache", C.c_uint32),
                ("us_per_step", C.c_double), ("default_us_per_step", C.c_double)]


class BatchShape(C.Structure):
    _fields_ = [("rows_per_thread", C.c_uint32), ("walkers_per_item", C.c_uint32),
                ("chunk_floats", C.c_uint32), ("walkers_per_thread", C.c_uint32)]


class BatchTuneResult(C.Structure):
    _fields_ = [("shape", BatchShape), ("candidates", C.c_uint32), ("from_cache", C.c_uint32),
                ("us_per_step", C.c_double), ("default_us_per_step", C.c_double)]


class AdaptResult(C.Structure):
    _fields_ = [("a", C.c_double), ("acc_rate", C.c_double), ("probes", C.c_uint32)]


class RunResult(C.Structure):
    _fields_ = [("acceptance_rate", C.c_double), ("a", C.c_float), ("lag", C.c_uint32),
                ("steps", C.c_uint64), ("acor_status", C.c_int)]


# name -> (restype, argtypes); every function returns the int status unless noted.
P = C.c_void_p
_SIGNATURES = {
    "bay_last_error": (C.c_char_p, []),
    "bay_version": (None, [C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "bay_ctx_create": (C.c_int, [C.POINTER(CtxOpts), C.POINTER(P)]),
    "bay_ctx_release": (C.c_int, [P]),
    "bay_ctx_processing_elements": (C.c_int, [P, C.POINTER(C.c_uint64)]),
    "bay_ctx_stream": (C.c_int, [P, C.POINTER(P)]),
    "bay_ctx_synchronize": (C.c_int, [P]),
    "bay_ctx_allocated": (C.c_int, [P, C.POINTER(C.c_uint64)]),
    "bay_launch_count": (C.c_int, [C.POINTER(C.c_uint64)]),
    "bay_model_compile": (C.c_int, [P, C.POINTER(ModelDesc), C.POINTER(P)]),
    "bay_model_release": (C.c_int, [P]),
    "bay_model_check": (C.c_int, [C.POINTER(ModelDesc), C.c_uint32]),
    "bay_sampler_create": (C.c_int, [P, C.c_uint32, C.c_uint64, P, C.c_uint64, C.POINTER(P)]),
    "bay_sampler_create_device": (C.c_int, [P, C.c_uint32, C.c_uint64, P, C.c_uint64,
                                            C.POINTER(P)]),
    "bay_sampler_release": (C.c_int, [P]),
    "bay_sampler_info_get": (C.c_int, [P, C.POINTER(SamplerInfo)]),
    "bay_init": (C.c_int, [P, C.c_uint32]),
    "bay_init_position_limits": (C.c_int, [P, C.c_uint32, P]),
    "bay_init_position_copy": (C.c_int, [P, P]),
    "bay_init_position_host": (C.c_int, [P, P]),
    "bay_init_position_normal": (C.c_int, [P, C.c_uint32, C.c_float, C.c_float]),
    "bay_burn_in": (C.c_int, [P, C.c_uint64, C.c_float]),
    "bay_anneal": (C.c_int, [P, P, C.c_uint64, C.c_float]),
    "bay_acc_rate": (C.c_int, [P, C.c_float, C.POINTER(C.c_double)]),
    "bay_adapt_a": (C.c_int, [P, C.c_uint32, C.c_double, C.c_double, C.c_double,
                              C.POINTER(AdaptResult)]),
    "bay_run_sampler": (C.c_int, [P, C.c_uint64, C.c_float, C.POINTER(RunResult), P, P, P, P]),
    "bay_sample": (C.c_int, [P, C.c_uint64, P]),
    "bay_mean": (C.c_int, [P, P]),
    "bay_variance": (C.c_int, [P, P]),
    "bay_sd": (C.c_int, [P, P]),
    "bay_histogram": (C.c_int, [P, C.c_uint32, C.c_uint32, C.c_uint32, P, P, P]),
    "bay_acor": (C.c_int, [P, P, C.c_uint32, C.c_uint64, P, P, P, C.POINTER(C.c_uint32)]),
    "bay_acor_noalloc": (C.c_int, [P, P, C.c_uint32, C.c_uint64, P, P, P,
                                   C.POINTER(C.c_uint32)]),
    "bay_state_export": (C.c_int, [P, P, P, P]),
    "bay_state_import": (C.c_int, [P, P, P, P]),
    "bay_logfn_values": (C.c_int, [P, P]),
    "bay_sampler_set_graphs": (C.c_int, [P, C.c_int]),
    "bay_sampler_set_persistent": (C.c_int, [P, C.c_int]),
    "bay_sampler_test_barrier_timeout": (C.c_int, [P, C.c_int]),
    "bay_sample_direct": (C.c_int, [P, C.c_uint32, P, C.c_uint32, C.c_uint64, P]),
    "bay_log_density": (C.c_int, [P, P, C.c_uint64, P, C.c_uint64, P]),
    "bay_density": (C.c_int, [P, P, C.c_uint64, P, C.c_uint64, P]),
    "bay_evidence": (C.c_int, [P, P, C.c_uint64, P, C.c_uint64, C.POINTER(C.c_double)]),
    "bay_data_moments": (C.c_int, [P, P, C.c_uint32, C.c_uint64, P, P]),
    "bay_data_histogram": (C.c_int, [P, P, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, P, P,
                                     P]),
    "bay_batch_create": (C.c_int, [P, C.POINTER(BatchMember), C.c_uint32, C.POINTER(P)]),
    "bay_batch_set_persistent": (C.c_int, [P, C.c_int]),
    "bay_batch_test_barrier_timeout": (C.c_int, [P, C.c_int]),
    "bay_batch_create_shaped": (C.c_int, [P, C.POINTER(BatchMember), C.c_uint32,
                                          C.POINTER(BatchShape), C.POINTER(P)]),
    "bay_autotune": (C.c_int, [P, C.POINTER(ModelDesc), C.c_uint64, P, C.c_uint64, P,
                               C.POINTER(TuneResult)]),
    "bay_batch_autotune": (C.c_int, [P, C.POINTER(BatchMember), C.c_uint32,
                                     C.POINTER(BatchTuneResult)]),
    "bay_batch_release": (C.c_int, [P]),
    "bay_batch_init_position_normal": (C.c_int, [P, P, C.c_float, C.c_float]),
    "bay_batch_init_position_host": (C.c_int, [P, P]),
    "bay_batch_burn_in": (C.c_int, [P, C.c_uint64, C.c_float]),
    "bay_batch_run_sampler": (C.c_int, [P, C.c_uint64, C.c_float, P, P]),
    "bay_batch_state_export": (C.c_int, [P, P, P]),
    "bay_batch_info": (C.c_int, [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                 C.POINTER(C.c_uint64)]),
    "bay_batch_set_graphs": (C.c_int, [P, C.c_int]),
}

_lib = None


def exported_symbols():
    return sorted(_SIGNATURES)


def lib():
    """The loaded library (built in-tree by bayadera_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                "libbayadera_gb300.so is not built (expected at %s); run "
                "`python -m bayadera_gb300.build` -- there is no CPU fallback" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def launch_count():
    v = C.c_uint64()
    call("bay_launch_count", C.byref(v))
    return v.value


def last_error():
    return lib().bay_last_error().decode(errors="replace")


def check(code):
    if code == BAY_OK:
        return
    msg = last_error()
    if code == BAY_ERR_ARG:
        raise IllegalArgument(code, msg)
    if code == BAY_ERR_COMPILE:
        raise CompileError(code, msg)
    raise BayaderaError(code, msg)


def call(name, *args):
    check(getattr(lib(), name)(*args))
