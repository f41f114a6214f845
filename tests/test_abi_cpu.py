"""CPU-only checks of the C ABI library: it loads, exports every symbol the header
declares, and NVRTC compiles every model form (no device needed)."""
import ctypes as C
import os
import re

import pytest

from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "bayadera_gb300.h")


@pytest.fixture(scope="module")
def native():
    from bayadera_gb300 import build, _native
    build.build()
    _native.lib()
    return _native


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bay_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = header_functions()
    for n in ("bay_ctx_create", "bay_model_compile", "bay_sampler_create", "bay_burn_in",
              "bay_run_sampler", "bay_histogram", "bay_acor", "bay_mean", "bay_variance"):
        assert n in names


def test_library_exports_every_header_symbol(native):
    lib = C.CDLL(native.LIB_PATH)
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert missing == []


def test_binding_covers_header(native):
    assert sorted(native.exported_symbols()) == header_functions()


def test_last_error_empty_at_start(native):
    assert isinstance(native.last_error(), str)


def test_ctx_create_without_gpu_fails_cleanly(native):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    opts = native.CtxOpts(0, 1024, None, 0)
    h = C.c_void_p()
    rc = native.lib().bay_ctx_create(C.byref(opts), C.byref(h))
    assert rc != native.BAY_OK
    assert native.last_error() != ""


def _check(model, form=None, **kw):
    from bayadera_gb300.engine import check_model
    check_model(model, form, **kw)


def test_model_check_builtin_library(native):
    from bayadera_gb300 import models as M
    for name, m in M.distribution_models().items():
        _check(m)
    # posterior of every likelihood with a gaussian prior
    prior = M.distribution_models()["gaussian"]
    for name, lik in M.likelihood_models().items():
        _check(M.device_posterior_model(prior, "post_" + name, lik))
    # the reference's beta-binomial posterior (nvidia_gtx_test.clj:133-159)
    _check(M.device_posterior_model(M.distribution_models()["beta"], "beta_binomial",
                                    M.likelihood_models()["binomial"]))


def test_model_check_benchmark_models(native):
    from bayadera_gb300 import models as M
    _check(M.gaussian_posterior_model(), "plain")
    _check(M.gaussian_posterior_model(), "tiled")
    _check(M.gaussian_posterior_model(), "plain", accept_ref=True)
    _check(M.mvn_precision_model(50))
    _check(M.logistic_model(8))
    _check(M.robust_t_model(8))
    _check(M.hierarchical_model(4))


def test_model_check_reference_compat_flags(native):
    """The reference-compatibility modules compile: the stretch factor's fast-math
    expression (every form), the element-offset partner (plain and tiled forms); the
    element partner is an argument error for the GEMM forms."""
    from bayadera_gb300 import models as M
    uni = M.distribution_models()["uniform"]
    _check(uni, stretch_ref=True)
    _check(uni, partner_element=True)
    _check(uni, stretch_ref=True, partner_element=True, accept_ref=True)
    _check(M.gaussian_posterior_model(), "tiled", partner_element=True, stretch_ref=True)
    _check(M.mvn_precision_model(50), "gemm", tensor=True, stretch_ref=True)
    _check(M.hierarchical_rows_batch_model(16), "batch", stretch_ref=True)
    with pytest.raises(native.IllegalArgument, match="plain and tiled"):
        _check(M.mvn_precision_model(8), "gemm", partner_element=True)


def test_model_check_batch_form(native):
    """The batched engine's kernels (runtime dimension) compile for the hierarchical family;
    a model without a batch form is an argument error."""
    from bayadera_gb300 import models as M
    _check(M.hierarchical_rows_batch_model(128), "batch")
    _check(M.hierarchical_rows_model(7), "plain")
    with pytest.raises(ValueError, match="batch form"):
        _check(M.logistic_model(8), "batch")


def test_model_check_density_engines(native):
    """The plain-form modules carry the density engines' point kernels; a likelihood
    compiles through its 5-argument adapter."""
    from bayadera_gb300 import models as M
    from bayadera_gb300.engine import _LIK_ADAPTER
    lik = M.likelihood_models()["gaussian"]
    name = "%s_bay_points" % lik.loglik
    src = lik.sources + [_LIK_ADAPTER % {"name": name, "loglik": lik.loglik}]
    dm = M.device_distribution_model(src, name=name, logpdf=name, dimension=2, params_size=0)
    _check(dm, "plain")


def test_model_check_tensor_core_form(native):
    """The tcgen05 rows kernels compile for sm_103a across the feature-chunk counts (1 to
    5 chunks of 64, one or two walker sub-tiles per CTA); more than 320 features is an
    argument error, reported before any device work."""
    from bayadera_gb300 import models as M
    for F in (7, 64, 130, 256, 320):
        _check(M.logistic_model(F), "gemm", tensor=True)
    _check(M.robust_t_model(256), "gemm", tensor=True)
    with pytest.raises(native.IllegalArgument, match="320 features"):
        _check(M.logistic_model(321), "gemm", tensor=True)


def test_model_check_reports_nvrtc_log(native):
    from bayadera_gb300 import models as M
    bad = M.device_distribution_model("extern \"C\" { inline REAL broken_logpdf( { } }",
                                      name="broken")
    with pytest.raises(native.CompileError) as e:
        _check(bad)
    assert "error" in str(e.value)


def test_model_check_rejects_bad_names(native):
    from bayadera_gb300 import models as M
    m = M.device_distribution_model(M.get_source("gaussian"), name="g",
                                    logpdf="gaussian_logpdf; int x")
    with pytest.raises(native.IllegalArgument):
        _check(m)


def test_model_check_autotuner_shapes(native):
    """Every shape the autotuner times compiles: the tiled form's (walkers per CTA, CTA
    threads) pairs, the streamed tensor-core form's sub-tiles and stages, the resident
    form's tile groups; shapes outside the kernels' limits are argument errors."""
    from bayadera_gb300 import models as M
    post = M.gaussian_posterior_model()
    for wpc, cta in ((8, 256), (2, 256), (4, 256), (4, 512), (4, 128), (8, 128), (16, 256),
                     (32, 256), (8, 512), (16, 512), (32, 512), (32, 1024)):
        _check(post, "tiled", walkers_per_cta=wpc, cta_threads=cta)
    for bad in ((3, 256), (64, 256), (32, 16)):
        with pytest.raises(native.IllegalArgument):
            _check(post, "tiled", walkers_per_cta=bad[0], cta_threads=bad[1])
    _check(post, "tiled", tile_slices=16)          # row slices: a launch parameter, 1..16
    with pytest.raises(native.IllegalArgument, match="tile_slices"):
        _check(post, "tiled", tile_slices=17)
    lg = M.logistic_model(64)
    for g, st in ((2, 2), (2, 3), (2, 4), (1, 2), (1, 6)):
        _check(lg, "gemm", tensor=True, tc_subtiles=g, tc_stages=st)
    with pytest.raises(native.IllegalArgument, match="do not fit"):
        _check(M.logistic_model(320), "gemm", tensor=True, tc_subtiles=2, tc_stages=6)
    for g in (1, 2):
        _check(M.mvn_precision_model(50), "gemm", tensor=True, tc_groups=g)
    with pytest.raises(native.IllegalArgument, match="tc_groups"):
        _check(M.mvn_precision_model(50), "gemm", tensor=True, tc_groups=3)
