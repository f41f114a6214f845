/*
 * bayadera_gb300.h -- C ABI of libbayadera_gb300.so, the GB300 (sm_103a) engine for
 * Bayadera's affine-invariant ensemble (stretch-move) MCMC path.
 *
 * The entry points replace the CUDA engine behind the reference's protocols
 * (src/clojure/uncomplicate/bayadera/internal/protocols.clj): each declaration
 * names the reference function it stands in for.  Plain pointers and sizes only.
 *
 * Conventions
 *  - Every call returns an int status: BAY_OK (0) or a BAY_ERR_* code; the message of
 *    the last failure on the calling thread is bay_last_error().  No call aborts.
 *  - Host arrays belong to the caller; device buffers and handles belong to the
 *    library and are freed by the matching *_release.
 *  - Walker positions crossing the ABI are dim x walkers column-major (walker k's
 *    coordinates contiguous), the reference's GE matrix layout.  Histogram pdf and
 *    ranks are bins x dim column-major; limits 2 x dim; acor series dim x n.
 *  - Calls on one context are serialised on its stream (like the reference's single
 *    hstream); different contexts may run concurrently.
 */
#ifndef BAYADERA_GB300_H
#define BAYADERA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum bay_status {
    BAY_OK = 0,
    BAY_ERR_ARG = 1,     /* invalid argument (IllegalArgumentException in the reference) */
    BAY_ERR_CUDA = 2,    /* a CUDA runtime/driver call failed */
    BAY_ERR_COMPILE = 3, /* NVRTC rejected the model source; the log is in bay_last_error */
    BAY_ERR_ALLOC = 4,   /* device memory exhausted or over the context's limit */
    BAY_ERR_STATE = 5,   /* call out of order (e.g. no positions yet) */
    BAY_ERR_DEVICE = 6   /* a device-side check failed (status word set by a kernel) */
};

typedef struct bay_ctx bay_ctx;
typedef struct bay_model bay_model;
typedef struct bay_sampler bay_sampler;

/* Message of the last failed call on this thread ("" if none). */
const char* bay_last_error(void);
void bay_version(int* major, int* minor);

/* ------------------------------------------------------------------ context
 * Replaces gtx-bayadera-factory (nvidia_gtx.clj:793-807) and with-default-bayadera
 * (cuda.clj:19-31): a device, one stream, and WGS, the reference's work-group size
 * (default 1024 = max-block-dim-x).  WGS keeps its reference meaning (default
 * histogram bins, acor window blocks, processing elements); the kernels' own CTA
 * shapes are chosen by the library. */
typedef struct bay_ctx_opts {
    int device;          /* CUDA device ordinal */
    uint32_t wgs;        /* 0 = 1024 */
    void* stream;        /* cudaStream_t to run on; NULL = a new non-blocking stream */
    uint64_t mem_limit;  /* bytes of device memory this context may allocate; 0 = no limit */
} bay_ctx_opts;

int bay_ctx_create(const bay_ctx_opts* opts, bay_ctx** out);
int bay_ctx_release(bay_ctx* ctx);
/* processing-elements (nvidia_gtx.clj:790-791): SM count * WGS. */
int bay_ctx_processing_elements(bay_ctx* ctx, uint64_t* out);
int bay_ctx_stream(bay_ctx* ctx, void** stream);
int bay_ctx_synchronize(bay_ctx* ctx);
/* Bytes currently allocated by this context. */
int bay_ctx_allocated(bay_ctx* ctx, uint64_t* out);
/* Kernels this library has enqueued in this process, all contexts (each replayed graph
 * counts its kernel nodes).  No reference counterpart: an instrumentation counter. */
int bay_launch_count(uint64_t* out);

/* ------------------------------------------------------------------ models
 * Replaces gtx-stretch-factory (nvidia_gtx.clj:747-757): NVRTC-compiles the model's C
 * source for sm_103a into the fused stretch kernels (Philox draw, proposal, density,
 * accept, acceptance count).  Same source contract as the reference
 * (models.clj:102-115, cuda/distributions/posterior.cu:5-10): `logfn` names
 *   REAL f(uint32_t data_len, uint32_t params_len, const REAL* params,
 *          uint32_t dim, const REAL* x)
 * with params = data || hyperparameters; REAL is float; the source may include
 * <stdint.h>.  Compiled with -use_fast_math like the reference.
 *
 * BAY_FORM_TILED is the data-tiled form for likelihoods that sum over data rows:
 *   void  prep(const REAL* hyper, uint32_t hyper_len, uint32_t dim, const REAL* x,
 *              REAL* prep);                         per walker, prep_len values
 *   REAL  term(const REAL* row, const REAL* prep);   one row of row_len floats
 *   REAL  walker(uint64_t n_rows, const REAL* hyper, uint32_t hyper_len,
 *                uint32_t dim, const REAL* x);       every term not summed over rows
 * log density = walker(x) + sum over rows of term(row, prep(x)); the sum is spread
 * over a CTA with compensated fp32 partial sums and an FP64 combine; data length is
 * 64-bit.
 *
 * BAY_FORM_GEMM is the linear-predictor form: with A a rows x gemm_features matrix in
 * the params (row r at block + gemm_offset + r * gemm_ld, the block being the data or
 * the hyperparameters) and eta = A x[gemm_coef : gemm_coef + gemm_features],
 *   REAL  term(REAL eta_r, const REAL* aux_r, uint64_t r, const REAL* x,
 *              const REAL* prep);                    aux_r = gemm_aux_len values at
 *                                                     column gemm_aux_col of row r
 * log density = walker(x) + sum_r term(eta_r, aux_r, r, x, prep(x)).  With the matrix
 * resident in shared memory (rows * features up to about 40960 floats) walkers are
 * tiled 64 per CTA in one launch per half-step; larger matrices are streamed (128-walker
 * x 128-row register tiles, per-row-block partial sums; row index 32-bit, element
 * offsets 64-bit; features <= 384).  With BAY_MODEL_GEMM_TENSOR the streamed eta runs
 * on the tensor cores (split bf16, see the flag).  Covers Gaussian targets (A =
 * precision matrix, term = -eta_r x_r/2) and regression likelihoods (A = design matrix,
 * aux = response). */
/* BAY_FORM_BATCH compiles a model family for bay_batch (many independent models advanced
 * together), row form with the dimension known only at run time:
 *   void  prep(const REAL* hyper, uint32_t hyper_len, uint32_t dim, const REAL* x,
 *              REAL* prep);                         per walker, prep_len values
 *   REAL  term(const REAL* row, const REAL* x, const REAL* prep);  one row of row_len floats
 *   REAL  walker(uint64_t n_rows, const REAL* hyper, uint32_t hyper_len, uint32_t dim,
 *                const REAL* x);                     every term not summed over rows
 * dim in the description is the largest member dimension. */
enum bay_form { BAY_FORM_PLAIN = 0, BAY_FORM_TILED = 1, BAY_FORM_GEMM = 2, BAY_FORM_BATCH = 3 };
enum bay_model_flags {
    /* accept if u <= z^(D-1) exp(beta dlogfn) in fp32, the reference's formula
     * (nvidia-gtx-mcmc-stretch.cu:84-88); default compares logs in FP64. */
    BAY_MODEL_ACCEPT_REF = 1u << 0,
    /* BAY_FORM_GEMM: always stream the matrix from device memory (three launches per
     * half-step), even when it would fit in shared memory; matrices that do not fit are
     * streamed regardless. */
    BAY_MODEL_GEMM_STREAMING = 1u << 1,
    /* BAY_FORM_GEMM, streamed, with eta = A b on the tensor cores (tcgen05, bf16 inputs,
     * fp32 accumulation): A and b are each split into bf16 hi + lo and the three products
     * hi.hi + hi.lo + lo.hi are accumulated, which leaves a relative error of about 2^-16
     * per product term (fp32 SIMT: 2^-24).  The sampler keeps a bf16 hi + lo copy of A
     * (4 bytes per element).  At most 320 features and 2^31 - 256 rows.  No counterpart
     * in the reference (which evaluates every density per walker in fp32). */
    BAY_MODEL_GEMM_TENSOR = 1u << 2,
    /* the stretch factor z (nvidia-gtx-mcmc-stretch.cu:71-72) with its 1/a by the
     * compiler's fast division, the flavour of the reference's -use_fast_math build;
     * default: IEEE 1/a.  Both keep the operation order that the reference's golden
     * trajectories pin, and agree at a = 2. */
    BAY_MODEL_STRETCH_REF = 1u << 3,
    /* plain and tiled forms: the reference's partner offset (uint)(u0 * K * dim)
     * (nvidia-gtx-mcmc-stretch.cu:75-81, quirk Q1), an element offset that straddles
     * walkers for dim > 1.  Elements past the half's end, which the reference reads out
     * of bounds (or racing with the moving half), read as 0.  Default: partner walker
     * (uint)(u0 * K), clamped to the half (identical at dim = 1). */
    BAY_MODEL_PARTNER_ELEMENT = 1u << 4
};

typedef struct bay_model_desc {
    const char* source;       /* NUL-terminated C source */
    const char* logfn;        /* BAY_FORM_PLAIN: density function name */
    uint32_t dim;             /* walker dimension (protocols.clj:39-44 dimension) */
    uint32_t params_size;     /* hyperparameter count (params-size) */
    uint32_t form;            /* bay_form */
    const char* tile_prep;    /* BAY_FORM_TILED function names */
    const char* tile_term;
    const char* tile_walker;
    uint32_t row_len;         /* BAY_FORM_TILED: floats per data row */
    uint32_t prep_len;        /* BAY_FORM_TILED: per-walker precomputed values (>= 1) */
    uint32_t walkers_per_cta; /* BAY_FORM_TILED: 0 = library choice */
    uint32_t cta_threads;     /* 0 = library choice (multiple of 32, <= 1024) */
    uint32_t flags;           /* bay_model_flags */
    /* BAY_FORM_GEMM (tile_prep / tile_term / tile_walker name the three functions) */
    uint32_t gemm_features;   /* columns of A */
    uint32_t gemm_coef;       /* first walker coordinate multiplied by A */
    uint32_t gemm_block;      /* 0: A in the data, 1: A in the hyperparameters */
    uint32_t gemm_ld;         /* floats between rows of A */
    uint64_t gemm_offset;     /* floats from the block start to row 0 */
    uint64_t gemm_rows;       /* rows of A; 0 = (block length - offset) / ld */
    uint32_t gemm_aux_col;    /* column of the row's auxiliary values */
    uint32_t gemm_aux_len;    /* auxiliary values per row (0..8) */
    /* BAY_MODEL_GEMM_TENSOR, streamed: 128-walker sub-tiles per CTA (1 or 2) and shared-
     * memory ring stages (2..6); 0 = library choice (bay_autotune picks them). */
    uint32_t tc_subtiles;
    uint32_t tc_stages;
    /* BAY_MODEL_GEMM_TENSOR with the matrix resident: 64-walker tile groups per CTA of the
     * move kernels (1 or 2: one matrix copy and one tensor-memory allocation per group or
     * per pair); 0 = library choice (bay_autotune picks it). */
    uint32_t tc_groups;
    /* BAY_FORM_TILED: row slices per walker group (1..16): each slice's CTA sums its rows,
     * the group's last CTA combines the slices in order and decides.  More CTAs when the
     * walkers are few; the sums' order depends on it.  0 = library choice (1; bay_autotune
     * picks it). */
    uint32_t tile_slices;
} bay_model_desc;

int bay_model_compile(bay_ctx* ctx, const bay_model_desc* desc, bay_model** out);
int bay_model_release(bay_model* model);
/* Compile-check a model without a device (NVRTC only); the reference surfaces the same
 * errors from clojurecuda compile! (nvidia_gtx.clj:748-754).  wgs 0 = 1024. */
int bay_model_check(const bay_model_desc* desc, uint32_t wgs);

/* ------------------------------------------------------------------ samplers
 * Replaces GTXStretchFactory.create-sampler (nvidia_gtx.clj:548-610) followed by
 * init! (:391-400).  params = data || hyperparameters (n_params floats, the data being
 * n_params - params_size floats, impl.clj:150-163).  Walkers must be even and >= 4;
 * the reference's "multiple of 2*WGS" restriction (:552, :609-610) is lifted. */
int bay_sampler_create(bay_model* model, uint32_t seed, uint64_t walkers, const float* params,
                       uint64_t n_params, bay_sampler** out);
/* Same, with params already resident on the device (not copied; must outlive the
 * sampler).  d_params must be 16-byte aligned. */
int bay_sampler_create_device(bay_model* model, uint32_t seed, uint64_t walkers,
                              const float* d_params, uint64_t n_params, bay_sampler** out);
int bay_sampler_release(bay_sampler* s);

typedef struct bay_sampler_info {
    uint64_t walkers;
    uint32_t dim;
    uint32_t wgs;
    uint64_t iteration_counter; /* Info (nvidia_gtx.clj:332-335) */
    uint64_t data_len;
} bay_sampler_info;
int bay_sampler_info_get(bay_sampler* s, bay_sampler_info* out);

/* MCMC/init! (nvidia_gtx.clj:391-400): bare-move seeds (seed, seed+1), a = 2, beta = 1,
 * move counter 0. */
int bay_init(bay_sampler* s, uint32_t seed);
/* MCMC/init-position! with limits (nvidia_gtx.clj:409-418): uniform in [lo, hi] per dim
 * (limits 2 x dim: lo_0, hi_0, lo_1, hi_1, ...), then the log density of every walker. */
int bay_init_position_limits(bay_sampler* s, uint32_t seed, const float* limits);
/* init-position! from another sampler's walkers (nvidia_gtx.clj:401-408). */
int bay_init_position_copy(bay_sampler* s, const bay_sampler* src);
/* Positions from the host (dim x walkers column-major). */
int bay_init_position_host(bay_sampler* s, const float* positions);
/* Extension: N(mean, sd^2) i.i.d. in every coordinate. */
int bay_init_position_normal(bay_sampler* s, uint32_t seed, float mean, float sd);

/* MCMC/burn-in! (nvidia_gtx.clj:419-429): n bare steps at stretch a, beta = 1. */
int bay_burn_in(bay_sampler* s, uint64_t steps, float a);
/* MCMC/anneal! (nvidia_gtx.clj:430-440): step i runs at beta = 1/temperatures[i]. */
int bay_anneal(bay_sampler* s, const float* temperatures, uint64_t steps, float a);
/* MCMC/acc-rate! (nvidia_gtx.clj:466-478): one accu step; accepted / walkers. */
int bay_acc_rate(bay_sampler* s, float a, double* rate);

/* The a-adaptation loop of mix! (mcmc.clj:84-91) on the device.  Starting from a, each
 * probe is acc-rate! (init-move! and one accu step, as bay_acc_rate); after probe i the
 * loop stops if step < i, else moves a toward the acceptance window -- below min_acc
 * a = 1 + (a - 1) r / t, above max_acc a = a r / t, t = (min_acc + max_acc) / 2, in FP64 --
 * and stops once r lies inside it.  The whole loop is one CUDA graph whose conditional
 * WHILE node runs the probes, the rule deciding on the device: no host readback per probe.
 * Results: the final a, the last probe's acceptance rate and the number of probes (at most
 * step + 2); the sampler is left as the same sequence of bay_acc_rate calls leaves it.
 * No reference counterpart as an engine call (the reference runs this loop on the host). */
typedef struct bay_adapt_result {
    double a;
    double acc_rate;
    uint32_t probes;
} bay_adapt_result;
int bay_adapt_a(bay_sampler* s, uint32_t step, double a, double min_acc, double max_acc,
                bay_adapt_result* out);

/* MCMC/run-sampler! (nvidia_gtx.clj:441-465): n accu steps with fresh accu seeds
 * (+2 per call), then acor of the per-step ensemble means.  Results:
 * acceptance rate, and per dim tau, mean, sigma (each dim doubles); lag.  means_out
 * (nullable) receives the dim x steps column-major per-step means. */
typedef struct bay_run_result {
    double acceptance_rate;
    float a;
    uint32_t lag;
    uint64_t steps;
    int acor_status;           /* BAY_OK, or BAY_ERR_ARG if steps < 5 * lag */
} bay_run_result;
int bay_run_sampler(bay_sampler* s, uint64_t steps, float a, bay_run_result* result,
                    double* tau, double* mean, double* sigma, float* means_out);

/* RandomSampler/sample! (nvidia_gtx.clj:371-389): bare steps at beta = 1, after each
 * the walkers' positions fill the next columns of out (dim x n_cols), the last copy
 * truncated.  out may be host or device memory. */
int bay_sample(bay_sampler* s, uint64_t n_cols, float* out);

/* Location/mean and Spread/variance, sd (nvidia_gtx.clj:513-541): per-dim statistics of
 * the current walkers, accumulated in FP64 (population variance, divisor W). */
int bay_mean(bay_sampler* s, double* out);
int bay_variance(bay_sampler* s, double* out);
int bay_sd(bay_sampler* s, double* out);

/* EstimateEngine/histogram! (nvidia_gtx.clj:480-512): limits = per-dim [min, max] of
 * the current walkers; integer counts over `cycles` snapshots (a bare step between
 * snapshots); pdf = (bins / (cycles W)) / (hi - lo) * count; ranks = bin indices by
 * decreasing pdf (the reference's bitonic network).  bins: power of two <= 1024,
 * 0 = WGS.  flags: BAY_HIST_COMPAT_START1 (CUDA reference: counts start at 1,
 * nvidia_gtx.clj:500), BAY_HIST_COMPAT_ZERO_LIMITS (reference min/max reduction folds
 * 0.0 into partial blocks, nvidia-gtx-estimate.cu:91-106).  limits 2 x dim, pdf and
 * ranks bins x dim (host or device memory). */
enum bay_hist_flags {
    BAY_HIST_COMPAT_START1 = 1u << 0,
    BAY_HIST_COMPAT_ZERO_LIMITS = 1u << 1,
    /* the bin from the reference's expression (uint)((x - lo) / (hi - lo) * bins)
     * (nvidia-gtx-estimate.cu:22) compiled with -use_fast_math, i.e. the compiler's fast
     * division; default: IEEE division.  The two differ only for values within a few ulp
     * of a bin edge. */
    BAY_HIST_COMPAT_FASTDIV = 1u << 2
};
int bay_histogram(bay_sampler* s, uint32_t cycles, uint32_t bins, uint32_t flags, float* limits,
                  float* pdf, float* ranks);

/* AcorEngine/acor (nvidia_gtx.clj:240-278, nvidia-gtx-acor.cu): integrated
 * autocorrelation time by Sokal/Goodman pairwise blocking of a dim x n column-major
 * series (host or device memory), in FP64.  lag = max(10, min(n/5, WGS, 64));
 * BAY_ERR_ARG if n < 5 lag. */
int bay_acor(bay_ctx* ctx, const float* series, uint32_t dim, uint64_t n, double* tau,
             double* mean, double* sigma, uint32_t* lag);

/* acor that allocates nothing.  No counterpart in the reference: it is for callers
 * that may not allocate device memory when they call -- for instance a host that runs
 * inside a framework whose caching allocator owns the device memory, or a real-time
 * loop with a fixed memory budget.  The caller passes the series in device memory
 * (dim x n column-major) and the outputs (device or host memory); the work space is a
 * fixed 8 MiB scratch array compiled into the library, so dim * n + 3 * dim must not
 * exceed 1,048,576 doubles (BAY_ERR_ARG otherwise).  The array becomes resident on a GPU
 * when the library's module loads there (with CUDA_MODULE_LOADING=LAZY, at first use)
 * and stays until the process exits; bay_ctx_create looks its device address up, so a
 * call itself does no set-up.  A series in device memory of a GPU other than the
 * context's is refused (BAY_ERR_ARG).  All calls share the one array: calls whose
 * kernels overlap on the GPU (other contexts, other streams) race and must be
 * serialised by the caller.  Same results as bay_acor. */
int bay_acor_noalloc(bay_ctx* ctx, const float* d_series, uint32_t dim, uint64_t n,
                     double* tau, double* mean, double* sigma, uint32_t* lag);

/* Checkpoint/resume: positions (dim x walkers), log densities (walkers) and the RNG
 * state (8 words: bare seed, accu seed, bare step, accu step, iteration counter lo/hi,
 * a bits, beta bits).  Counter-based RNG: an imported state resumes bit-exactly. */
int bay_state_export(bay_sampler* s, float* positions, float* logfn, uint32_t* rng_state);
int bay_state_import(bay_sampler* s, const float* positions, const float* logfn,
                     const uint32_t* rng_state);
/* Log densities of the current walkers (walkers floats). */
int bay_logfn_values(bay_sampler* s, float* out);

/* Execution control (no reference counterpart: the reference launches every half-step
 * from the JVM).  CUDA-graph replay of the step loops (default on). */
int bay_sampler_set_graphs(bay_sampler* s, int enabled);
/* Execution control of the resident tensor-core GEMM form (no reference counterpart):
 * one persistent cooperative launch per chunk of steps with a grid barrier between
 * half-steps, or one launch per half-step with programmatic dependent launch (default:
 * faster on GB300).  Both give the same results; other forms ignore it. */
int bay_sampler_set_persistent(bay_sampler* s, int enabled);
/* Testing the device failure path (no reference counterpart): with enabled != 0 the
 * persistent form's grid barriers wait for one more CTA than the launch has, so every CTA
 * gives up after its bounded wait (2 s), raises the abort flag and the status word, and
 * the launch ends; the next status check returns BAY_ERR_DEVICE.  No fault, trap or
 * unbounded wait is involved. */
int bay_sampler_test_barrier_timeout(bay_sampler* s, int enabled);

/* ---------------------------------------------------------------- direct samplers
 * Replace GTXDirectSamplerEngine.sample (nvidia_gtx.clj:48-63) over
 * cuda/rng/{uniform,gaussian,exponential,erlang}-sampler.cu: n samples (n a multiple of
 * 4, the reference's rule) of the distribution with the given parameters and seed, the
 * reference's Philox stream; params and out host or device memory. */
enum bay_direct_kind {
    BAY_DIRECT_UNIFORM = 0,      /* params {lower, upper} */
    BAY_DIRECT_GAUSSIAN = 1,     /* params {mu, sigma} */
    BAY_DIRECT_EXPONENTIAL = 2,  /* params {lambda} */
    BAY_DIRECT_ERLANG = 3        /* params {lambda, k} */
};
int bay_sample_direct(bay_ctx* ctx, uint32_t kind, const float* params, uint32_t seed,
                      uint64_t n, float* out);

/* ---------------------------------------------------------------- density engines
 * Replace GTXDistributionEngine.log-density / density and GTXLikelihoodEngine
 * .log-density / density / evidence (nvidia_gtx.clj:67-141): the model's density (its
 * plain-form logfn; a likelihood is compiled through a 5-argument adapter) at n points,
 * x dim x n column-major; params = data || hyperparameters.  bay_evidence is the mean of
 * exp(logfn) over the points (FP64 sums in a fixed order).  The model must be compiled in
 * the plain form; all arrays host or device memory. */
int bay_log_density(bay_model* model, const float* params, uint64_t n_params, const float* x,
                    uint64_t n, float* out);
int bay_density(bay_model* model, const float* params, uint64_t n_params, const float* x,
                uint64_t n, float* out);
int bay_evidence(bay_model* model, const float* params, uint64_t n_params, const float* x,
                 uint64_t n, double* out);

/* ---------------------------------------------------------------- dataset engine
 * Replace GTXDatasetEngine.data-mean / data-variance / histogram (nvidia_gtx.clj:145-228):
 * per-dimension mean and population variance (FP64; mean or variance may be NULL) and the
 * histogram (limits 2 x dim, pdf and bin ranks bins x dim; counts start at 0 as on the
 * reference's dataset path) of a data matrix x, dim x n column-major, host or device. */
int bay_data_moments(bay_ctx* ctx, const float* x, uint32_t dim, uint64_t n, double* mean,
                     double* variance);
int bay_data_histogram(bay_ctx* ctx, const float* x, uint32_t dim, uint64_t n, uint32_t bins,
                       uint32_t flags, float* limits, float* pdf, float* ranks);

/* ---------------------------------------------------------------- batched models
 * Many independent models of one BAY_FORM_BATCH family -- each with its own dimension,
 * walkers, data and seed -- advanced together: every half-step of every member is three
 * phases over balanced work lists (propose, row terms, accept), as three launches or within
 * one persistent launch per chunk of steps (bay_batch_set_persistent), and the step loops
 * replay as CUDA graphs.  Member m behaves as a sampler created with its seed (same
 * Philox counters and keys, same init!/init-move! seed rules), so the per-member
 * semantics are those of the functions above.  No counterpart in the reference, which
 * runs one model per sampler. */
typedef struct bay_batch bay_batch;
typedef struct bay_batch_member {
    uint32_t dim;             /* walker dimension, <= the model's dim */
    uint32_t seed;            /* the member's seed (as bay_sampler_create) */
    uint64_t walkers;         /* even, >= 4 */
    const float* params;      /* rows (row_len floats each) || hyperparameters, host memory */
    uint64_t n_params;        /* floats in params */
    uint64_t rows;            /* data rows at the start of params */
} bay_batch_member;

int bay_batch_create(bay_model* model, const bay_batch_member* members, uint32_t n,
                     bay_batch** out);
/* The same with the shape of the row-term work lists (0 in a field = library choice):
 * rows_per_thread sets a work item's row chunk (about 256 x rows_per_thread / walkers
 * rows), walkers_per_item caps the walkers of one item (a power of two <= 64; fewer when a
 * member's dimension or walker count asks for it), chunk_floats caps the staged floats of
 * a chunk (64..16384).  Results agree with any shape up to the order of the row sums.
 * bay_batch_autotune picks a shape by timing. */
typedef struct bay_batch_shape {
    uint32_t rows_per_thread;   /* default 128 */
    uint32_t walkers_per_item;  /* default 64 */
    uint32_t chunk_floats;      /* default 4096, at most 16384 */
    uint32_t walkers_per_thread; /* 1, 2 or 4 walkers per thread of the row-term kernel, which
                                    then shares each staged row between them; default 1.  A
                                    member with fewer walkers per item gets padded slots */
} bay_batch_shape;
int bay_batch_create_shaped(bay_model* model, const bay_batch_member* members, uint32_t n,
                            const bay_batch_shape* shape, bay_batch** out);
int bay_batch_release(bay_batch* b);
/* Walkers of member m ~ N(mean, sd^2) i.i.d. with seeds[m] (bay_init_position_normal). */
int bay_batch_init_position_normal(bay_batch* b, const uint32_t* seeds, float mean, float sd);
/* Positions of every member from host memory (member-major, walkers x dim each). */
int bay_batch_init_position_host(bay_batch* b, const float* positions);
int bay_batch_burn_in(bay_batch* b, uint64_t steps, float a);
/* init-move! and `steps` accu steps of every member: acc_rates[m] (n doubles) and, when
 * means is not NULL, the per-step ensemble means of each member (member-major, steps x
 * dim each, the layout bay_acor reads). */
int bay_batch_run_sampler(bay_batch* b, uint64_t steps, float a, double* acc_rates,
                          float* means);
/* Positions (member-major, walkers x dim each) and log densities (member-major), host. */
int bay_batch_state_export(bay_batch* b, float* positions, float* logfn);
/* total walkers, total positions (floats), rows work items of a move half-step */
int bay_batch_info(bay_batch* b, uint64_t* walkers, uint64_t* floats, uint64_t* items);
int bay_batch_set_graphs(bay_batch* b, int enabled);
/* One persistent cooperative launch per chunk of steps for every member (the proposals,
 * row terms and accept phases of each half-step separated by bounded grid barriers), or
 * three launches per half-step (default).  Both give the same results.  No reference
 * counterpart (the reference runs one model per sampler). */
int bay_batch_set_persistent(bay_batch* b, int enabled);
/* Testing the device failure path (no reference counterpart): with enabled != 0 the
 * persistent launch's grid barriers wait for one more CTA than the launch has, so every CTA
 * gives up after its bounded wait (2 s), raises the abort flag and the status word, and the
 * launch ends; the next status check returns BAY_ERR_DEVICE.  No fault, trap or unbounded
 * wait is involved. */
int bay_batch_test_barrier_timeout(bay_batch* b, int enabled);

/* ---------------------------------------------------------------- autotuner
 * Kernel shapes chosen by timing (no reference counterpart: the reference fixes its work-
 * group size at max-block-dim-x, nvidia_gtx.clj:803-807).  bay_autotune times the
 * candidate shapes of a model description on a workload -- walkers, params (host or
 * device) and optional starting positions (dim x walkers; NULL = N(0, I)) -- over bare
 * steps with CUDA events, and returns the fastest: for BAY_FORM_TILED walkers_per_cta,
 * cta_threads and tile_slices, for the BAY_MODEL_GEMM_TENSOR form tc_subtiles and
 * tc_stages (streamed) or tc_groups (matrix resident) -- set them in the bay_model_desc to
 * compile the chosen shape.  Other forms have nothing to tune (the defaults come back,
 * candidates 0).  Results are cached per (model, walkers,
 * params size, device) for the life of the process (from_cache 1).  Shapes change only the
 * order of the log-density sums. */
typedef struct bay_tune_result {
    uint32_t walkers_per_cta;     /* BAY_FORM_TILED */
    uint32_t cta_threads;         /* BAY_FORM_TILED */
    uint32_t tc_subtiles;         /* streamed tensor-core GEMM form */
    uint32_t tc_stages;           /* streamed tensor-core GEMM form */
    uint32_t tc_groups;           /* tensor-core GEMM form, matrix resident */
    uint32_t tile_slices;         /* BAY_FORM_TILED */
    uint32_t candidates;          /* shapes timed */
    uint32_t from_cache;
    double us_per_step;           /* the chosen shape: microseconds per ensemble step */
    double default_us_per_step;   /* the library's default shape */
} bay_tune_result;
int bay_autotune(bay_ctx* ctx, const bay_model_desc* desc, uint64_t walkers, const float* params,
                 uint64_t n_params, const float* positions, bay_tune_result* out);

/* The batched engine's work-list shape (bay_batch_shape) by timing whole-batch bare steps
 * of the members (walkers N(0, I) with the members' seeds); cached per (model, members'
 * sizes, device). */
typedef struct bay_batch_tune_result {
    bay_batch_shape shape;
    uint32_t candidates;
    uint32_t from_cache;
    double us_per_step;
    double default_us_per_step;
} bay_batch_tune_result;
int bay_batch_autotune(bay_model* model, const bay_batch_member* members, uint32_t n,
                       bay_batch_tune_result* out);

#ifdef __cplusplus
}
#endif
#endif
