/*
 * bay_oracle.h -- CPU oracle for the ensemble stretch-move MCMC path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * __graft_entry__.smoke() and the cpu_baseline / reference arm of bench.py
 * call it.  The product (bayadera_gb300, libbayadera_gb300.so) never links,
 * loads or calls it.
 *
 * It restates, in plain C, the reference's algorithm for the path:
 *   - Philox4x32-10 (Random123 philox.h, not vendored in the reference; the
 *     published method of Salmon, Moraes, Dror & Shaw, SC'11) and
 *     u01fpt_oo_32_24 (src/device/.../cuda/rng/uniform-sampler.cu:11-13);
 *   - the direct samplers (cuda/rng/{uniform,gaussian,exponential,erlang}-sampler.cu);
 *   - init_walkers, stretch_move, stretch_move_accu, stretch_move_bare, logfn
 *     (cuda/engines/nvidia-gtx-mcmc-stretch.cu:35-206);
 *   - the block tree reductions (nvidia-gtx-mcmc-stretch.cu:8-33, 210-248;
 *     nvidia-gtx-estimate.cu:48-87) and launch-reduce! from clojurecuda 0.7.2;
 *   - mean/variance/histogram/bitonic ranks (nvidia-gtx-estimate.cu:5-187 and
 *     internal/device/nvidia_gtx.clj:480-537);
 *   - acor (cuda/engines/nvidia-gtx-acor.cu:5-168, nvidia_gtx.clj:240-278).
 * Each function below names the file:line it follows.
 *
 * Parity pins: the reference's golden vectors in
 * test/clojure/uncomplicate/bayadera/internal/nvidia_gtx_test.clj, extracted to
 * tests/golden/ by tests/golden/make_golden.py.
 *
 * Build: gcc -O2 -fopenmp -ffp-contract=off (no -ffast-math, no -march):
 * every fused multiply-add the reference's GPU build performs is written out
 * with fmaf(), so x86-64 and aarch64 give the same bits.
 */
#ifndef BAY_ORACLE_H
#define BAY_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- Philox4x32-10 and uniforms ---------------- */
void bo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float bo_u01_oo_32_24(uint32_t i);

/* ---------------- direct samplers (cuda/rng/<kind>-sampler.cu) ---------------- */
void bo_sample_uniform(uint32_t n, float lower, float upper, uint32_t seed, float* out);
void bo_sample_gaussian(uint32_t n, float mu, float sigma, uint32_t seed, float* out);
void bo_sample_exponential(uint32_t n, float lambda, uint32_t seed, float* out);
void bo_sample_erlang(uint32_t n, float lambda, float k, uint32_t seed, float* out);

/* ---------------- walker init (nvidia-gtx-mcmc-stretch.cu:158-195) ------- */
/* xs: AoS, xs[k*dim + d]; limits: 2*dim floats (lo, hi) per dim. dim*walkers % 4 == 0. */
void bo_init_walkers(uint32_t dim, uint64_t walkers, uint32_t seed, const float* limits,
                     float* xs);
/* Gaussian N(mean, sd^2) walker init (an extension; Box-Muller on Philox with
 * key {seed, 0x9a55a9e5}); same AoS layout. */
void bo_init_walkers_normal(uint32_t dim, uint64_t walkers, uint32_t seed, float mean, float sd,
                            float* xs);

/* ---------------- models ---------------- */
/* Returns 0 if the named model exists.  Names: see bay_oracle.c bo_models[]. */
int bo_model_exists(const char* name);
/* FP32 (reference formula, serial sum) and FP64 log-density of one walker. */
float bo_logfn32(const char* name, uint32_t data_len, uint32_t params_len, const float* params,
                 uint32_t dim, const float* x);
double bo_logfn64(const char* name, uint32_t data_len, uint32_t params_len, const float* params,
                  uint32_t dim, const double* x);
/* logfn over many walkers (nvidia-gtx-mcmc-stretch.cu:197-206), AoS x. */
void bo_logfn_all(const char* name, uint64_t walkers, uint32_t dim, uint32_t data_len,
                  uint32_t params_len, const float* params, const float* xs, float* res,
                  int threads);

/* ---------------- stretch move ---------------- */
enum {
    BO_PARTNER_ELEMENT = 1u << 0, /* reference Q1: j0 = (uint)(u*K*DIM) element offset */
    BO_ACCEPT_LOG      = 1u << 1, /* accept if log u <= (D-1) log z + beta dlogfn: the
                                     library's fp32 test with its logarithm (bo_log_det) */
};

typedef struct {
    uint32_t K;           /* walkers in each half */
    uint32_t dim;
    uint32_t seed;        /* Philox key[0] */
    uint32_t stream;      /* counter word 2 (odd_or_even): 1111/2222/3333/4444 */
    uint32_t step;        /* counter word 1 */
    float a;
    float beta;
    uint32_t data_len;
    uint32_t params_len;
    const float* params;
    const char* model;
    const float* S;       /* complementary half, AoS K*dim */
    float* X;             /* moving half, AoS K*dim */
    float* logfn_X;       /* K */
    uint32_t flags;
    uint8_t* accepted;    /* optional, K */
    int threads;
} bo_stretch_args;

/* The library kernels' fp32 logarithm, restated bit for bit (positive normal x). */
float bo_log_det(float x);
/* One half-step: stretch_move for k in [0, K) (nvidia-gtx-mcmc-stretch.cu:35-99). */
void bo_stretch_half(const bo_stretch_args* a);
/* The same half-step in two parts, for checking a kernel whose model density is evaluated
 * elsewhere: the proposals Y (K x dim), stretch factors z and accept uniforms u2; then the
 * accept test given the proposals' log densities ly (K), updating X, logfn_X, accepted. */
void bo_stretch_propose(const bo_stretch_args* a, float* Y, float* zs, float* u2s);
void bo_stretch_accept(const bo_stretch_args* a, const float* Y, const float* zs,
                       const float* u2s, const float* ly);

/* Statistics that stretch_move_accu adds after the move
 * (nvidia-gtx-mcmc-stretch.cu:101-134): with G = ceil(K/wgs) blocks,
 * accept[b] += #accepted in block b, means[b + G*(step*dim + i)] += tree sum of X[.,i]. */
void bo_accu_stats(uint32_t K, uint32_t dim, uint32_t wgs, uint32_t step, const float* X,
                   const uint8_t* accepted, uint32_t* accept_blocks, float* means_blocks);

/* ---------------- reductions ---------------- */
/* block_reduction_sum pattern (nvidia-gtx-mcmc-stretch.cu:8-33) on one block of L values. */
float bo_tree_sum_f32(const float* v, uint32_t L);
/* launch-reduce! with a 1-D block of wgs over n values: level-by-level tree sums. */
float bo_launch_reduce_f32(const float* v, uint64_t n, uint32_t wgs);
/* sum_means_vertical + reduction (nvidia-gtx-mcmc-stretch.cu:250-260): sums the
 * G per-block partials of m rows into acc[m], tree order with block wgs. */
void bo_sum_means_vertical(uint32_t m, uint32_t G, uint32_t wgs, const float* means_blocks,
                           float* acc);

/* ---------------- moments (nvidia_gtx.clj:513-537) ---------------- */
/* Reference (fp32 tree, then scal 1/W) and FP64 versions over walkers of AoS xs. */
void bo_mean_ref(uint32_t dim, uint64_t walkers, uint32_t wgs, const float* xs, float* mean);
void bo_variance_ref(uint32_t dim, uint64_t walkers, uint32_t wgs, const float* xs, float* var);
void bo_mean64(uint32_t dim, uint64_t walkers, const float* xs, double* mean);
void bo_variance64(uint32_t dim, uint64_t walkers, const float* xs, double* var);

/* ---------------- histogram (nvidia-gtx-estimate.cu:5-147, nvidia_gtx.clj:480-512) ---- */
enum {
    BO_HIST_START1      = 1u << 0, /* reference Q3: sampler-path bins start at 1 */
    BO_HIST_ZERO_LIMITS = 1u << 1, /* reference Q7: partial min/max blocks fold in 0.0 */
};
/* limits[2*dim]: per-dim [min, max] over walkers (+ Q7 when flagged; wgs = reduction block). */
void bo_limits(uint32_t dim, uint64_t walkers, uint32_t wgs, const float* xs, uint32_t flags,
               float* limits);
/* counts[bins*dim] += bin counts of xs (AoS) under limits (bins-major per dim). */
void bo_histogram_counts(uint32_t dim, uint64_t walkers, uint32_t bins, const float* limits,
                         const float* xs, uint32_t* counts);
/* pdf[b + bins*d] = (bins/n)/(hi-lo) * count (uint_to_real). */
void bo_uint_to_real(uint32_t dim, uint32_t bins, uint64_t n, const float* limits,
                     const uint32_t* counts, float* pdf);
/* bitonic_local ranks per dim (bins a power of two). */
void bo_bitonic_ranks(uint32_t dim, uint32_t bins, const float* pdf, float* ranks);

/* ---------------- acor (nvidia-gtx-acor.cu:5-168, nvidia_gtx.clj:240-278) -------- */
/* series: D x n column-major (series[t*D + d]); modified copy is made internally.
 * Returns 0, or -1 if n < 5*lag (the reference's IllegalArgumentException). */
int bo_acor_ref(uint32_t D, uint32_t n, uint32_t wgs, const float* series, float* tau,
                float* mean, float* sigma, uint32_t* lag_out);
/* Same recursion in FP64 arithmetic (mean, C0 and D sums, tau and sigma). */
int bo_acor64(uint32_t D, uint32_t n, uint32_t wgs, const float* series, double* tau,
              double* mean, double* sigma, uint32_t* lag_out);

#ifdef __cplusplus
}
#endif
#endif
