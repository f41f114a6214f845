/*
 * bay_oracle.c -- CPU oracle for the ensemble stretch-move MCMC path.
 *
 * TEST INFRASTRUCTURE ONLY (see bay_oracle.h): used by tests/, by
 * __graft_entry__.smoke() and by bench.py's cpu_baseline / reference arm as
 * the checker and the timed CPU restatement.  Never part of the product.
 *
 * Every fused multiply-add that the reference's NVRTC build contracts is
 * written as fmaf(); the file is compiled with -ffp-contract=off so nothing
 * else is fused, on x86-64 and aarch64 alike.  Transcendentals use libm
 * (the reference uses CUDA fast-math intrinsics, so those paths are compared
 * with a stated tolerance, never bit-for-bit).
 */
#include "bay_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ======================= Philox4x32-10 ==================================
 * Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As Easy as 1, 2, 3",
 * SC'11: four 32-bit words, two multipliers, Weyl key schedule, 10 rounds.
 * The reference takes it from Random123 philox.h (bundled in the
 * uncomplicate/neanderthal 0.25.7-SNAPSHOT jar, not in the reference tree). */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void bo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        if (r > 0) {
            k0 += PHILOX_W0;
            k1 += PHILOX_W1;
        }
        const uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        const uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* u01fpt_oo_32_24: cuda/rng/uniform-sampler.cu:11-13 -- (0.5 + (i>>9)) * 2^-23, exact. */
float bo_u01_oo_32_24(uint32_t i) {
    return (0.5f + (float)(i >> 9)) * 1.1920928955078125E-7f;
}

static void philox_u01x4(const uint32_t ctr[4], const uint32_t key[2], float u[4]) {
    uint32_t r[4];
    bo_philox4x32_10(ctr, key, r);
    for (int w = 0; w < 4; w++) u[w] = bo_u01_oo_32_24(r[w]);
}

/* ======================= direct samplers ================================ */
/* cuda/rng/uniform-sampler.cu:15-44: key {seed, 0xdecafaaa},
 * ctr {gid, 0xf00dcafe, 0xdeadbeef, 0xbeeff00d}; x = u*range + lower (fused). */
void bo_sample_uniform(uint32_t n, float lower, float upper, uint32_t seed, float* out) {
    const float range = upper - lower;
    const uint32_t key[2] = {seed, 0xdecafaaau};
    for (uint32_t gid = 0; gid * 4 < n; gid++) {
        const uint32_t ctr[4] = {gid, 0xf00dcafeu, 0xdeadbeefu, 0xbeeff00du};
        float u[4];
        philox_u01x4(ctr, key, u);
        for (int w = 0; w < 4 && gid * 4 + w < n; w++) out[gid * 4 + w] = fmaf(u[w], range, lower);
    }
}

/* cuda/rng/gaussian-sampler.cu:19-61: Box-Muller on the 4 uniforms. */
void bo_sample_gaussian(uint32_t n, float mu, float sigma, uint32_t seed, float* out) {
    const float two_pi = 6.2831855f;
    const uint32_t key[2] = {seed, 0xdecafaaau};
    for (uint32_t gid = 0; gid * 4 < n; gid++) {
        const uint32_t ctr[4] = {gid, 0xf00dcafeu, 0xdeadbeefu, 0xbeeff00du};
        float u[4], r[4];
        philox_u01x4(ctr, key, u);
        const float ry = sqrtf(-2.0f * logf(u[1]));
        const float rw = sqrtf(-2.0f * logf(u[3]));
        r[0] = sinf(two_pi * u[0]) * ry;
        r[1] = cosf(two_pi * u[0]) * ry;
        r[2] = sinf(two_pi * u[2]) * rw;
        r[3] = cosf(two_pi * u[2]) * rw;
        for (int w = 0; w < 4 && gid * 4 + w < n; w++) out[gid * 4 + w] = fmaf(r[w], sigma, mu);
    }
}

/* cuda/rng/exponential-sampler.cu:15-44: x = -1/lambda * log(1 - u). */
void bo_sample_exponential(uint32_t n, float lambda, uint32_t seed, float* out) {
    const uint32_t key[2] = {seed, 0xdecafaaau};
    const float m = -1.0f / lambda;
    for (uint32_t gid = 0; gid * 4 < n; gid++) {
        const uint32_t ctr[4] = {gid, 0xf00dcafeu, 0xdeadbeefu, 0xbeeff00du};
        float u[4];
        philox_u01x4(ctr, key, u);
        for (int w = 0; w < 4 && gid * 4 + w < n; w++) out[gid * 4 + w] = m * logf(1.0f - u[w]);
    }
}

/* cuda/rng/erlang-sampler.cu:15-61: sum of k logs of uniforms (counter word 3 = i),
 * divided by -lambda. */
void bo_sample_erlang(uint32_t n, float lambda, float k, uint32_t seed, float* out) {
    const uint32_t key[2] = {seed, 0xdecafaaau};
    const float nl = -lambda;
    for (uint32_t gid = 0; gid * 4 < n; gid++) {
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (uint32_t i = 0; (float)i < k; i++) {
            const uint32_t ctr[4] = {gid, 0xf00dcafeu, 0xdeadbeefu, i};
            float u[4];
            philox_u01x4(ctr, key, u);
            for (int w = 0; w < 4; w++) acc[w] += logf(u[w]);
        }
        for (int w = 0; w < 4 && gid * 4 + w < n; w++) out[gid * 4 + w] = acc[w] / nl;
    }
}

/* ======================= walker init ===================================
 * nvidia-gtx-mcmc-stretch.cu:158-195: thread gid fills xs[4gid .. 4gid+3] from one
 * Philox call, key {seed, 0xdecafaaa}, ctr {gid, 0xf00dcafe, 0xdeadbeef, 0xbeeff00d};
 * x = u*hi + (1-u)*lo with the first product fused. */
void bo_init_walkers(uint32_t dim, uint64_t walkers, uint32_t seed, const float* limits,
                     float* xs) {
    const uint64_t n = (uint64_t)dim * walkers / 4;
    const uint32_t key[2] = {seed, 0xdecafaaau};
    for (uint64_t gid = 0; gid < n; gid++) {
        const uint32_t ctr[4] = {(uint32_t)gid, 0xf00dcafeu, 0xdeadbeefu, 0xbeeff00du};
        float u[4];
        philox_u01x4(ctr, key, u);
        for (int w = 0; w < 4; w++) {
            const uint64_t i = gid * 4 + w;
            const float lo = limits[2 * (i % dim)];
            const float hi = limits[2 * (i % dim) + 1];
            xs[i] = fmaf(u[w], hi, (1.0f - u[w]) * lo);
        }
    }
}

/* N(mean, sd^2) init (extension): element i = k*dim + d uses Philox ctr
 * {i/2, 0x6e6f726d, 0x77616c6b, 0xbeeff00d}, key {seed, 0x9a55a9e5}; words (0,1)
 * give the pair for even i, i+1 via Box-Muller in double, rounded to float. */
void bo_init_walkers_normal(uint32_t dim, uint64_t walkers, uint32_t seed, float mean, float sd,
                            float* xs) {
    const uint64_t n = (uint64_t)dim * walkers;
    const uint32_t key[2] = {seed, 0x9a55a9e5u};
    for (uint64_t p = 0; 2 * p < n; p++) {
        const uint32_t ctr[4] = {(uint32_t)p, 0x6e6f726du, 0x77616c6bu, 0xbeeff00du};
        float u[4];
        philox_u01x4(ctr, key, u);
        const double r = sqrt(-2.0 * log((double)u[1]));
        const double t = 6.283185307179586 * (double)u[0];
        const double z0 = r * cos(t), z1 = r * sin(t);
        xs[2 * p] = (float)((double)mean + (double)sd * z0);
        if (2 * p + 1 < n) xs[2 * p + 1] = (float)((double)mean + (double)sd * z1);
    }
}

/* ======================= models ========================================
 * FP32 forms follow the reference's sources (cuda/distributions/<name>.cu) with
 * serial fp32 sums; FP64 forms are the same densities in double. */
#define LOG_SQRT_2PI_F 0.9189385332046727f
#define LOG_SQRT_2PI 0.91893853320467274178

/* gaussian.cu:9-11 */
static float gauss_unscaled32(float mu, float sigma, float x) {
    return (x - mu) * (x - mu) / (-2.0f * sigma * sigma);
}
/* gaussian.cu:13-15 */
static float gauss_scale32(float sigma) { return -logf(sigma) - LOG_SQRT_2PI_F; }
/* uniform.cu:3-11 */
static float uniform_log32(float lower, float upper, float x) {
    const int in_range = (lower <= x) && (x <= upper);
    return logf(in_range ? (1.0f / (upper - lower)) : 0.0f);
}
static double uniform_log64(double lower, double upper, double x) {
    const int in_range = (lower <= x) && (x <= upper);
    return in_range ? -log(upper - lower) : -INFINITY;
}

/* gaussian.cu:33-46 gaussian_loglik */
static float gaussian_loglik32(uint32_t data_len, const float* data, const float* ms) {
    const float mu = ms[0], sigma = ms[1];
    if (0.0f < sigma) {
        float res = fmaf((float)data_len, gauss_scale32(sigma), gauss_unscaled32(mu, sigma, data[0]));
        for (uint32_t i = 1; i < data_len; i++) res += gauss_unscaled32(mu, sigma, data[i]);
        return res;
    }
    return NAN;
}
static double gaussian_loglik64(uint32_t data_len, const float* data, const double* ms) {
    const double mu = ms[0], sigma = ms[1];
    if (0.0 < sigma) {
        double res = -(double)data_len * (log(sigma) + LOG_SQRT_2PI);
        const double c = -0.5 / (sigma * sigma);
        for (uint32_t i = 0; i < data_len; i++) {
            const double d = (double)data[i] - mu;
            res += d * d * c;
        }
        return res;
    }
    return NAN;
}

/* student-t.cu:9-19 */
static float student_t_unscaled32(float nu, float mu, float sigma, float x) {
    const float r = (x - mu) / sigma;
    return -(0.5f * (nu + 1.0f) * logf(1.0f + r * r / nu));
}

typedef float (*logfn32_t)(uint32_t, uint32_t, const float*, uint32_t, const float*);
typedef double (*logfn64_t)(uint32_t, uint32_t, const float*, uint32_t, const double*);

/* uniform_logpdf (uniform.cu:14-17) */
static float m_uniform32(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const float* x) {
    (void)pl; (void)dim;
    return uniform_log32(p[dl], p[dl + 1], x[0]);
}
static double m_uniform64(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const double* x) {
    (void)pl; (void)dim;
    return uniform_log64(p[dl], p[dl + 1], x[0]);
}
/* gaussian_mcmc_logpdf (gaussian.cu:23-26) */
static float m_gaussian32(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const float* x) {
    (void)pl; (void)dim;
    return gauss_unscaled32(p[dl], p[dl + 1], x[0]);
}
static double m_gaussian64(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const double* x) {
    (void)pl; (void)dim;
    const double d = x[0] - p[dl], s = p[dl + 1];
    return -d * d / (2.0 * s * s);
}
/* student_t_mcmc_logpdf (student-t.cu:25-28) */
static float m_student_t32(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const float* x) {
    (void)pl; (void)dim;
    return student_t_unscaled32(p[dl], p[dl + 1], p[dl + 2], x[0]);
}
static double m_student_t64(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const double* x) {
    (void)pl; (void)dim;
    const double nu = p[dl], r = (x[0] - p[dl + 1]) / p[dl + 2];
    return -0.5 * (nu + 1.0) * log1p(r * r / nu);
}

/* 2-D Gaussian (mu, sigma) posterior: gaussian_loglik (gaussian.cu:33-46) over the
 * data plus the prior  N(mu | h0, h1^2) + Uniform(sigma | h2, h3), composed as in
 * cuda/distributions/posterior.cu:5-10 (loglik(data) + prior(&params[data_len])). */
static float m_gauss_post32(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const float* x) {
    (void)pl; (void)dim;
    const float* h = p + dl;
    const float prior = (gauss_unscaled32(h[0], h[1], x[0]) + gauss_scale32(h[1]))
        + uniform_log32(h[2], h[3], x[1]);
    return gaussian_loglik32(dl, p, x) + prior;
}
static double m_gauss_post64(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const double* x) {
    (void)pl; (void)dim;
    const float* h = p + dl;
    const double d = x[0] - h[0];
    const double prior = -d * d / (2.0 * (double)h[1] * h[1]) - log((double)h[1]) - LOG_SQRT_2PI
        + uniform_log64(h[2], h[3], x[1]);
    return gaussian_loglik64(dl, p, x) + prior;
}

/* Zero-mean Gaussian with precision matrix P (dim x dim row-major in the
 * hyperparameters): -1/2 x'Px. */
static float m_mvn32(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const float* x) {
    (void)pl;
    const float* P = p + dl;
    float acc = 0.0f;
#ifdef BO_SPEED
    /* speed build (the timed CPU baseline, not a checker): plain sums that -ffast-math
     * lets the compiler reassociate and vectorise */
    for (uint32_t i = 0; i < dim; i++) {
        float t = 0.0f;
        for (uint32_t j = 0; j < dim; j++) t += P[i * dim + j] * x[j];
        acc += x[i] * t;
    }
#else
    for (uint32_t i = 0; i < dim; i++) {
        float t = 0.0f;
        for (uint32_t j = 0; j < dim; j++) t = fmaf(P[i * dim + j], x[j], t);
        acc = fmaf(x[i], t, acc);
    }
#endif
    return -0.5f * acc;
}
static double m_mvn64(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const double* x) {
    (void)pl;
    const float* P = p + dl;
    double acc = 0.0;
    for (uint32_t i = 0; i < dim; i++) {
        double t = 0.0;
        for (uint32_t j = 0; j < dim; j++) t += (double)P[i * dim + j] * x[j];
        acc += x[i] * t;
    }
    return -0.5 * acc;
}

/* Bayesian logistic regression.  data: N rows of (x_1..x_F, y), F = dim;
 * hyper: {prior_sd}.  loglik = sum y*eta - softplus(eta); prior N(0, sd^2 I). */
static float softplus32(float e) { return fmaxf(e, 0.0f) + logf(1.0f + expf(-fabsf(e))); }
static float m_logistic32(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const float* x) {
    (void)pl;
    const uint32_t row = dim + 1, N = dl / row;
    float res = 0.0f;
    for (uint32_t n = 0; n < N; n++) {
        const float* r = p + (uint64_t)n * row;
        float eta = 0.0f;
        for (uint32_t f = 0; f < dim; f++) eta = fmaf(r[f], x[f], eta);
        res += fmaf(r[dim], eta, -softplus32(eta));
    }
    const float sd = p[dl];
    float pr = 0.0f;
    for (uint32_t f = 0; f < dim; f++) pr = fmaf(x[f], x[f], pr);
    return res - pr / (2.0f * sd * sd);
}
static double m_logistic64(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const double* x) {
    (void)pl;
    const uint32_t row = dim + 1, N = dl / row;
    double res = 0.0;
    for (uint32_t n = 0; n < N; n++) {
        const float* r = p + (uint64_t)n * row;
        double eta = 0.0;
        for (uint32_t f = 0; f < dim; f++) eta += (double)r[f] * x[f];
        res += (double)r[dim] * eta - (fmax(eta, 0.0) + log1p(exp(-fabs(eta))));
    }
    const double sd = p[dl];
    double pr = 0.0;
    for (uint32_t f = 0; f < dim; f++) pr += x[f] * x[f];
    return res - pr / (2.0 * sd * sd);
}

/* Robust linear regression, Student-t(nu) residuals.  x = (beta_1..beta_F, log sigma),
 * dim = F + 1; data: N rows of (x_1..x_F, y); hyper {nu, beta_sd, logsigma_sd}.
 * loglik = sum -(nu+1)/2 log(1 + r^2/nu) - N log sigma, r = (y - eta)/sigma. */
static float m_robust32(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const float* x) {
    (void)pl;
    const uint32_t F = dim - 1, row = F + 1, N = dl / row;
    const float* h = p + dl;
    const float nu = h[0], ls = x[F], inv_s = expf(-ls);
    float res = 0.0f;
    for (uint32_t n = 0; n < N; n++) {
        const float* r = p + (uint64_t)n * row;
        float eta = 0.0f;
        for (uint32_t f = 0; f < F; f++) eta = fmaf(r[f], x[f], eta);
        const float z = (r[F] - eta) * inv_s;
        res += -0.5f * (nu + 1.0f) * logf(1.0f + z * z / nu);
    }
    float pb = 0.0f;
    for (uint32_t f = 0; f < F; f++) pb = fmaf(x[f], x[f], pb);
    return res - (float)N * ls - pb / (2.0f * h[1] * h[1]) - ls * ls / (2.0f * h[2] * h[2]);
}
static double m_robust64(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const double* x) {
    (void)pl;
    const uint32_t F = dim - 1, row = F + 1, N = dl / row;
    const float* h = p + dl;
    const double nu = h[0], ls = x[F], inv_s = exp(-ls);
    double res = 0.0;
    for (uint32_t n = 0; n < N; n++) {
        const float* r = p + (uint64_t)n * row;
        double eta = 0.0;
        for (uint32_t f = 0; f < F; f++) eta += (double)r[f] * x[f];
        const double z = ((double)r[F] - eta) * inv_s;
        res += -0.5 * (nu + 1.0) * log1p(z * z / nu);
    }
    double pb = 0.0;
    for (uint32_t f = 0; f < F; f++) pb += x[f] * x[f];
    return res - (double)N * ls - pb / (2.0 * (double)h[1] * h[1])
        - ls * ls / (2.0 * (double)h[2] * h[2]);
}

/* Gaussian hierarchical model (eight-schools form).  x = (theta_1..theta_J, mu, log tau),
 * dim = J + 2.  data (float-encoded): [J, sigma_1..sigma_J, off_0..off_J, y_0..y_{N-1}],
 * group j owns y[off_j .. off_{j+1}).  hyper {mu_sd, logtau_sd}.
 * logfn = sum_j sum_i -(y_ij - theta_j)^2/(2 sigma_j^2)
 *       + sum_j [-(theta_j - mu)^2/(2 tau^2) - log tau] - mu^2/(2 mu_sd^2) - (log tau)^2/(2 lt_sd^2). */
static float m_hier32(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const float* x) {
    (void)pl;
    const uint32_t J = (uint32_t)p[0];
    const float* sig = p + 1;
    const float* off = p + 1 + J;
    const float* y = p + 2 + 2 * J;
    const float* h = p + dl;
    const float mu = x[J], lt = x[J + 1], inv_t2 = expf(-2.0f * lt);
    float res = 0.0f;
    for (uint32_t j = 0; j < J; j++) {
        const float c = -0.5f / (sig[j] * sig[j]);
        const uint32_t b = (uint32_t)off[j], e = (uint32_t)off[j + 1];
        float s = 0.0f;
        for (uint32_t i = b; i < e; i++) {
            const float d = y[i] - x[j];
            s = fmaf(d * d, c, s);
        }
        const float dt = x[j] - mu;
        res += s - 0.5f * dt * dt * inv_t2 - lt;
    }
    (void)dim;
    return res - mu * mu / (2.0f * h[0] * h[0]) - lt * lt / (2.0f * h[1] * h[1]);
}
static double m_hier64(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const double* x) {
    (void)pl; (void)dim;
    const uint32_t J = (uint32_t)p[0];
    const float* sig = p + 1;
    const float* off = p + 1 + J;
    const float* y = p + 2 + 2 * J;
    const float* h = p + dl;
    const double mu = x[J], lt = x[J + 1], inv_t2 = exp(-2.0 * lt);
    double res = 0.0;
    for (uint32_t j = 0; j < J; j++) {
        const double c = -0.5 / ((double)sig[j] * sig[j]);
        const uint32_t b = (uint32_t)off[j], e = (uint32_t)off[j + 1];
        for (uint32_t i = b; i < e; i++) {
            const double d = (double)y[i] - x[j];
            res += d * d * c;
        }
        const double dt = x[j] - mu;
        res += -0.5 * dt * dt * inv_t2 - lt;
    }
    return res - mu * mu / (2.0 * (double)h[0] * h[0]) - lt * lt / (2.0 * (double)h[1] * h[1]);
}

/* The same hierarchical model on observation rows (y, g, c = -1/(2 sigma_g^2)), data
 * length 3 N, hyper {mu_sd, logtau_sd}: the batch-form model of the library
 * (csrc/library/hierarchical_rows.h), rows summed in order. */
static float m_hrows32(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const float* x) {
    (void)pl;
    const uint32_t n = dl / 3, J = dim - 2;
    const float* h = p + dl;
    float res = 0.0f;
    for (uint32_t i = 0; i < n; i++) {
        const float* r = p + 3 * (uint64_t)i;
        const float d = r[0] - x[(uint32_t)r[1]];
        res += r[2] * d * d;
    }
    const float mu = x[J], lt = x[J + 1], c = -0.5f * expf(-2.0f * lt);
    float s = 0.0f;
    for (uint32_t j = 0; j < J; j++) {
        const float d = x[j] - mu;
        s = fmaf(d * d, c, s);
    }
    return res + (s - (float)J * lt - mu * mu / (2.0f * h[0] * h[0]) - lt * lt / (2.0f * h[1] * h[1]));
}
static double m_hrows64(uint32_t dl, uint32_t pl, const float* p, uint32_t dim, const double* x) {
    (void)pl;
    const uint32_t n = dl / 3, J = dim - 2;
    const float* h = p + dl;
    double res = 0.0;
    for (uint32_t i = 0; i < n; i++) {
        const float* r = p + 3 * (uint64_t)i;
        const double d = (double)r[0] - x[(uint32_t)r[1]];
        res += (double)r[2] * d * d;
    }
    const double mu = x[J], lt = x[J + 1], c = -0.5 * exp(-2.0 * lt);
    for (uint32_t j = 0; j < J; j++) {
        const double d = x[j] - mu;
        res += d * d * c;
    }
    return res - (double)J * lt - mu * mu / (2.0 * (double)h[0] * h[0])
        - lt * lt / (2.0 * (double)h[1] * h[1]);
}

typedef struct {
    const char* name;
    logfn32_t f32;
    logfn64_t f64;
} bo_model;

static const bo_model bo_models[] = {
    {"uniform", m_uniform32, m_uniform64},
    {"gaussian", m_gaussian32, m_gaussian64},
    {"student_t", m_student_t32, m_student_t64},
    {"gaussian_posterior", m_gauss_post32, m_gauss_post64},
    {"mvn_precision", m_mvn32, m_mvn64},
    {"logistic", m_logistic32, m_logistic64},
    {"robust_t", m_robust32, m_robust64},
    {"hierarchical", m_hier32, m_hier64},
    {"hrows", m_hrows32, m_hrows64},
};

static const bo_model* find_model(const char* name) {
    for (size_t i = 0; i < sizeof(bo_models) / sizeof(bo_models[0]); i++)
        if (strcmp(bo_models[i].name, name) == 0) return &bo_models[i];
    return NULL;
}

int bo_model_exists(const char* name) { return find_model(name) ? 0 : -1; }

float bo_logfn32(const char* name, uint32_t data_len, uint32_t params_len, const float* params,
                 uint32_t dim, const float* x) {
    const bo_model* m = find_model(name);
    return m ? m->f32(data_len, params_len, params, dim, x) : NAN;
}

double bo_logfn64(const char* name, uint32_t data_len, uint32_t params_len, const float* params,
                  uint32_t dim, const double* x) {
    const bo_model* m = find_model(name);
    return m ? m->f64(data_len, params_len, params, dim, x) : NAN;
}

void bo_logfn_all(const char* name, uint64_t walkers, uint32_t dim, uint32_t data_len,
                  uint32_t params_len, const float* params, const float* xs, float* res,
                  int threads) {
    const bo_model* m = find_model(name);
    if (!m) return;
    (void)threads;
#pragma omp parallel for schedule(static) num_threads(threads > 0 ? threads : 1)
    for (int64_t k = 0; k < (int64_t)walkers; k++)
        res[k] = m->f32(data_len, params_len, params, dim, xs + (uint64_t)k * dim);
}

/* ======================= stretch move ==================================
 * nvidia-gtx-mcmc-stretch.cu:35-99 (OpenCL twin amd-gcn-mcmc-stretch.cl:31-81).
 * Philox key {seed, 0xdecafbad}, ctr {k, step, stream, 0xbeeff00d};
 * z = (a - 2 + 1/a) u1^2 + 2(1 - 1/a) u1 + 1/a [Christen 2007], first product fused;
 * partner j = (uint)(u0*K) (walker), clamped to the half; with BO_PARTNER_ELEMENT the
 * reference's element offset (uint)(u0*K*DIM) (:75), whose elements past the half's end
 * (read out of bounds, or racing with the moving half, in the reference) read as 0 here
 * and in the library's compat kernels;
 * Y_i = S_ji + z (X_ki - S_ji) fused; accept if u2 <= z^(D-1) exp(beta (f(Y) - f(X_k)))
 * (fp32, as the reference), or in log space with BO_ACCEPT_LOG (the library's test). */
/* Walker k's draws and proposal: z, u2 and Y (D floats). */
static void stretch_propose_one(const bo_stretch_args* A, uint32_t k, float* Y, float* z_out,
                                float* u2_out) {
    const uint32_t K = A->K, D = A->dim;
    const float a = A->a;
    const float inv_a = 1.0f / a;
    const float c1 = (a - 2.0f) + inv_a;
    const float c2 = 2.0f * (1.0f - inv_a);
    const float c3 = inv_a;
    const uint32_t key[2] = {A->seed, 0xdecafbadu};
    const uint32_t ctr[4] = {k, A->step, A->stream, 0xbeeff00du};
    float u[4];
    philox_u01x4(ctr, key, u);
    const float z = fmaf(c1 * u[1], u[1], c2 * u[1]) + c3;
    uint64_t j0;
    if (A->flags & BO_PARTNER_ELEMENT) {
        j0 = (uint32_t)(u[0] * (float)K * (float)D);
    } else {
        uint32_t j = (uint32_t)(u[0] * (float)K);
        if (j >= K) j = K - 1;
        j0 = (uint64_t)j * D;
    }
    const uint64_t k0 = (uint64_t)k * D;
    const uint64_t half_len = (uint64_t)K * D;
    for (uint32_t i = 0; i < D; i++) {
        const float s = (j0 + i < half_len) ? A->S[j0 + i] : 0.0f;
        Y[i] = fmaf(z, A->X[k0 + i] - s, s);
    }
    *z_out = z;
    *u2_out = u[2];
}

/* The library kernels' logarithm (bay_log_det), restated with the same operations, each
 * rounded on its own (this build has -ffp-contract=off): x = m 2^e, m in [sqrt(1/2),
 * sqrt(2)), log m = 2 atanh(s) with s = (m - 1)/(m + 1) by its series to s^11, plus e ln 2
 * with ln 2 in two parts.  Same bits as the kernels for positive normal x. */
float bo_log_det(float x) {
    uint32_t b;
    memcpy(&b, &x, sizeof b);
    int e = (int)(b >> 23) - 127;
    const uint32_t mb = (b & 0x007fffffu) | 0x3f800000u;
    float m;
    memcpy(&m, &mb, sizeof m);
    if (m > 1.41421354f) {
        m = m * 0.5f;
        e += 1;
    }
    const float f = m - 1.0f;
    const float s = f / (2.0f + f);
    const float w = s * s;
    float p = fmaf(w, 0.181818187f, 0.222222224f);
    p = fmaf(w, p, 0.285714298f);
    p = fmaf(w, p, 0.400000006f);
    p = fmaf(w, p, 0.666666687f);
    const float lm = fmaf(s * w, p, s + s);
    const float fe = (float)e;
    return fmaf(fe, 0.693145752f, fmaf(fe, 1.42860677e-06f, lm));
}

/* Walker k's accept test given its proposal's log density ly; on accept Y and ly replace
 * the walker's position and log density.  Returns the decision.  BO_ACCEPT_LOG: the
 * library's default test, log u <= (D-1) log z + beta (ly - lx) in fp32 with bo_log_det;
 * else the reference's u <= z^(D-1) exp(beta (ly - lx)). */
static int stretch_accept_one(const bo_stretch_args* A, uint32_t k, const float* Y, float z,
                              float u2, float ly) {
    const uint32_t D = A->dim;
    int accepted;
    if (A->flags & BO_ACCEPT_LOG) {
        const float dl = A->beta * (ly - A->logfn_X[k]);
        accepted = isfinite(ly) && bo_log_det(u2) <= fmaf((float)(D - 1), bo_log_det(z), dl);
    } else {
        const float q = isfinite(ly)
            ? powf(z, (float)(D - 1)) * expf(A->beta * (ly - A->logfn_X[k])) : 0.0f;
        accepted = u2 <= q;
    }
    if (accepted) {
        const uint64_t k0 = (uint64_t)k * D;
        for (uint32_t i = 0; i < D; i++) A->X[k0 + i] = Y[i];
        A->logfn_X[k] = ly;
    }
    if (A->accepted) A->accepted[k] = (uint8_t)accepted;
    return accepted;
}

void bo_stretch_half(const bo_stretch_args* A) {
    const bo_model* m = find_model(A->model);
    if (!m) return;
    const uint32_t K = A->K, D = A->dim;
#pragma omp parallel num_threads(A->threads > 0 ? A->threads : 1)
    {
        float* Y = (float*)malloc(sizeof(float) * (D > 0 ? D : 1));
#pragma omp for schedule(static)
        for (int64_t kk = 0; kk < (int64_t)K; kk++) {
            const uint32_t k = (uint32_t)kk;
            float z, u2;
            stretch_propose_one(A, k, Y, &z, &u2);
            const float ly = m->f32(A->data_len, A->params_len, A->params, D, Y);
            stretch_accept_one(A, k, Y, z, u2, ly);
        }
        free(Y);
    }
}

void bo_stretch_propose(const bo_stretch_args* A, float* Y, float* zs, float* u2s) {
    for (uint32_t k = 0; k < A->K; k++)
        stretch_propose_one(A, k, Y + (uint64_t)k * A->dim, &zs[k], &u2s[k]);
}

void bo_stretch_accept(const bo_stretch_args* A, const float* Y, const float* zs,
                       const float* u2s, const float* ly) {
    for (uint32_t k = 0; k < A->K; k++)
        stretch_accept_one(A, k, Y + (uint64_t)k * A->dim, zs[k], u2s[k], ly[k]);
}

/* ======================= reductions ==================================== */
/* block_reduction_sum_uint pattern (nvidia-gtx-mcmc-stretch.cu:8-33): at each level
 * with i active slots, slot l < i/2 adds slot l + i/2, and when i is odd the last
 * active slot first adds the stray slot i-1.  Simulated sequentially. */
float bo_tree_sum_f32(const float* v, uint32_t L) {
    if (L == 0) return 0.0f;
    float* lacc = (float*)malloc(sizeof(float) * L);
    memcpy(lacc, v, sizeof(float) * L);
    uint32_t i = L;
    while (i > 0) {
        const int odd = (i & 1u) != 0;
        const uint32_t h = i >> 1;
        for (uint32_t l = 0; l < h; l++) {
            float p = lacc[l];
            if (odd && l == h - 1) p += lacc[l + h + 1];
            p += lacc[l + h];
            lacc[l] = p;
        }
        i = h;
    }
    const float r = lacc[0];
    free(lacc);
    return r;
}

/* launch-reduce! (clojurecuda 0.7.2 toolbox): the main kernel reduces blocks of
 * B = min(count, wgs) values (the grid helpers clamp a block to the problem size),
 * then the reduction kernel reduces the partials again, block by block, until one
 * value is left.  Past-the-end slots of a partial block contribute 0.  The clamp is
 * pinned by the golden vertical means sum (nvidia_gtx_test.clj:255-258). */
float bo_launch_reduce_f32(const float* v, uint64_t n, uint32_t wgs) {
    if (n == 0) return 0.0f;
    uint64_t cnt = n;
    float* cur = (float*)malloc(sizeof(float) * n);
    memcpy(cur, v, sizeof(float) * n);
    float* blk = (float*)malloc(sizeof(float) * wgs);
    do {
        const uint32_t B = cnt < wgs ? (uint32_t)cnt : wgs;
        const uint64_t G = (cnt + B - 1) / B;
        for (uint64_t b = 0; b < G; b++) {
            for (uint32_t l = 0; l < B; l++) {
                const uint64_t t = b * B + l;
                blk[l] = t < cnt ? cur[t] : 0.0f;
            }
            cur[b] = bo_tree_sum_f32(blk, B);
        }
        cnt = G;
    } while (cnt > 1);
    const float r = cur[0];
    free(blk);
    free(cur);
    return r;
}

void bo_accu_stats(uint32_t K, uint32_t dim, uint32_t wgs, uint32_t step, const float* X,
                   const uint8_t* accepted, uint32_t* accept_blocks, float* means_blocks) {
    const uint32_t G = (K + wgs - 1) / wgs;
    /* blocks are independent: any thread count gives the same sums */
#pragma omp parallel
    {
    float* blk = (float*)malloc(sizeof(float) * wgs);
#pragma omp for schedule(static)
    for (int64_t bb = 0; bb < (int64_t)G; bb++) {
        const uint32_t b = (uint32_t)bb;
        uint32_t cnt = 0;
        for (uint32_t l = 0; l < wgs; l++) {
            const uint32_t g = b * wgs + l;
            if (g < K && accepted[g]) cnt++;
        }
        accept_blocks[b] += cnt;
        for (uint32_t i = 0; i < dim; i++) {
            for (uint32_t l = 0; l < wgs; l++) {
                const uint32_t g = b * wgs + l;
                blk[l] = g < K ? X[(uint64_t)g * dim + i] : 0.0f;
            }
            means_blocks[b + (uint64_t)G * ((uint64_t)step * dim + i)] += bo_tree_sum_f32(blk, wgs);
        }
    }
    free(blk);
    }
}

/* sum_means_vertical (nvidia-gtx-mcmc-stretch.cu:250-260) run through launch-reduce!
 * with blocks (1, wgs): row r of the m x G partials, data[r*G + g], is tree-summed. */
void bo_sum_means_vertical(uint32_t m, uint32_t G, uint32_t wgs, const float* means_blocks,
                           float* acc) {
    for (uint32_t r = 0; r < m; r++) acc[r] = bo_launch_reduce_f32(means_blocks + (uint64_t)r * G, G, wgs);
}

/* ======================= moments ======================================= */
/* GTXStretch mean (nvidia_gtx.clj:513-522): mean_reduce via launch-reduce! with
 * blocks (1, WGS), then scal! by (float)(1.0/W). */
void bo_mean_ref(uint32_t dim, uint64_t walkers, uint32_t wgs, const float* xs, float* mean) {
    float* col = (float*)malloc(sizeof(float) * walkers);
    const float alpha = (float)(1.0 / (double)walkers);
    for (uint32_t d = 0; d < dim; d++) {
        for (uint64_t k = 0; k < walkers; k++) col[k] = xs[k * dim + d];
        mean[d] = bo_launch_reduce_f32(col, walkers, wgs) * alpha;
    }
    free(col);
}

/* GTXStretch variance (nvidia_gtx.clj:524-537): variance_reduce sums (x - mu)^2. */
void bo_variance_ref(uint32_t dim, uint64_t walkers, uint32_t wgs, const float* xs, float* var) {
    float* mu = (float*)malloc(sizeof(float) * dim);
    bo_mean_ref(dim, walkers, wgs, xs, mu);
    float* col = (float*)malloc(sizeof(float) * walkers);
    const float alpha = (float)(1.0 / (double)walkers);
    for (uint32_t d = 0; d < dim; d++) {
        for (uint64_t k = 0; k < walkers; k++) {
            const float df = xs[k * dim + d] - mu[d];
            col[k] = df * df;
        }
        var[d] = bo_launch_reduce_f32(col, walkers, wgs) * alpha;
    }
    free(col);
    free(mu);
}

void bo_mean64(uint32_t dim, uint64_t walkers, const float* xs, double* mean) {
    for (uint32_t d = 0; d < dim; d++) {
        double s = 0.0;
        for (uint64_t k = 0; k < walkers; k++) s += xs[k * dim + d];
        mean[d] = s / (double)walkers;
    }
}

void bo_variance64(uint32_t dim, uint64_t walkers, const float* xs, double* var) {
    for (uint32_t d = 0; d < dim; d++) {
        double s = 0.0;
        for (uint64_t k = 0; k < walkers; k++) s += xs[k * dim + d];
        const double mu = s / (double)walkers;
        double q = 0.0;
        for (uint64_t k = 0; k < walkers; k++) {
            const double df = xs[k * dim + d] - mu;
            q += df * df;
        }
        var[d] = q / (double)walkers;
    }
}

/* ======================= histogram ===================================== */
/* min_max_reduce / min_max_reduction via launch-reduce! (nvidia-gtx-estimate.cu:48-115,
 * nvidia_gtx.clj:487-499).  The exact min/max are order independent; the reference's
 * past-the-end slots carry 0.0 (estimate.cu:91-96, 105-106), which enters the result
 * whenever a reduction level has a partial block of B = min(count, wgsn) slots,
 * wgsn = WGS / min(dim, sqrt(WGS)). */
void bo_limits(uint32_t dim, uint64_t walkers, uint32_t wgs, const float* xs, uint32_t flags,
               float* limits) {
    int zero = 0;
    if (flags & BO_HIST_ZERO_LIMITS) {
        uint32_t sq = (uint32_t)sqrt((double)wgs);
        uint32_t wgsm = dim < sq ? dim : sq;
        if (wgsm == 0) wgsm = 1;
        const uint64_t wgsn = wgs / wgsm;
        uint64_t cnt = walkers;
        do {
            const uint64_t B = cnt < wgsn ? cnt : wgsn;
            if (cnt % B != 0) zero = 1;
            cnt = (cnt + B - 1) / B;
        } while (cnt > 1);
    }
    for (uint32_t d = 0; d < dim; d++) {
        float mn = xs[d], mx = xs[d];
        for (uint64_t k = 1; k < walkers; k++) {
            const float v = xs[k * dim + d];
            mn = v < mn ? v : mn;
            mx = v > mx ? v : mx;
        }
        if (zero) {
            mn = mn < 0.0f ? mn : 0.0f;
            mx = mx > 0.0f ? mx : 0.0f;
        }
        limits[2 * d] = mn;
        limits[2 * d + 1] = mx;
    }
}

/* histogram (nvidia-gtx-estimate.cu:5-32): bin = (uint)((x - lo)/(hi - lo) * B), with
 * the GPU's saturating float->uint conversion (negative and NaN give 0), clamped to B-1.
 * The division is IEEE here and in the build's kernel (the reference divides with the
 * fast-math approximation, which can move a value sitting on a bin edge). */
void bo_histogram_counts(uint32_t dim, uint64_t walkers, uint32_t bins, const float* limits,
                         const float* xs, uint32_t* counts) {
    for (uint32_t d = 0; d < dim; d++) {
        const float lo = limits[2 * d], hi = limits[2 * d + 1];
        const float range = hi - lo;
        for (uint64_t k = 0; k < walkers; k++) {
            const float v = (xs[k * dim + d] - lo) / range * (float)bins;
            uint32_t b;
            if (!(v > 0.0f)) b = 0;
            else if (v >= 4294967295.0f) b = 0xffffffffu;
            else b = (uint32_t)v;
            if (b >= bins) b = bins - 1;
            counts[(uint64_t)bins * d + b]++;
        }
    }
}

/* uint_to_real (nvidia-gtx-estimate.cu:34-44) with alpha = (float)(bins/n). */
void bo_uint_to_real(uint32_t dim, uint32_t bins, uint64_t n, const float* limits,
                     const uint32_t* counts, float* pdf) {
    const float alpha = (float)((double)bins / (double)n);
    for (uint32_t d = 0; d < dim; d++) {
        const float c = alpha / (limits[2 * d + 1] - limits[2 * d]);
        for (uint32_t b = 0; b < bins; b++)
            pdf[(uint64_t)bins * d + b] = c * (float)counts[(uint64_t)bins * d + b];
    }
}

/* bitonic_local (nvidia-gtx-estimate.cu:117-147): a bitonic network over (index, pdf)
 * pairs ordering bins by decreasing pdf; a compare between positions lid and j = lid^inc
 * treats equal pdfs as "smaller" when j < lid.  Simulated stage by stage. */
void bo_bitonic_ranks(uint32_t dim, uint32_t bins, const float* pdf, float* ranks) {
    float* ax = (float*)malloc(sizeof(float) * bins);
    float* ay = (float*)malloc(sizeof(float) * bins);
    float* nx = (float*)malloc(sizeof(float) * bins);
    float* ny = (float*)malloc(sizeof(float) * bins);
    for (uint32_t d = 0; d < dim; d++) {
        for (uint32_t l = 0; l < bins; l++) {
            ax[l] = (float)l;
            ay[l] = pdf[(uint64_t)bins * d + l];
        }
        for (uint32_t length = 1; length < bins; length <<= 1) {
            for (uint32_t inc = length; inc > 0; inc >>= 1) {
                for (uint32_t l = 0; l < bins; l++) {
                    const int direction = (l & (length << 1)) != 0;
                    const uint32_t j = l ^ inc;
                    const int smaller = (ay[l] < ay[j]) || (ay[j] == ay[l] && j < l);
                    const int swap = smaller ^ (j < l) ^ direction;
                    nx[l] = swap ? ax[j] : ax[l];
                    ny[l] = swap ? ay[j] : ay[l];
                }
                memcpy(ax, nx, sizeof(float) * bins);
                memcpy(ay, ny, sizeof(float) * bins);
            }
        }
        for (uint32_t l = 0; l < bins; l++) ranks[(uint64_t)bins * d + l] = ax[l];
    }
    free(ax);
    free(ay);
    free(nx);
    free(ny);
}

/* ======================= acor ==========================================
 * GTXAcorEngine.acor (nvidia_gtx.clj:240-278) + acor kernels (nvidia-gtx-acor.cu:5-168). */
#define ACOR_MIN_FAC 5u
#define ACOR_MIN_LAG 10u
#define ACOR_MAX_LAG 64u

static uint32_t acor_lag(uint32_t n, uint32_t wgs) {
    uint32_t l = n / ACOR_MIN_FAC;
    if (wgs < l) l = wgs;
    if (ACOR_MAX_LAG < l) l = ACOR_MAX_LAG;
    return l < ACOR_MIN_LAG ? ACOR_MIN_LAG : l;
}

/* acor_1d (nvidia-gtx-acor.cu:40-103) for one dim, fp32, blocks of B = min(wgs, n):
 * x_t = m[t] if t + lag < n else 0; within a block the lag window reads these x,
 * across the block edge it reads raw m (the next block's first lag entries).
 * Per block c0 = tree sum x_t^2, d = tree sum x_t (x_t + 2 sum_{s=1..lag} window);
 * blocks are added in block order (the reference uses atomicAdd). */
static void acor_pass32(uint32_t n, uint32_t wgs, uint32_t lag, const float* m, uint64_t stride,
                        float* c0acc, float* dacc) {
    const uint32_t B = wgs < n ? wgs : n;
    const uint32_t G = (n - 1) / B + 1;
    float* loc = (float*)malloc(sizeof(float) * 2 * B);
    float* vc = (float*)malloc(sizeof(float) * B);
    float* vd = (float*)malloc(sizeof(float) * B);
    for (uint32_t b = 0; b < G; b++) {
        for (uint32_t l = 0; l < B; l++) {
            const uint64_t t = (uint64_t)b * B + l;
            loc[l] = (t + lag < n) ? m[t * stride] : 0.0f;
            const int load = (l < lag) && (b + 1 < G);
            const uint64_t t2 = t + B;
            loc[l + B] = (load && t2 < n) ? m[t2 * stride] : 0.0f;
        }
        for (uint32_t l = 0; l < B; l++) {
            const float x = loc[l];
            float acc = 0.0f;
            for (uint32_t s = 0; s < lag; s++) acc += loc[l + s + 1];
            vd[l] = x * fmaf(2.0f, acc, x);
            vc[l] = x * x;
        }
        *c0acc += bo_tree_sum_f32(vc, B);
        *dacc += bo_tree_sum_f32(vd, B);
    }
    free(loc);
    free(vc);
    free(vd);
}

int bo_acor_ref(uint32_t D, uint32_t n, uint32_t wgs, const float* series, float* tau,
                float* mean, float* sigma, uint32_t* lag_out) {
    const uint32_t lag = acor_lag(n, wgs);
    if (lag_out) *lag_out = lag;
    if (lag * ACOR_MIN_FAC > n) return -1;
    float* m = (float*)malloc(sizeof(float) * (uint64_t)D * n);
    memcpy(m, series, sizeof(float) * (uint64_t)D * n);
    float* row = (float*)malloc(sizeof(float) * n);
    const float alpha = (float)(1.0 / (double)n);
    for (uint32_t d = 0; d < D; d++) {
        /* mean: sum_reduce_horizontal through launch-reduce! with blocks of
         * wgsn = WGS / min(16, D, WGS) along the series, then scal! 1/n. */
        uint32_t wgsm = 16;
        if (D < wgsm) wgsm = D;
        if (wgs < wgsm) wgsm = wgs;
        const uint32_t wgsn = wgs / wgsm;
        for (uint32_t t = 0; t < n; t++) row[t] = m[(uint64_t)t * D + d];
        const float mu = bo_launch_reduce_f32(row, n, wgsn) * alpha;
        mean[d] = mu;
        for (uint32_t t = 0; t < n; t++) m[(uint64_t)t * D + d] -= mu; /* subtract_mean */

        float* md = m + d;
        float c0a = 0.0f, da = 0.0f;
        acor_pass32(n, wgs, lag, md, D, &c0a, &da);
        const float c0 = c0a;
        float t = da / c0;
        uint32_t lag2 = lag, n2 = n, stride = 1;
        while ((ACOR_MIN_LAG < lag2) && ((float)lag2 < t * (float)ACOR_MIN_FAC)) {
            n2 /= 2;
            lag2 = ((lag * ACOR_MIN_FAC) < n2) ? lag : ((n2 / ACOR_MIN_FAC) > 10u ? n2 / ACOR_MIN_FAC : 10u);
            const float c0prev = c0a;
            c0a = 0.0f;
            da = 0.0f;
            /* sum_pairwise (acor.cu:28-38): x[2g*S] += x[(2g+1)*S], S = stride*D */
            for (uint32_t g = 0; g < n2; g++)
                md[(uint64_t)2 * g * stride * D] += md[(uint64_t)(2 * g + 1) * stride * D];
            stride *= 2;
            acor_pass32(n2, wgs, lag2, md, (uint64_t)stride * D, &c0a, &da);
            t = da / c0prev;
        }
        const float scale = (float)stride * (float)(n2 - lag2);
        tau[d] = da * (float)(n - lag) / (scale * c0);
        sigma[d] = sqrtf(da / (scale * (float)n));
    }
    free(row);
    free(m);
    return 0;
}

/* Same recursion with double arithmetic and serial sums (the block-edge window rule is
 * kept: it is part of the reference's definition of D). */
static void acor_pass64(uint32_t n, uint32_t wgs, uint32_t lag, const double* m, uint64_t stride,
                        double* c0acc, double* dacc) {
    const uint32_t B = wgs < n ? wgs : n;
    double c0 = 0.0, dd = 0.0;
    for (uint64_t t = 0; t + lag < n; t++) {
        const double x = m[t * stride];
        const uint64_t blk_end = (t / B + 1) * B;
        double acc = 0.0;
        for (uint32_t s = 1; s <= lag; s++) {
            const uint64_t u = t + s;
            double v;
            if (u < blk_end) v = (u + lag < n) ? m[u * stride] : 0.0;
            else v = (u < n) ? m[u * stride] : 0.0;
            acc += v;
        }
        c0 += x * x;
        dd += x * (x + 2.0 * acc);
    }
    *c0acc = c0;
    *dacc = dd;
}

int bo_acor64(uint32_t D, uint32_t n, uint32_t wgs, const float* series, double* tau,
              double* mean, double* sigma, uint32_t* lag_out) {
    const uint32_t lag = acor_lag(n, wgs);
    if (lag_out) *lag_out = lag;
    if (lag * ACOR_MIN_FAC > n) return -1;
    double* md = (double*)malloc(sizeof(double) * n);
    for (uint32_t d = 0; d < D; d++) {
        double s = 0.0;
        for (uint32_t t = 0; t < n; t++) s += series[(uint64_t)t * D + d];
        const double mu = s / (double)n;
        mean[d] = mu;
        for (uint32_t t = 0; t < n; t++) md[t] = (double)series[(uint64_t)t * D + d] - mu;
        double c0a, da;
        acor_pass64(n, wgs, lag, md, 1, &c0a, &da);
        const double c0 = c0a;
        double t = da / c0;
        uint32_t lag2 = lag, n2 = n, stride = 1;
        while ((ACOR_MIN_LAG < lag2) && ((double)lag2 < t * (double)ACOR_MIN_FAC)) {
            n2 /= 2;
            lag2 = ((lag * ACOR_MIN_FAC) < n2) ? lag : ((n2 / ACOR_MIN_FAC) > 10u ? n2 / ACOR_MIN_FAC : 10u);
            const double c0prev = c0a;
            for (uint32_t g = 0; g < n2; g++) md[(uint64_t)2 * g * stride] += md[(uint64_t)(2 * g + 1) * stride];
            stride *= 2;
            acor_pass64(n2, wgs, lag2, md, stride, &c0a, &da);
            t = da / c0prev;
        }
        const double scale = (double)stride * (double)(n2 - lag2);
        tau[d] = da * (double)(n - lag) / (scale * c0);
        sigma[d] = sqrt(da / (scale * (double)n));
    }
    free(md);
    return 0;
}
