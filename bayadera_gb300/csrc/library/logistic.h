// Bayesian logistic regression: data rows (x_1..x_F, y) with y in {0, 1}, F = dim;
// hyperparameter h0 = prior sd of every coefficient.
// log density = sum_n [y_n eta_n - softplus(eta_n)] - |beta|^2 / (2 h0^2),
// eta_n = x_n . beta, softplus(e) = max(e, 0) + log(1 + exp(-|e|)); log(1 + t) for
// t = exp(-|e|) in (0, 1] has an absolute rounding error below 2^-24 (fast-math exp and
// log are single MUFU operations; log1pf is not).
#include <stdint.h>
extern "C" {
inline REAL logistic_softplus(const REAL e) { return fmaxf(e, 0.0f) + logf(1.0f + expf(-fabsf(e))); }
inline REAL logistic_logpdf(const uint32_t data_len, const uint32_t hyper_len,
                            const REAL* params, const uint32_t dim, const REAL* beta) {
    const uint32_t row = dim + 1, n = data_len / row;
    REAL res = 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        const REAL* r = params + (uint64_t)i * row;
        REAL eta = 0.0f;
        for (uint32_t f = 0; f < dim; ++f) eta = fmaf(r[f], beta[f], eta);
        res += fmaf(r[dim], eta, -logistic_softplus(eta));
    }
    const REAL sd = params[data_len];
    REAL pr = 0.0f;
    for (uint32_t f = 0; f < dim; ++f) pr = fmaf(beta[f], beta[f], pr);
    return res - pr / (2.0f * sd * sd);
}
// GEMM form: A = the data rows' features, aux = y.
inline void logistic_prep(const REAL* hyper, const uint32_t hyper_len, const uint32_t dim,
                          const REAL* beta, REAL* prep) {}
inline REAL logistic_term(const REAL eta, const REAL* aux, const uint64_t row, const REAL* beta,
                          const REAL* prep) {
    return fmaf(aux[0], eta, -logistic_softplus(eta));
}
inline REAL logistic_walker(const uint64_t rows, const REAL* hyper, const uint32_t hyper_len,
                            const uint32_t dim, const REAL* beta) {
    REAL pr = 0.0f;
    for (uint32_t f = 0; f < dim; ++f) pr = fmaf(beta[f], beta[f], pr);
    return -pr / (2.0f * hyper[0] * hyper[0]);
}
}
