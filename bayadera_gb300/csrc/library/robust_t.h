// Robust linear regression with Student-t(nu) residuals: x = (beta_1..beta_F, log sigma),
// dim = F + 1; data rows (x_1..x_F, y); hyperparameters (nu, beta_sd, logsigma_sd).
// log density = sum_n -(nu+1)/2 log(1 + r_n^2/nu) - N log sigma
//             - |beta|^2/(2 beta_sd^2) - (log sigma)^2/(2 logsigma_sd^2),  r = (y - x.beta)/sigma.
#include <stdint.h>
extern "C" {
inline REAL robust_t_logpdf(const uint32_t data_len, const uint32_t hyper_len,
                            const REAL* params, const uint32_t dim, const REAL* x) {
    const uint32_t F = dim - 1, row = F + 1, n = data_len / row;
    const REAL* h = params + data_len;
    const REAL nu = h[0], ls = x[F], inv_s = expf(-ls);
    REAL res = 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        const REAL* r = params + (uint64_t)i * row;
        REAL eta = 0.0f;
        for (uint32_t f = 0; f < F; ++f) eta = fmaf(r[f], x[f], eta);
        const REAL z = (r[F] - eta) * inv_s;
        res += -0.5f * (nu + 1.0f) * logf(1.0f + z * z / nu);
    }
    REAL pb = 0.0f;
    for (uint32_t f = 0; f < F; ++f) pb = fmaf(x[f], x[f], pb);
    return res - (REAL)n * ls - pb / (2.0f * h[1] * h[1]) - ls * ls / (2.0f * h[2] * h[2]);
}
// GEMM form: A = the data rows' features, aux = y; prep = (1/sigma, 1/(nu sigma^2),
// -(nu+1)/2), so that a row term is two multiply-adds and one log.
inline void robust_t_prep(const REAL* h, const uint32_t hyper_len, const uint32_t dim,
                          const REAL* x, REAL* prep) {
    prep[0] = expf(-x[dim - 1]);
    prep[1] = prep[0] * prep[0] / h[0];
    prep[2] = -0.5f * (h[0] + 1.0f);
}
inline REAL robust_t_term(const REAL eta, const REAL* aux, const uint64_t row, const REAL* x,
                          const REAL* prep) {
    const REAL r = aux[0] - eta;
    return prep[2] * logf(fmaf(r * r, prep[1], 1.0f));
}
inline REAL robust_t_walker(const uint64_t rows, const REAL* h, const uint32_t hyper_len,
                            const uint32_t dim, const REAL* x) {
    const uint32_t F = dim - 1;
    const REAL ls = x[F];
    REAL pb = 0.0f;
    for (uint32_t f = 0; f < F; ++f) pb = fmaf(x[f], x[f], pb);
    return -(REAL)rows * ls - pb / (2.0f * h[1] * h[1]) - ls * ls / (2.0f * h[2] * h[2]);
}
}
