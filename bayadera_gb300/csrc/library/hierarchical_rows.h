// Gaussian hierarchical model on observation rows: y_i ~ N(theta_{g_i}, sigma_{g_i}^2)
// with known sigma, theta_j ~ N(mu, tau^2), mu ~ N(0, h0^2), log tau ~ N(0, h1^2);
// x = (theta_1..theta_J, mu, log tau), dim = J + 2.
// Data rows (y, g, c): the observation, its group index as a float, and
// c = -1 / (2 sigma_g^2); hyperparameters (h0, h1) after the rows.
// log density = sum_i c_i (y_i - theta_{g_i})^2
//             + sum_j [-(theta_j - mu)^2 / (2 tau^2) - log tau]
//             - mu^2 / (2 h0^2) - (log tau)^2 / (2 h1^2)         (constants dropped)
#include <stdint.h>
extern "C" {
inline REAL hrows_walker(const uint64_t n_rows, const REAL* h, const uint32_t hyper_len,
                         const uint32_t dim, const REAL* x) {
    const uint32_t J = dim - 2;
    const REAL mu = x[J], lt = x[J + 1];
    const REAL c = -0.5f * expf(-2.0f * lt);
    REAL s = 0.0f;
#pragma unroll 8
    for (uint32_t j = 0; j < J; ++j) {     // (unrolled: several coordinates' loads in flight)
        const REAL d = x[j] - mu;
        s = fmaf(d * d, c, s);
    }
    return s - (REAL)J * lt - mu * mu / (2.0f * h[0] * h[0]) - lt * lt / (2.0f * h[1] * h[1]);
}
// batch form: one row's term; x is the walker's position
inline REAL hrows_term(const REAL* row, const REAL* x, const REAL* prep) {
    const REAL d = row[0] - x[(uint32_t)row[1]];
    return row[2] * d * d;
}
inline void hrows_prep(const REAL* h, const uint32_t hyper_len, const uint32_t dim,
                       const REAL* x, REAL* prep) {}
// plain form (reference ABI): the whole density of one walker
inline REAL hrows_logpdf(const uint32_t data_len, const uint32_t hyper_len,
                         const REAL* params, const uint32_t dim, const REAL* x) {
    const uint32_t n = data_len / 3;
    REAL res = 0.0f;
    for (uint32_t i = 0; i < n; ++i) res += hrows_term(params + 3 * (uint64_t)i, x, x);
    return res + hrows_walker(n, params + data_len, hyper_len, dim, x);
}
}
// batch form, four walkers at once: x4[i] holds coordinate i of the four walkers (one
// 16-byte load per row for all four); the same operations as hrows_term, lane by lane
inline bay_v4 hrows_term4(const REAL* row, const bay_v4* x4, const bay_v4* prep4) {
    const bay_v4 d = row[0] - x4[(uint32_t)row[1]];
    return row[2] * d * d;
}
#define BAY_BATCH_TERM4 hrows_term4
