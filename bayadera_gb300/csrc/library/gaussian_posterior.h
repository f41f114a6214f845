// Unknown-mean-and-sd Gaussian posterior: the data likelihood gaussian_loglik with the
// prior N(mu | h0, h1^2) x Uniform(sigma | h2, h3); x = (mu, sigma).
//  - gaussian_posterior_logpdf: the reference's posterior composition
//    (cuda/distributions/posterior.cu:5-10), loglik(data) + prior(&params[data_len]).
//  - gaussian_posterior_{prep,term,walker}: the same density in the data-tiled form.
#include <stdint.h>
extern "C" {
inline REAL gaussian_posterior_prior(const uint32_t data_len, const uint32_t hyper_len,
                                     const REAL* h, const uint32_t dim, const REAL* x) {
    return gaussian_log(h[0], h[1], x[0]) + uniform_log(h[2], h[3], x[1]);
}
inline REAL gaussian_posterior_logpdf(const uint32_t data_len, const uint32_t hyper_len,
                                      const REAL* params, const uint32_t dim, const REAL* x) {
    return gaussian_loglik(data_len, params, dim, x)
        + gaussian_posterior_prior(data_len, hyper_len, &params[data_len], dim, x);
}
inline void gaussian_posterior_prep(const REAL* h, const uint32_t hyper_len, const uint32_t dim,
                                    const REAL* x, REAL* prep) {
    prep[0] = x[0];
    prep[1] = -0.5f / (x[1] * x[1]);
}
inline REAL gaussian_posterior_term(const REAL* row, const REAL* prep) {
    const REAL d = row[0] - prep[0];
    return d * d * prep[1];
}
inline REAL gaussian_posterior_walker(const uint64_t n_rows, const REAL* h,
                                      const uint32_t hyper_len, const uint32_t dim, const REAL* x) {
    if (!(0.0f < x[1])) return nanf("");
    return (REAL)n_rows * gaussian_log_scale(x[1]) + gaussian_posterior_prior(0, hyper_len, h, dim, x);
}
}
// data-tiled form, four walkers at once (prep4[i]: prep value i of the four walkers); the
// same operations as gaussian_posterior_term, lane by lane
inline bay_v4 gaussian_posterior_term4(const REAL* row, const bay_v4* prep4) {
    const bay_v4 d = row[0] - prep4[0];
    return d * d * prep4[1];
}
#define BAY_TILE_TERM4 gaussian_posterior_term4
