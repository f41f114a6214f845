// Binomial family (cuda/distributions/binomial.cu names): params (n, p[, k]).
#include <stdint.h>
extern "C" {
inline REAL lbinco(const REAL n, const REAL k) {
    return lgamma(n + 1.0f) - lgamma(k + 1.0f) - lgamma(n - k + 1.0f);
}
inline REAL binomial_log_unscaled(const REAL n, const REAL p, const REAL k) {
    return k * log(p) + (n - k) * log(1.0f - p);
}
inline REAL binomial_log(const REAL n, const REAL p, const REAL k) {
    return binomial_log_unscaled(n, p, k) + lbinco(n, k);
}
inline REAL binomial_mcmc_logpdf(const uint32_t data_len, const uint32_t params_len,
                                 const REAL* params, const uint32_t dim, const REAL* k) {
    return binomial_log_unscaled(params[0], params[1], k[0]);
}
inline REAL binomial_logpdf(const uint32_t data_len, const uint32_t params_len,
                            const REAL* params, const uint32_t dim, const REAL* k) {
    return binomial_log(params[0], params[1], k[0]);
}
// data = (n, k) trials and successes, x = (p).
inline REAL binomial_loglik(const uint32_t data_len, const REAL* data, const uint32_t dim,
                            const REAL* p) {
    return binomial_log_unscaled(data[0], p[0], data[1]);
}
}
