// Erlang family (cuda/distributions/erlang.cu names): params (lambda, k[, log-norm]).
#include <stdint.h>
extern "C" {
inline REAL erlang_log_unscaled(const REAL lambda, const REAL k, const REAL x) {
    return (k - 1.0f) * log(x) - lambda * x;
}
inline REAL erlang_log_scale(const REAL lambda, const REAL k) { return k * log(lambda) - lgamma(k); }
inline REAL erlang_log(const REAL lambda, const REAL k, const REAL x) {
    return erlang_log_unscaled(lambda, k, x) + erlang_log_scale(lambda, k);
}
inline REAL erlang_mcmc_logpdf(const uint32_t data_len, const uint32_t params_len,
                               const REAL* params, const uint32_t dim, const REAL* x) {
    return erlang_log_unscaled(params[0], params[1], x[0]);
}
inline REAL erlang_logpdf(const uint32_t data_len, const uint32_t params_len, const REAL* params,
                          const uint32_t dim, const REAL* x) {
    return erlang_log_unscaled(params[0], params[1], x[0]) + params[2];
}
}
