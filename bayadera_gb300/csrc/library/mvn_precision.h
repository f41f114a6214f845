// Zero-mean multivariate Gaussian given its precision matrix P (dim x dim, row-major,
// the hyperparameters): log density -1/2 x'Px up to a constant.
#include <stdint.h>
extern "C" {
inline REAL mvn_precision_logpdf(const uint32_t data_len, const uint32_t hyper_len,
                                 const REAL* params, const uint32_t dim, const REAL* x) {
    const REAL* P = params + data_len;
    REAL acc = 0.0f;
    for (uint32_t i = 0; i < dim; ++i) {
        REAL t = 0.0f;
        for (uint32_t j = 0; j < dim; ++j) t = fmaf(P[i * dim + j], x[j], t);
        acc = fmaf(x[i], t, acc);
    }
    return -0.5f * acc;
}
// The same density in the GEMM form: A = P (the hyperparameters), eta = P x,
// log density = sum_r -x_r eta_r / 2.
inline void mvn_precision_prep(const REAL* hyper, const uint32_t hyper_len, const uint32_t dim,
                               const REAL* x, REAL* prep) {}
inline REAL mvn_precision_term(const REAL eta, const REAL* aux, const uint64_t row,
                               const REAL* x, const REAL* prep) {
    return -0.5f * x[row] * eta;
}
inline REAL mvn_precision_walker(const uint64_t rows, const REAL* hyper, const uint32_t hyper_len,
                                 const uint32_t dim, const REAL* x) {
    return 0.0f;
}
}
