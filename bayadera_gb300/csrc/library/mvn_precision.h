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
}
