// Gaussian hierarchical model: y_ij ~ N(theta_j, sigma_j^2) with known sigma_j,
// theta_j ~ N(mu, tau^2), mu ~ N(0, h0^2), log tau ~ N(0, h1^2);
// x = (theta_1..theta_J, mu, log tau), dim = J + 2.
// Data (float-encoded): [J, sigma_1..sigma_J, off_0..off_J, y_0..y_{N-1}], group j owns
// y[off_j .. off_{j+1}).
#include <stdint.h>
extern "C" {
inline REAL hierarchical_logpdf(const uint32_t data_len, const uint32_t hyper_len,
                                const REAL* params, const uint32_t dim, const REAL* x) {
    const uint32_t J = (uint32_t)params[0];
    const REAL* sig = params + 1;
    const REAL* off = params + 1 + J;
    const REAL* y = params + 2 + 2 * J;
    const REAL* h = params + data_len;
    const REAL mu = x[J], lt = x[J + 1], inv_t2 = expf(-2.0f * lt);
    REAL res = 0.0f;
    for (uint32_t j = 0; j < J; ++j) {
        const REAL c = -0.5f / (sig[j] * sig[j]);
        const uint32_t b = (uint32_t)off[j], e = (uint32_t)off[j + 1];
        REAL s = 0.0f;
        for (uint32_t i = b; i < e; ++i) {
            const REAL d = y[i] - x[j];
            s = fmaf(d * d, c, s);
        }
        const REAL dt = x[j] - mu;
        res += s - 0.5f * dt * dt * inv_t2 - lt;
    }
    return res - mu * mu / (2.0f * h[0] * h[0]) - lt * lt / (2.0f * h[1] * h[1]);
}
}
