// bay_stretch.cuh -- fused affine-invariant stretch move, compiled by NVRTC per model.
//
// One launch moves one half of the ensemble against the other (red/black update):
// Philox draw, stretch factor z ~ g(z) (Christen 2007), partner from the
// complementary half, proposal Y = S_j + z (X_k - S_j), the model's log density at Y,
// the accept step, and (in the "accu" variant) the acceptance count and the per-step
// ensemble sums that feed acor.  Reference: cuda/engines/nvidia-gtx-mcmc-stretch.cu
// stretch_move :35-99, stretch_move_accu :101-134, stretch_move_bare :136-154.
//
// Counter and key words are the reference's: key {seed_h, 0xdecafbad}, counter
// {k, step, stream, 0xbeeff00d}; stream 3333/4444 (bare) and 1111/2222 (accu) for
// halves 0/1; seed_h = seed (half 0) or seed + 1 (half 1).
//
// Layout (both forms): positions structure-of-arrays, xs[d * W + w] (W walkers,
// half h = walkers [h*K, h*K + K)); logfn contiguous, logfn[w].
//
// Macros supplied by the host when it compiles a model:
//   DIM            walker dimension
//   BAY_LOGFN      plain form: REAL f(uint32 data_len, uint32 params_len,
//                  const REAL* params, uint32 dim, const REAL* x)  (reference ABI)
//   BAY_TILED      1 for the data-tiled form, with
//     BAY_TILE_PREP(hyper, hyper_len, dim, x, prep)   per-walker precompute
//     BAY_TILE_TERM(row, prep) -> REAL                 one data row
//     BAY_TILE_WALKER(n_rows, hyper, hyper_len, dim, x) -> REAL   the rest
//     BAY_ROW_LEN, BAY_PREP_LEN, BAY_WPC (walkers per CTA)
//   BAY_CTA        threads per CTA
//   BAY_ACCEPT_REF 1: accept if u <= z^(D-1) exp(beta dl) in fp32 (the reference's
//                  formula); 0 (default): log u <= (D-1) log z + beta dl in FP64.

#ifndef BAY_CTA
#define BAY_CTA 256
#endif
#ifndef BAY_ACCEPT_REF
#define BAY_ACCEPT_REF 0
#endif
#ifndef BAY_TILED
#define BAY_TILED 0
#endif

// Sampler control block, resident in device memory so that captured CUDA graphs
// replay without parameter patching.
struct bay_ctl {
    unsigned int step[2];           // [0] bare move counter, [1] accu move counter
    unsigned int seed[2];           // [0] bare seed, [1] accu seed (half 1 adds 1)
    float a;
    float beta;
    unsigned int ticket[2];         // last-CTA tickets of the accu reductions
    unsigned long long accepted;    // accu: accepted proposals since the last reset
    unsigned int status;            // nonzero: a device-detected error
    unsigned int pad;
};

struct bay_stretch_params {
    const float* params;            // data || hyperparameters
    float* xs;                      // SoA positions
    float* logfn;                   // W log densities
    bay_ctl* ctl;
    double* part;                   // accu: per-CTA partial sums [gridDim.x][DIM]
    double* half_sum;               // accu: [DIM] sums of half 0, consumed by half 1
    float* means;                   // accu: per-step ensemble means, means[step*DIM + d]
    unsigned long long data_len;    // floats of data in params
    unsigned int params_len;        // hyperparameters after the data
    unsigned int W, K;
    unsigned int half;
    unsigned int step_off;          // added to the device step counter
    unsigned int means_cap;         // steps the means buffer holds
    float inv_W;
};

__device__ __forceinline__ float bay_stretch_z(float a, float u1) {
    // z = (a - 2 + 1/a) u1^2 + 2 (1 - 1/a) u1 + 1/a with the first product fused,
    // each other operation IEEE-rounded (matches the oracle and the golden vectors).
    const float inv_a = __fdiv_rn(1.0f, a);
    const float c1 = __fadd_rn(__fsub_rn(a, 2.0f), inv_a);
    const float c2 = __fmul_rn(2.0f, __fsub_rn(1.0f, inv_a));
    return __fadd_rn(__fmaf_rn(__fmul_rn(c1, u1), u1, __fmul_rn(c2, u1)), inv_a);
}

__device__ __forceinline__ unsigned int bay_partner(float u0, unsigned int K) {
    // Walker j = (uint)(u0 * K) of the complementary half; u0 < 1 can still round
    // u0*K up to K, so clamp (the reference would read past the half there).
    unsigned int j = __float2uint_rz(__fmul_rn(u0, (float)K));
    return j < K ? j : K - 1;
}

__device__ __forceinline__ bool bay_accept(float u2, float z, float ly, float lx, float beta) {
#if BAY_ACCEPT_REF
    const float q = isfinite(ly) ? powf(z, (float)(DIM - 1)) * expf(beta * (ly - lx)) : 0.0f;
    return u2 <= q;
#else
    if (!isfinite(ly)) return false;
    const double lq = (double)(DIM - 1) * (double)__logf(z)
        + (double)beta * ((double)ly - (double)lx);
    return (double)__logf(u2) <= lq;
#endif
}

// Per-CTA sum of one value per thread (fp32 within warps, FP64 across warps), result
// valid in thread 0.  Fixed order: deterministic.
__device__ __forceinline__ double bay_cta_sum(float v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = (double)v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    __syncthreads();
    return s;
}

// Accu epilogue: per-CTA accept count and per-dim sums of the moved half, reduced
// across CTAs by the last CTA to finish (ticket), in CTA order.  Half 0 parks its
// sums in half_sum; half 1 adds them and writes the step's ensemble means.
__device__ void bay_accu_epilogue(const bay_stretch_params& P, bool accepted, bool valid,
                                  const float* mine, unsigned int step, double* red) {
    const int n_acc = __syncthreads_count(accepted);
    if (threadIdx.x == 0 && n_acc) atomicAdd(&P.ctl->accepted, (unsigned long long)n_acc);
    for (int d = 0; d < DIM; ++d) {
        const double s = bay_cta_sum(valid ? mine[d] : 0.0f, red);
        if (threadIdx.x == 0) P.part[(size_t)blockIdx.x * DIM + d] = s;
    }
    __shared__ bool last;
    __threadfence();
    if (threadIdx.x == 0) {
        const unsigned int t = atomicAdd(&P.ctl->ticket[P.half], 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int d = threadIdx.x; d < DIM; d += blockDim.x) {
        double s = 0.0;
        for (unsigned int b = 0; b < gridDim.x; ++b) s += ((volatile double*)P.part)[(size_t)b * DIM + d];
        if (P.half == 0) {
            P.half_sum[d] = s;
        } else if (step < P.means_cap) {
            P.means[(size_t)step * DIM + d] = (float)((P.half_sum[d] + s) * (double)P.inv_W);
        }
    }
    if (threadIdx.x == 0) P.ctl->ticket[P.half] = 0;
}

#if !BAY_TILED
// ---------------------------------------------------------------- plain form
// One thread per walker of the moving half, the model's LOGFN evaluated per thread
// (the reference's structure, with SoA coalesced loads and registers for Y).
template <bool ACCU>
__device__ __forceinline__ void bay_stretch_plain(const bay_stretch_params& P) {
    const unsigned int kind = ACCU ? 1u : 0u;
    const unsigned int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = k < P.K;
    const unsigned int step = P.ctl->step[kind] + P.step_off;
    const unsigned int seed = P.ctl->seed[kind] + P.half;
    const float a = P.ctl->a;
    const float beta = ACCU ? 1.0f : P.ctl->beta;
    const unsigned int stream = ACCU ? (P.half ? 2222u : 1111u) : (P.half ? 4444u : 3333u);
    float* X = P.xs + (size_t)P.half * P.K;
    const float* S = P.xs + (size_t)(1u - P.half) * P.K;
    float Y[DIM];
    bool accepted = false;
    if (valid) {
        bay_u4 c;
        c.x = k;
        c.y = step;
        c.z = stream;
        c.w = 0xbeeff00du;
        const bay_u4 r = bay_philox4x32_10(c, seed, 0xdecafbadu);
        const float u0 = bay_u01(r.x), u1 = bay_u01(r.y), u2 = bay_u01(r.z);
        const float z = bay_stretch_z(a, u1);
        const unsigned int j = bay_partner(u0, P.K);
#pragma unroll
        for (int i = 0; i < DIM; ++i) {
            const float s = S[(size_t)i * P.W + j];
            Y[i] = __fmaf_rn(z, __fsub_rn(X[(size_t)i * P.W + k], s), s);
        }
        const float ly = BAY_LOGFN((unsigned int)P.data_len, P.params_len, P.params, DIM, Y);
        const float lx = P.logfn[(size_t)P.half * P.K + k];
        accepted = bay_accept(u2, z, ly, lx, beta);
        if (accepted) {
#pragma unroll
            for (int i = 0; i < DIM; ++i) X[(size_t)i * P.W + k] = Y[i];
            P.logfn[(size_t)P.half * P.K + k] = ly;
        } else if (ACCU) {
#pragma unroll
            for (int i = 0; i < DIM; ++i) Y[i] = X[(size_t)i * P.W + k];
        }
    }
    if (ACCU) {
        __shared__ double red[BAY_CTA / 32];
        bay_accu_epilogue(P, accepted, valid, Y, step, red);
    }
}

extern "C" __global__ void __launch_bounds__(BAY_CTA) bay_stretch_bare(bay_stretch_params P) {
    bay_stretch_plain<false>(P);
}
extern "C" __global__ void __launch_bounds__(BAY_CTA) bay_stretch_accu(bay_stretch_params P) {
    bay_stretch_plain<true>(P);
}

// logfn over all W walkers (nvidia-gtx-mcmc-stretch.cu:197-206), SoA input.
extern "C" __global__ void __launch_bounds__(BAY_CTA) bay_logfn_all(bay_stretch_params P) {
    const unsigned int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.W) return;
    float x[DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i) x[i] = P.xs[(size_t)i * P.W + k];
    P.logfn[k] = BAY_LOGFN((unsigned int)P.data_len, P.params_len, P.params, DIM, x);
}

#else
// ---------------------------------------------------------------- tiled form
// A CTA owns BAY_WPC walkers; all its threads sweep the data rows, each row read
// once per CTA and applied to every walker of the tile, with per-thread Kahan sums
// and a fixed-order (deterministic) CTA reduction.
#ifndef BAY_WPC
#define BAY_WPC 8
#endif

__device__ __forceinline__ void bay_tiled_logfn_rows(const bay_stretch_params& P,
                                                    const float (*prep)[BAY_PREP_LEN],
                                                    double (*red)[BAY_WPC], double* out) {
    const unsigned long long n_rows = P.data_len / BAY_ROW_LEN;
    float acc[BAY_WPC], cmp[BAY_WPC], pv[BAY_WPC][BAY_PREP_LEN];
#pragma unroll
    for (int w = 0; w < BAY_WPC; ++w) {
        acc[w] = 0.0f;
        cmp[w] = 0.0f;
#pragma unroll
        for (int i = 0; i < BAY_PREP_LEN; ++i) pv[w][i] = prep[w][i];
    }
    for (unsigned long long r = threadIdx.x; r < n_rows; r += blockDim.x) {
        const float* row = P.params + r * BAY_ROW_LEN;
        float rv[BAY_ROW_LEN];
#pragma unroll
        for (int c = 0; c < BAY_ROW_LEN; ++c) rv[c] = __ldg(row + c);
#pragma unroll
        for (int w = 0; w < BAY_WPC; ++w) {
            const float t = BAY_TILE_TERM(rv, pv[w]);
            // Kahan step (nvcc does not reassociate, so the compensation survives)
            const float y = __fsub_rn(t, cmp[w]);
            const float s = __fadd_rn(acc[w], y);
            cmp[w] = __fsub_rn(__fsub_rn(s, acc[w]), y);
            acc[w] = s;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int w = 0; w < BAY_WPC; ++w) {
        double v = (double)acc[w] - (double)cmp[w];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < BAY_WPC) {
        double s = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i][threadIdx.x];
        out[threadIdx.x] = s;
    }
    __syncthreads();
}

template <bool ACCU>
__device__ __forceinline__ void bay_stretch_tiled(const bay_stretch_params& P) {
    const unsigned int kind = ACCU ? 1u : 0u;
    __shared__ float sY[BAY_WPC][DIM];
    __shared__ float sPrep[BAY_WPC][BAY_PREP_LEN];
    __shared__ float sW[BAY_WPC], sZ[BAY_WPC], sU2[BAY_WPC];
    __shared__ double sRed[BAY_CTA / 32][BAY_WPC];
    __shared__ double sSum[BAY_WPC];
    __shared__ double red1[BAY_CTA / 32];
    const unsigned int step = P.ctl->step[kind] + P.step_off;
    const unsigned int seed = P.ctl->seed[kind] + P.half;
    const float a = P.ctl->a;
    const float beta = ACCU ? 1.0f : P.ctl->beta;
    const unsigned int stream = ACCU ? (P.half ? 2222u : 1111u) : (P.half ? 4444u : 3333u);
    float* X = P.xs + (size_t)P.half * P.K;
    const float* S = P.xs + (size_t)(1u - P.half) * P.K;
    const float* hyper = P.params + P.data_len;
    const unsigned int k0 = blockIdx.x * BAY_WPC;
    const unsigned long long n_rows = P.data_len / BAY_ROW_LEN;

    if (threadIdx.x < BAY_WPC) {
        const unsigned int t = threadIdx.x, k = k0 + t;
        if (k < P.K) {
            bay_u4 c;
            c.x = k;
            c.y = step;
            c.z = stream;
            c.w = 0xbeeff00du;
            const bay_u4 r = bay_philox4x32_10(c, seed, 0xdecafbadu);
            const float u0 = bay_u01(r.x), u1 = bay_u01(r.y);
            const float z = bay_stretch_z(a, u1);
            const unsigned int j = bay_partner(u0, P.K);
            float Y[DIM];
#pragma unroll
            for (int i = 0; i < DIM; ++i) {
                const float s = S[(size_t)i * P.W + j];
                Y[i] = __fmaf_rn(z, __fsub_rn(X[(size_t)i * P.W + k], s), s);
                sY[t][i] = Y[i];
            }
            float pr[BAY_PREP_LEN];
            BAY_TILE_PREP(hyper, P.params_len, DIM, Y, pr);
#pragma unroll
            for (int i = 0; i < BAY_PREP_LEN; ++i) sPrep[t][i] = pr[i];
            sW[t] = BAY_TILE_WALKER(n_rows, hyper, P.params_len, DIM, Y);
            sZ[t] = z;
            sU2[t] = bay_u01(r.z);
        } else {
#pragma unroll
            for (int i = 0; i < BAY_PREP_LEN; ++i) sPrep[t][i] = 0.0f;
            sW[t] = 0.0f;
        }
    }
    __syncthreads();
    bay_tiled_logfn_rows(P, sPrep, sRed, sSum);
    bool accepted = false;
    const unsigned int t = threadIdx.x, k = k0 + t;
    const bool valid = t < BAY_WPC && k < P.K;
    float mine[DIM];
    if (valid) {
        const float ly = (float)((double)sW[t] + sSum[t]);
        const float lx = P.logfn[(size_t)P.half * P.K + k];
        accepted = bay_accept(sU2[t], sZ[t], ly, lx, beta);
        if (accepted) {
#pragma unroll
            for (int i = 0; i < DIM; ++i) X[(size_t)i * P.W + k] = sY[t][i];
            P.logfn[(size_t)P.half * P.K + k] = ly;
        }
        if (ACCU) {
#pragma unroll
            for (int i = 0; i < DIM; ++i) mine[i] = accepted ? sY[t][i] : X[(size_t)i * P.W + k];
        }
    }
    if (ACCU) bay_accu_epilogue(P, accepted, valid, mine, step, red1);
}

extern "C" __global__ void __launch_bounds__(BAY_CTA) bay_stretch_bare(bay_stretch_params P) {
    bay_stretch_tiled<false>(P);
}
extern "C" __global__ void __launch_bounds__(BAY_CTA) bay_stretch_accu(bay_stretch_params P) {
    bay_stretch_tiled<true>(P);
}

// log density of all W walkers with the tiled sum (one CTA per BAY_WPC walkers).
extern "C" __global__ void __launch_bounds__(BAY_CTA) bay_logfn_all(bay_stretch_params P) {
    __shared__ float sPrep[BAY_WPC][BAY_PREP_LEN];
    __shared__ float sW[BAY_WPC];
    __shared__ double sRed[BAY_CTA / 32][BAY_WPC];
    __shared__ double sSum[BAY_WPC];
    const float* hyper = P.params + P.data_len;
    const unsigned long long n_rows = P.data_len / BAY_ROW_LEN;
    const unsigned int k0 = blockIdx.x * BAY_WPC;
    if (threadIdx.x < BAY_WPC) {
        const unsigned int t = threadIdx.x, k = k0 + t;
        if (k < P.W) {
            float x[DIM];
#pragma unroll
            for (int i = 0; i < DIM; ++i) x[i] = P.xs[(size_t)i * P.W + k];
            float pr[BAY_PREP_LEN];
            BAY_TILE_PREP(hyper, P.params_len, DIM, x, pr);
#pragma unroll
            for (int i = 0; i < BAY_PREP_LEN; ++i) sPrep[t][i] = pr[i];
            sW[t] = BAY_TILE_WALKER(n_rows, hyper, P.params_len, DIM, x);
        } else {
#pragma unroll
            for (int i = 0; i < BAY_PREP_LEN; ++i) sPrep[t][i] = 0.0f;
            sW[t] = 0.0f;
        }
    }
    __syncthreads();
    bay_tiled_logfn_rows(P, sPrep, sRed, sSum);
    const unsigned int t = threadIdx.x, k = k0 + t;
    if (t < BAY_WPC && k < P.W) P.logfn[k] = (float)((double)sW[t] + sSum[t]);
}
#endif
