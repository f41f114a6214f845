// bay_kernels.cu -- nvcc-compiled kernels of the stretch-move engine: walker init,
// SoA<->AoS layout changes, FP64 moments, the integer histogram with its bitonic
// ranks, acor, and the device-resident control block.  The per-model fused stretch
// kernels are in device/bay_stretch.cuh (NVRTC).
#include <atomic>

#include "bay_kernels.cuh"
#include "device/bay_rng.cuh"

namespace {

constexpr unsigned FULL = 0xffffffffu;

// Fixed-order block sum of a double (deterministic); all threads get the result.
__device__ double block_sum_d(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        red[32] = s;
    }
    __syncthreads();
    const double r = red[32];
    __syncthreads();
    return r;
}

__global__ void ctl_apply(bay_ctl* c, bay_ctl_op op) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const unsigned m = op.mask;
    if (m & BAY_CTL_SET_STEP0) c->step[0] = op.step[0];
    if (m & BAY_CTL_SET_STEP1) c->step[1] = op.step[1];
    if (m & BAY_CTL_ADD_STEP0) c->step[0] += op.step[0];
    if (m & BAY_CTL_ADD_STEP1) c->step[1] += op.step[1];
    if (m & BAY_CTL_SET_SEED0) c->seed[0] = op.seed[0];
    if (m & BAY_CTL_SET_SEED1) c->seed[1] = op.seed[1];
    if (m & BAY_CTL_SET_A) c->a = op.a;
    if (m & BAY_CTL_SET_BETA) c->beta = op.beta;
    if (m & BAY_CTL_RESET_ACCEPTED) c->accepted = 0ull;
    if (m & BAY_CTL_RESET_TICKETS) {
        c->ticket[0] = 0u;
        c->ticket[1] = 0u;
    }
}

// mix!'s a-adaptation probes (mcmc.clj:84-91): init-move! before the probe's accu step,
// the loop's rule after it.  The rule runs in FP64 with explicit IEEE operations (no fused
// multiply-add), so a follows the same sequence as the host loop.
__global__ void mix_begin(bay_ctl* c, const bay_mix_state* st) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    c->seed[1] += 2u;
    c->step[1] = 0u;
    c->a = (float)st->a;
    c->accepted = 0ull;
    c->ticket[0] = 0u;
    c->ticket[1] = 0u;
}

__global__ void mix_end(bay_ctl* c, bay_mix_state* st, unsigned long long W, unsigned int step,
                        double min_acc, double max_acc, cudaGraphConditionalHandle cont) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    c->step[1] += 1u;                                   // the probe's one accu step
    const double r = __ddiv_rn((double)c->accepted, (double)W);
    const double target = __ddiv_rn(__dadd_rn(max_acc, min_acc), 2.0);
    st->rate = r;
    st->probes += 1u;
    unsigned int go = 0u;
    if (!(step < st->i)) {
        if (r < min_acc) {
            st->a = __dadd_rn(1.0, __dmul_rn(__dsub_rn(st->a, 1.0), __ddiv_rn(r, target)));
            go = 1u;
        } else if (max_acc < r) {
            st->a = __dmul_rn(st->a, __ddiv_rn(r, target));
            go = 1u;
        }
        if (go) st->i += 1u;
        if (go && !((float)st->a > 1.0f)) {
            st->bad = 1u;
            go = 0u;
        }
    }
    cudaGraphSetConditional(cont, go);
}

// init_walkers (nvidia-gtx-mcmc-stretch.cu:158-195): element e = w*D + d (the
// reference's AoS index) takes word e%4 of Philox(ctr {e/4, 0xf00dcafe, 0xdeadbeef,
// 0xbeeff00d}, key {seed, 0xdecafaaa}); x = u*hi + (1-u)*lo, first product fused.
// The walker state is walker-major, so element e is written at xs[e] (coalesced).
__global__ void init_uniform(float* xs, uint32_t D, uint64_t W, uint32_t seed,
                             const float* limits) {
    const uint64_t n = (uint64_t)D * W;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t d = e % D;
        bay_u4 c;
        c.x = (unsigned)(e >> 2);
        c.y = 0xf00dcafeu;
        c.z = 0xdeadbeefu;
        c.w = 0xbeeff00du;
        const bay_u4 r = bay_philox4x32_10(c, seed, 0xdecafaaau);
        const unsigned word = (e & 3) == 0 ? r.x : (e & 3) == 1 ? r.y : (e & 3) == 2 ? r.z : r.w;
        const float u = bay_u01(word);
        const float lo = limits[2 * d], hi = limits[2 * d + 1];
        xs[e] = __fmaf_rn(u, hi, __fmul_rn(__fsub_rn(1.0f, u), lo));
    }
}

// N(mean, sd^2) init: element e = w*D + d uses pair p = e/2, Philox(ctr {p, 0x6e6f726d,
// 0x77616c6b, 0xbeeff00d}, key {seed, 0x9a55a9e5}); Box-Muller in FP64 on words 0, 1.
__global__ void init_normal(float* xs, uint32_t D, uint64_t W, uint32_t seed, float mean,
                            float sd) {
    const uint64_t n = (uint64_t)D * W;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < n;
         e += (uint64_t)gridDim.x * blockDim.x) {
        bay_u4 c;
        c.x = (unsigned)(e >> 1);
        c.y = 0x6e6f726du;
        c.z = 0x77616c6bu;
        c.w = 0xbeeff00du;
        const bay_u4 r = bay_philox4x32_10(c, seed, 0x9a55a9e5u);
        const double rr = sqrt(-2.0 * log((double)bay_u01(r.y)));
        const double t = 6.283185307179586 * (double)bay_u01(r.x);
        const double z = (e & 1) ? rr * sin(t) : rr * cos(t);
        xs[e] = (float)((double)mean + (double)sd * z);
    }
}

// 32x32 tiled transposes between SoA (D rows of W) and AoS (W rows of D).
__global__ void soa_to_aos(const float* xs, uint32_t D, uint64_t W, uint64_t w0, uint64_t nw,
                           float* out) {
    __shared__ float tile[32][33];
    const uint64_t wb = w0 + (uint64_t)blockIdx.x * 32;
    const uint32_t db = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const uint32_t d = db + r;
        const uint64_t w = wb + threadIdx.x;
        if (d < D && w < w0 + nw) tile[r][threadIdx.x] = xs[(uint64_t)d * W + w];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const uint64_t w = wb + r;
        const uint32_t d = db + threadIdx.x;
        if (d < D && w < w0 + nw) out[(w - w0) * D + d] = tile[threadIdx.x][r];
    }
}

__global__ void aos_to_soa(const float* in, uint32_t D, uint64_t W, float* xs) {
    __shared__ float tile[32][33];
    const uint64_t wb = (uint64_t)blockIdx.x * 32;
    const uint32_t db = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const uint64_t w = wb + r;
        const uint32_t d = db + threadIdx.x;
        if (d < D && w < W) tile[r][threadIdx.x] = in[w * D + d];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const uint32_t d = db + r;
        const uint64_t w = wb + threadIdx.x;
        if (d < D && w < W) xs[(uint64_t)d * W + w] = tile[threadIdx.x][r];
    }
}

// One CTA per dim: FP64 mean, then FP64 sum of squared deviations (population variance).
__global__ void moments(const float* xs, uint32_t D, uint64_t W, double* mean, double* var) {
    __shared__ double red[33];
    const uint32_t d = blockIdx.x;
    const float* row = xs + (uint64_t)d * W;
    double s = 0.0;
    for (uint64_t w = threadIdx.x; w < W; w += blockDim.x) s += (double)row[w];
    const double mu = block_sum_d(s, red) / (double)W;
    double q = 0.0;
    for (uint64_t w = threadIdx.x; w < W; w += blockDim.x) {
        const double t = (double)row[w] - mu;
        q += t * t;
    }
    const double v = block_sum_d(q, red) / (double)W;
    if (threadIdx.x == 0) {
        if (mean) mean[d] = mu;
        if (var) var[d] = v;
    }
}

__global__ void minmax(const float* xs, uint32_t D, uint64_t W, int zero_fold, float* limits) {
    __shared__ float smn[32], smx[32];
    const uint32_t d = blockIdx.x;
    const float* row = xs + (uint64_t)d * W;
    float mn = row[0], mx = row[0];
    for (uint64_t w = threadIdx.x; w < W; w += blockDim.x) {
        mn = fminf(mn, row[w]);
        mx = fmaxf(mx, row[w]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_down_sync(FULL, mn, o));
        mx = fmaxf(mx, __shfl_down_sync(FULL, mx, o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        smn[warp] = mn;
        smx[warp] = mx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            mn = fminf(mn, smn[w]);
            mx = fmaxf(mx, smx[w]);
        }
        if (zero_fold) {
            mn = fminf(mn, 0.0f);
            mx = fmaxf(mx, 0.0f);
        }
        limits[2 * d] = mn;
        limits[2 * d + 1] = mx;
    }
}

// histogram (nvidia-gtx-estimate.cu:5-32): bin = (uint)((x - lo)/(hi - lo) * bins) with
// IEEE division and the saturating float->uint conversion, clamped to bins - 1.
// Shared-memory counts per CTA, one global atomic per non-empty bin.
__global__ void hist_count(const float* xs, uint32_t D, uint64_t W, uint32_t bins,
                           const float* limits, uint32_t* counts) {
    extern __shared__ uint32_t h[];
    const uint32_t d = blockIdx.y;
    for (uint32_t b = threadIdx.x; b < bins; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const float lo = limits[2 * d], hi = limits[2 * d + 1];
    const float range = __fsub_rn(hi, lo);
    const float fb = (float)bins;
    const float* row = xs + (uint64_t)d * W;
    for (uint64_t w = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; w < W;
         w += (uint64_t)gridDim.x * blockDim.x) {
        const float v = __fmul_rn(__fdiv_rn(__fsub_rn(row[w], lo), range), fb);
        uint32_t b = __float2uint_rz(v);
        b = b < bins ? b : bins - 1;
        atomicAdd(&h[b], 1u);
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < bins; b += blockDim.x)
        if (h[b]) atomicAdd(&counts[(uint64_t)d * bins + b], h[b]);
}

// uint_to_real (nvidia-gtx-estimate.cu:34-44) and bitonic_local (:117-147): the
// reference's compare-exchange network over (bin, pdf) pairs, decreasing pdf; equal
// pdfs count as "smaller" when the partner position j is below lid.
__global__ void hist_finish(const uint32_t* counts, const float* limits, uint32_t bins,
                            float alpha, float* pdf, float* ranks) {
    extern __shared__ float2 aux[];
    const uint32_t d = blockIdx.x, lid = threadIdx.x;
    const float c = __fdiv_rn(alpha, __fsub_rn(limits[2 * d + 1], limits[2 * d]));
    const float p = __fmul_rn(c, (float)counts[(uint64_t)d * bins + lid]);
    pdf[(uint64_t)d * bins + lid] = p;
    float2 v = make_float2((float)lid, p);
    aux[lid] = v;
    __syncthreads();
    for (uint32_t length = 1; length < bins; length <<= 1) {
        const bool direction = (lid & (length << 1)) != 0;
        for (uint32_t inc = length; inc > 0; inc >>= 1) {
            const uint32_t j = lid ^ inc;
            const float2 o = aux[j];
            const bool smaller = (v.y < o.y) || (o.y == v.y && j < lid);
            const bool swap = smaller ^ (j < lid) ^ direction;
            v = swap ? o : v;
            __syncthreads();
            aux[lid] = v;
            __syncthreads();
        }
    }
    ranks[(uint64_t)d * bins + lid] = v.x;
}

// One CTA per (step, dim): the 2 x G per-CTA sums part[((t*2 + h)*D + d)*G + b] read
// coalesced along b, summed in FP64 in a fixed order.
__global__ void reduce_means(const bay_ctl* ctl, const float* part, float* means,
                             uint32_t means_cap, uint32_t G, uint32_t D, double inv_W) {
    __shared__ double red[33];
    const uint32_t t = blockIdx.x, d = blockIdx.y;
    const uint32_t step = ctl->step[1] + t;
    double s = 0.0;
    for (uint32_t h = 0; h < 2; ++h) {
        const float* p = part + (((size_t)t * 2 + h) * D + d) * G;
        for (uint32_t b = threadIdx.x; b < G; b += blockDim.x) s += (double)p[b];
    }
    s = block_sum_d(s, red);
    if (threadIdx.x == 0 && step < means_cap) means[(size_t)step * D + d] = (float)(s * inv_W);
}

// The GEMM form's matrix laid out once per sampler: lay[f*NP + r] = A[r][f] (rows past
// `rows` zero), then lay[F*NP + r*auxs + c] = A[r][aux_col + c].
__global__ void gemm_layout(const float* A, uint64_t ld, uint32_t rows, uint32_t F, uint32_t NP,
                            uint32_t aux_col, uint32_t aux_len, uint32_t auxs, float* lay) {
    const uint64_t nA = (uint64_t)F * NP;
    const uint64_t n = nA + (uint64_t)NP * auxs;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        float v = 0.0f;
        if (i < nA) {
            const uint64_t f = i / NP, r = i % NP;
            if (r < rows) v = A[r * ld + f];
        } else {
            const uint64_t e = i - nA, r = e / auxs, c = e % auxs;
            if (r < rows && c < aux_len) v = A[r * ld + aux_col + c];
        }
        lay[i] = v;
    }
}

// bf16 of a float rounded to nearest even, as its 16 bits (NaN stays a quiet NaN)
__device__ __forceinline__ unsigned short bf16_rn(float x) {
    unsigned int u = __float_as_uint(x);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (unsigned short)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (unsigned short)(u >> 16);
}

// Tensor-core GEMM form: the matrix as bf16 hi + lo, row-major [rows_pad][Fp] (features
// past F and rows past `rows` zero), and the rows' aux values [rows_pad][auxs].
__global__ void gemm_split(const float* A, uint64_t ld, uint32_t rows, uint32_t F, uint32_t Fp,
                           uint64_t rows_pad, uint32_t aux_col, uint32_t aux_len, uint32_t auxs,
                           unsigned short* hi, unsigned short* lo, float* aux) {
    const uint64_t nA = rows_pad * Fp, n = nA + rows_pad * auxs;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (i < nA) {
            const uint64_t r = i / Fp, f = i % Fp;
            const float v = (r < rows && f < F) ? A[r * ld + f] : 0.0f;
            const unsigned short h = bf16_rn(v);
            hi[i] = h;
            lo[i] = bf16_rn(__fsub_rn(v, __uint_as_float((unsigned int)h << 16)));
        } else {
            const uint64_t e = i - nA, r = e / auxs, c = e % auxs;
            aux[e] = (r < rows && c < aux_len) ? A[r * ld + aux_col + c] : 0.0f;
        }
    }
}

// Resident tensor-core GEMM form: the matrix as the MMA's B operand -- bf16 hi atoms then
// lo atoms, each atom [NP rows][64 features] in 128-byte rows with 16-byte unit u of row r
// stored at unit u ^ (r % 8) -- followed by the rows' aux values [NP][auxs]; rows past
// `rows` and features past F are zero.
__global__ void gemm_tc_image(const float* A, uint64_t ld, uint32_t rows, uint32_t F, uint32_t KC,
                              uint32_t NP, uint32_t aux_col, uint32_t aux_len, uint32_t auxs,
                              unsigned char* img) {
    const uint64_t n_units = (uint64_t)KC * NP * 8;      // 16-byte units per hi (or lo) block
    const uint64_t n = n_units + (uint64_t)NP * auxs;
    const uint64_t lo_off = n_units * 16;
    float* aux = reinterpret_cast<float*>(img + 2 * lo_off);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        if (i < n_units) {
            const uint32_t c = (uint32_t)(i / ((uint64_t)NP * 8));
            const uint32_t rem = (uint32_t)(i - (uint64_t)c * NP * 8);
            const uint32_t r = rem >> 3, u = rem & 7u;
            unsigned int hw[4], lw[4];
            for (int q = 0; q < 4; ++q) {
                unsigned int hh[2], ll[2];
                for (int j = 0; j < 2; ++j) {
                    const uint32_t f = c * 64u + u * 8u + 2u * q + j;
                    const float v = (r < rows && f < F) ? A[(uint64_t)r * ld + f] : 0.0f;
                    const unsigned short h = bf16_rn(v);
                    hh[j] = h;
                    ll[j] = bf16_rn(__fsub_rn(v, __uint_as_float((unsigned int)h << 16)));
                }
                hw[q] = hh[0] | (hh[1] << 16);
                lw[q] = ll[0] | (ll[1] << 16);
            }
            const uint64_t off = (uint64_t)c * NP * 128 + (uint64_t)r * 128 + ((u ^ (r & 7u)) << 4);
            *reinterpret_cast<uint4*>(img + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
            *reinterpret_cast<uint4*>(img + lo_off + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        } else {
            const uint64_t e = i - n_units, r = e / auxs, cc = e % auxs;
            aux[e] = (r < rows && cc < aux_len) ? A[r * ld + aux_col + cc] : 0.0f;
        }
    }
}

__global__ void fill_u32(uint32_t* p, uint32_t v, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

__global__ void fill_bytes(uint4* p, uint64_t n16, unsigned int v) {
    const uint4 q = make_uint4(v, v, v, v);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n16;
         i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = q;
}

// One acor pass (nvidia-gtx-acor.cu:40-103) in FP64: x_t = m[t*stride] for t + lag < n;
// the lag window of t reads x (zeroed past n - lag) inside t's block of B = min(wgs, n)
// entries and raw m across the block edge, as the reference's shared-memory window does.
__device__ void acor_pass(const double* m, uint64_t stride, uint32_t n, uint32_t wgs,
                          uint32_t lag, double* red, double* c0_out, double* d_out) {
    const uint32_t B = wgs < n ? wgs : n;
    double c0 = 0.0, dd = 0.0;
    for (uint32_t t = threadIdx.x; t + lag < n; t += blockDim.x) {
        const double x = m[(uint64_t)t * stride];
        const uint32_t blk_end = (t / B + 1) * B;
        double acc = 0.0;
        for (uint32_t s = 1; s <= lag; ++s) {
            const uint32_t u = t + s;
            double v;
            if (u < blk_end) v = (u + lag < n) ? m[(uint64_t)u * stride] : 0.0;
            else v = m[(uint64_t)u * stride];
            acc += v;
        }
        c0 += x * x;
        dd += x * (x + 2.0 * acc);
    }
    const double C0 = block_sum_d(c0, red);
    const double DD = block_sum_d(dd, red);
    *c0_out = C0;
    *d_out = DD;
}

// acor (nvidia-gtx-acor.cu:116-168 + nvidia_gtx.clj:240-278) for one dim per CTA, with
// no dynamic parallelism: mean, centring, the first pass, then pairwise halving while
// 10 < lag2 and lag2 < 5 tau; tau = D (n - lag) / (stride (n2 - lag2) C0_first),
// sigma = sqrt(D / (stride (n2 - lag2) n)).
__global__ void acor_kernel(const float* series, uint32_t D, uint32_t n, uint32_t wgs,
                            uint32_t lag, double* work, double* tau_out, double* mean_out,
                            double* sigma_out) {
    __shared__ double red[33];
    const uint32_t d = blockIdx.x;
    double* m = work + (uint64_t)d * n;
    double s = 0.0;
    for (uint32_t t = threadIdx.x; t < n; t += blockDim.x) s += (double)series[(uint64_t)t * D + d];
    const double mu = block_sum_d(s, red) / (double)n;
    for (uint32_t t = threadIdx.x; t < n; t += blockDim.x)
        m[t] = (double)series[(uint64_t)t * D + d] - mu;
    __syncthreads();
    double c0a, da;
    acor_pass(m, 1, n, wgs, lag, red, &c0a, &da);
    const double c0 = c0a;
    double tau = da / c0;
    uint32_t lag2 = lag, n2 = n, stride = 1;
    while (10u < lag2 && (double)lag2 < tau * 5.0) {
        n2 /= 2;
        lag2 = (lag * 5u < n2) ? lag : ((n2 / 5u) > 10u ? n2 / 5u : 10u);
        const double c0prev = c0a;
        __syncthreads();
        for (uint32_t g = threadIdx.x; g < n2; g += blockDim.x)
            m[(uint64_t)2 * g * stride] += m[(uint64_t)(2 * g + 1) * stride];
        __syncthreads();
        stride *= 2;
        acor_pass(m, stride, n2, wgs, lag2, red, &c0a, &da);
        tau = da / c0prev;
    }
    if (threadIdx.x == 0) {
        const double scale = (double)stride * (double)(n2 - lag2);
        tau_out[d] = da * (double)(n - lag) / (scale * c0);
        mean_out[d] = mu;
        sigma_out[d] = sqrt(da / (scale * (double)n));
    }
}

// Fixed device scratch of the allocation-free acor entry point: the work copy of the
// series (dim * n doubles) followed by tau, mean and sigma (3 * dim doubles).  It is
// part of the module image, so every GPU that loads the library holds these 8 MiB
// until the process exits.  acor_kernel writes every slot it later reads, so nothing
// has to be cleared between calls; calls that overlap on the GPU share it and race.
__device__ __align__(256) double g_acor_noalloc_scratch[BAY_ACOR_NOALLOC_MAX_DOUBLES];

inline unsigned grid_for(uint64_t n, unsigned block, unsigned cap = 152u * 16u) {
    uint64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    return (unsigned)(g < cap ? g : cap);
}

}  // namespace

namespace bay {

std::atomic<unsigned long long> g_launches{0};

unsigned long long launch_count() { return g_launches.load(); }
void count_launches(unsigned long long n) { g_launches += n; }

cudaError_t launch_ctl_apply(bay_ctl* ctl, const bay_ctl_op& op, cudaStream_t s) {
    ctl_apply<<<1, 1, 0, s>>>(ctl, op);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_mix_begin(bay_ctl* ctl, bay_mix_state* st, cudaStream_t s) {
    mix_begin<<<1, 32, 0, s>>>(ctl, st);
    return cudaGetLastError();
}

cudaError_t launch_mix_end(bay_ctl* ctl, bay_mix_state* st, unsigned long long W, unsigned int step,
                           double min_acc, double max_acc, cudaGraphConditionalHandle cont,
                           cudaStream_t s) {
    mix_end<<<1, 32, 0, s>>>(ctl, st, W, step, min_acc, max_acc, cont);
    return cudaGetLastError();
}

cudaError_t launch_init_uniform(float* xs, uint32_t D, uint64_t W, uint32_t seed,
                                const float* limits, cudaStream_t s) {
    init_uniform<<<grid_for((uint64_t)D * W, 256), 256, 0, s>>>(xs, D, W, seed, limits);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_init_normal(float* xs, uint32_t D, uint64_t W, uint32_t seed, float mean,
                               float sd, cudaStream_t s) {
    init_normal<<<grid_for((uint64_t)D * W, 256), 256, 0, s>>>(xs, D, W, seed, mean, sd);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(const float* xs, uint32_t D, uint64_t W, uint64_t w0, uint64_t n,
                              float* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    dim3 grid((unsigned)((n + 31) / 32), (D + 31) / 32), block(32, 8);
    soa_to_aos<<<grid, block, 0, s>>>(xs, D, W, w0, n, out);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_aos_to_soa(const float* in, uint32_t D, uint64_t W, float* xs, cudaStream_t s) {
    dim3 grid((unsigned)((W + 31) / 32), (D + 31) / 32), block(32, 8);
    aos_to_soa<<<grid, block, 0, s>>>(in, D, W, xs);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_moments(const float* xs, uint32_t D, uint64_t W, double* mean, double* var,
                           cudaStream_t s) {
    moments<<<D, 512, 0, s>>>(xs, D, W, mean, var);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_minmax(const float* xs, uint32_t D, uint64_t W, int zero_fold, float* limits,
                          cudaStream_t s) {
    minmax<<<D, 512, 0, s>>>(xs, D, W, zero_fold, limits);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_hist_count(const float* xs, uint32_t D, uint64_t W, uint32_t bins,
                              const float* limits, uint32_t* counts, cudaStream_t s) {
    unsigned gx = grid_for(W, 256, 64);
    dim3 grid(gx, D);
    hist_count<<<grid, 256, bins * sizeof(uint32_t), s>>>(xs, D, W, bins, limits, counts);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_hist_finish(const uint32_t* counts, const float* limits, uint32_t D,
                               uint32_t bins, uint64_t n, float* pdf, float* ranks,
                               cudaStream_t s) {
    const float alpha = (float)((double)bins / (double)n);
    hist_finish<<<D, bins, bins * sizeof(float2), s>>>(counts, limits, bins, alpha, pdf, ranks);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_reduce_means(const bay_ctl* ctl, const float* part, float* means,
                                uint32_t means_cap, uint32_t G, uint32_t D, uint32_t nsteps,
                                double inv_W, cudaStream_t s) {
    if (nsteps == 0) return cudaSuccess;
    dim3 grid(nsteps, D);
    reduce_means<<<grid, 128, 0, s>>>(ctl, part, means, means_cap, G, D, inv_W);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_gemm_layout(const float* A, uint64_t ld, uint32_t rows, uint32_t F, uint32_t NP,
                               uint32_t aux_col, uint32_t aux_len, uint32_t auxs, float* lay,
                               cudaStream_t s) {
    const uint64_t n = (uint64_t)F * NP + (uint64_t)NP * auxs;
    gemm_layout<<<grid_for(n, 256), 256, 0, s>>>(A, ld, rows, F, NP, aux_col, aux_len, auxs, lay);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_gemm_split(const float* A, uint64_t ld, uint32_t rows, uint32_t F, uint32_t Fp,
                              uint64_t rows_pad, uint32_t aux_col, uint32_t aux_len, uint32_t auxs,
                              unsigned short* hi, unsigned short* lo, float* aux, cudaStream_t s) {
    const uint64_t n = rows_pad * Fp + rows_pad * auxs;
    gemm_split<<<grid_for(n, 256), 256, 0, s>>>(A, ld, rows, F, Fp, rows_pad, aux_col, aux_len, auxs,
                                                 hi, lo, aux);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_gemm_tc_image(const float* A, uint64_t ld, uint32_t rows, uint32_t F,
                                 uint32_t KC, uint32_t NP, uint32_t aux_col, uint32_t aux_len,
                                 uint32_t auxs, void* img, cudaStream_t s) {
    const uint64_t n = (uint64_t)KC * NP * 8 + (uint64_t)NP * auxs;
    gemm_tc_image<<<grid_for(n, 256), 256, 0, s>>>(A, ld, rows, F, KC, NP, aux_col, aux_len, auxs,
                                                    static_cast<unsigned char*>(img));
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_fill_u32(uint32_t* p, uint32_t v, uint64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    fill_u32<<<grid_for(n, 256), 256, 0, s>>>(p, v, n);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t launch_acor(const float* series, uint32_t D, uint32_t n, uint32_t wgs, uint32_t lag,
                        double* work, double* tau, double* mean, double* sigma, cudaStream_t s) {
    acor_kernel<<<D, 256, 0, s>>>(series, D, n, wgs, lag, work, tau, mean, sigma);
    g_launches++;
    return cudaGetLastError();
}

cudaError_t acor_noalloc_scratch(double** ptr) {
    // In host code g_acor_noalloc_scratch names a host-side stand-in, not the array: its
    // device address comes from cudaGetSymbolAddress, with the device current.
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_acor_noalloc_scratch);
    if (e != cudaSuccess) return e;
    *ptr = static_cast<double*>(p);
    return cudaSuccess;
}

cudaError_t launch_fill_bytes(void* p, uint64_t n, unsigned char v, cudaStream_t s) {
    const unsigned int w = 0x01010101u * v;
    const uint64_t n16 = n / 16;
    fill_bytes<<<grid_for(n16, 512, 152u * 8u), 512, 0, s>>>((uint4*)p, n16, w);
    g_launches++;
    return cudaGetLastError();
}

}  // namespace bay
