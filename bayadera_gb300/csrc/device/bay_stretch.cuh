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
// Layout (all forms): positions walker-major, xs[w * DIM + d] (W walkers,
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
//                  formula); 0 (default): log u <= (D-1) log z + beta dl in fp32 with
//                  the deterministic logarithm bay_log_det (bay_accept_log).
//   BAY_STRETCH_REF 1: the stretch factor's 1/a by the compiler's fast division (the
//                  reference's build flavour, -use_fast_math); 0 (default): IEEE 1/a.
//                  Both keep the operation order the golden trajectories pin.
//   BAY_PARTNER_ELEMENT 1 (plain and tiled forms): the reference's partner offset
//                  (uint)(u0 K DIM), an element offset that straddles walkers for
//                  DIM > 1; elements past the half's end read as 0.  0 (default): the
//                  partner is walker (uint)(u0 K), clamped to the half.

#ifndef BAY_CTA
#define BAY_CTA 256
#endif
#ifndef BAY_ACCEPT_REF
#define BAY_ACCEPT_REF 0
#endif
#ifndef BAY_TILED
#define BAY_TILED 0
#endif
#ifndef BAY_STRETCH_REF
#define BAY_STRETCH_REF 0
#endif
#ifndef BAY_PARTNER_ELEMENT
#define BAY_PARTNER_ELEMENT 0
#endif
#ifndef BAY_GEMM
#define BAY_GEMM 0
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
    unsigned int pad0[21];
    unsigned int gbar_count;        // grid barrier of the persistent form (byte 128): arrivals
    unsigned int pad1[31];
    unsigned int abort;             //   abandon flag (byte 256); both cleared before each launch
    unsigned int pad2[31];
};

struct bay_stretch_params {
    const float* params;            // data || hyperparameters
    float* xs;                      // positions, walker-major xs[w * DIM + d]
    float* logfn;                   // W log densities
    bay_ctl* ctl;
    float* part;                    // accu: per-CTA sums [step_off][half][DIM][cta]
    float* means;                   // unused by the stretch kernels (reduce_means writes it)
    unsigned long long data_len;    // floats of data in params
    unsigned int params_len;        // hyperparameters after the data
    unsigned int W, K;
    unsigned int half;
    unsigned int step_off;          // added to the device step counter
    unsigned int means_cap;         // steps the means buffer holds
    float inv_W;
    // GEMM form: matrix rows at params + gemm_base + r * gemm_ld, r < gemm_rows; the
    // sampler's copy laid out for the kernel: gemm_lay = [F][NP] feature-major, rows
    // zero-padded to NP (a multiple of 64), then [NP][aux] row-major
    unsigned long long gemm_base;
    unsigned long long gemm_rows;
    unsigned int gemm_ld;
    unsigned int gemm_np;
    const float* gemm_lay;
    // GEMM form, streaming (too many rows for shared memory): one half-step's per-walker
    // scratch and the per-row-block partial sums
    float* s_y;                     // [nk][DIM] proposals (current positions for logfn)
    float* s_b;                     // [nk][F] coefficient block
    float* s_prep;                  // [nk][BAY_PREP_LEN]
    float* s_w;                     // [nk] terms outside the row sum
    float* s_zu;                    // [nk][2] stretch factor and accept uniform
    float* s_part;                  // [nsb][nk] compensated (hi, lo) partial row sums
    unsigned int s_nsb;             // row super-blocks
    unsigned int s_sbrows;          // rows per super-block (a multiple of 128)
    // GEMM form on the tensor cores: the coefficient block split into bf16 hi + lo,
    // [walker][tc_fp] each (tc_fp = F rounded up to 64; padding columns stay zero)
    unsigned short* s_bh;
    unsigned short* s_bl;
    unsigned int tc_fp;
    unsigned int gbar_extra;        // persistent form: arrivals its grid barriers wait for beyond
                                    // the grid (0; 1 makes them run out, for tests)
    // data-tiled form split into t_slices row slices per walker group (1: none): each
    // slice's CTA leaves its walkers' partial sums in t_part[k][slice] (hi, lo) and takes a
    // ticket in t_ticket[group]; the last one combines them in slice order and decides
    unsigned int t_slices;
    unsigned int pad_t;
    float* t_part;
    unsigned int* t_ticket;
};

__device__ __forceinline__ float bay_stretch_z(float a, float u1) {
    // z = (a - 2 + 1/a) u1^2 + 2 (1 - 1/a) u1 + 1/a with the first product fused and
    // every other operation rounded on its own: the order the reference's golden
    // trajectories pin (the current compiler contracts the reference's spelling of the
    // expression, nvidia-gtx-mcmc-stretch.cu:71-72, differently).  1/a is IEEE by default;
    // BAY_STRETCH_REF takes the reference build's flavour, the compiler's fast division
    // (this module is compiled with -use_fast_math, as the reference's is).
#if BAY_STRETCH_REF
    const float inv_a = 1.0f / a;
#else
    const float inv_a = __fdiv_rn(1.0f, a);
#endif
    const float c1 = __fadd_rn(__fsub_rn(a, 2.0f), inv_a);
    const float c2 = __fmul_rn(2.0f, __fsub_rn(1.0f, inv_a));
    return __fadd_rn(__fmaf_rn(__fmul_rn(c1, u1), u1, __fmul_rn(c2, u1)), inv_a);
}

__device__ __forceinline__ unsigned int bay_partner(float u0, unsigned int K) {
#if BAY_PARTNER_ELEMENT
    // the reference's element offset (uint)(u0 * K * DIM), two fp32 products
    return __float2uint_rz(__fmul_rn(__fmul_rn(u0, (float)K), (float)DIM));
#else
    // Walker j = (uint)(u0 * K) of the complementary half; u0 < 1 can still round
    // u0*K up to K, so clamp (the reference would read past the half there).
    unsigned int j = __float2uint_rz(__fmul_rn(u0, (float)K));
    return j < K ? j : K - 1;
#endif
}

// Coordinate i of the partner j (bay_partner) in the complementary half S of K walkers.
__device__ __forceinline__ float bay_partner_coord(const float* S, unsigned int K, unsigned int j,
                                                   unsigned int i) {
#if BAY_PARTNER_ELEMENT
    // an element offset: past the half's last element the reference reads out of bounds
    // (or the moving half, racing with its writes); here those elements read as 0
    const unsigned long long e = (unsigned long long)j + i;
    return e < (unsigned long long)K * DIM ? S[e] : 0.0f;
#else
    return S[(size_t)j * DIM + i];
#endif
}

__device__ __forceinline__ bool bay_accept(float u2, float z, float ly, float lx, float beta) {
#if BAY_ACCEPT_REF
    const float q = isfinite(ly) ? powf(z, (float)(DIM - 1)) * expf(beta * (ly - lx)) : 0.0f;
    return u2 <= q;
#else
    return bay_accept_log(u2, z, ly, lx, beta, DIM - 1);
#endif
}

// Compensated fp32 pairs (hi, lo), hi + lo the value: sums carried without FP64 (FP64
// issue is a small fraction of FP32 on this part).  bay_cadd is symmetric in its
// arguments (TwoSum of the highs, then the lows), so an xor-butterfly of it leaves the
// same bits in every lane: the combine order is fixed and the result deterministic.
struct bay_cf {
    float hi, lo;
};
__device__ __forceinline__ bay_cf bay_cadd(bay_cf a, bay_cf b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    const float lo = __fadd_rn(__fadd_rn(a.lo, b.lo), e);
    const float hi = __fadd_rn(s, lo);
    bay_cf r;
    r.hi = hi;
    r.lo = __fsub_rn(lo, __fsub_rn(hi, s));
    return r;
}
__device__ __forceinline__ bay_cf bay_cf_shfl_xor(bay_cf v, int o) {
    bay_cf r;
    r.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
    r.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
    return r;
}
// a + (s.hi + s.lo), rounded once to fp32
__device__ __forceinline__ float bay_cf_total(float a, bay_cf s) {
    bay_cf t;
    t.hi = a;
    t.lo = 0.0f;
    t = bay_cadd(t, s);
    return __fadd_rn(t.hi, t.lo);
}

// Accu epilogue: the CTA's accept count (one 64-bit atomic, integer: deterministic) and,
// when per-step means are wanted, the CTA's per-dim sums of the moved half: fp32 warp
// shuffles, per-warp sums staged in shared memory (one barrier per 64 dims), combined
// across warps with compensated fp32 in warp order, stored to part[(step_off*2 + half)][dim][cta].  The
// per-step ensemble means are reduced from these partials by a separate kernel.
#define BAY_SUM_CHUNK 64
__device__ void bay_accu_epilogue(const bay_stretch_params& P, bool accepted, bool valid,
                                  const float* mine, float (*red)[BAY_SUM_CHUNK],
                                  unsigned int slot, unsigned int nslots) {
    const int n_acc = __syncthreads_count(accepted);
    if (threadIdx.x == 0 && n_acc) atomicAdd(&P.ctl->accepted, (unsigned long long)n_acc);
    if (P.means_cap == 0) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    float* out = P.part + ((size_t)P.step_off * 2 + P.half) * DIM * nslots + slot;
#pragma unroll
    for (int d0 = 0; d0 < DIM; d0 += BAY_SUM_CHUNK) {
#pragma unroll
        for (int d = d0; d < DIM && d < d0 + BAY_SUM_CHUNK; ++d) {
            float v = valid ? mine[d] : 0.0f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) red[warp][d - d0] = v;
        }
        __syncthreads();
        const int nd = (DIM - d0) < BAY_SUM_CHUNK ? (DIM - d0) : BAY_SUM_CHUNK;
        for (int d = threadIdx.x; d < nd; d += blockDim.x) {
            bay_cf s;
            s.hi = 0.0f;
            s.lo = 0.0f;
            for (int w = 0; w < nwarps; ++w) {
                bay_cf y;
                y.hi = red[w][d];
                y.lo = 0.0f;
                s = bay_cadd(s, y);
            }
            out[(size_t)(d0 + d) * nslots] = __fadd_rn(s.hi, s.lo);
        }
        __syncthreads();
    }
}

#if BAY_GEMM
// ---------------------------------------------------------------- GEMM form
// log density = BAY_GEMM_WALKER(rows, hyper, hyper_len, dim, x)
//             + sum_r BAY_GEMM_TERM(eta_r, aux_r, r, x, prep),   eta = A x[COEF : COEF+F],
// A = the rows x F matrix at params + gemm_base (row stride gemm_ld; aux values of row r
// at column BAY_GEMM_AUXCOL).  A CTA owns BAY_WT walkers.  The matrix (feature-major,
// rows padded to 64) and the proposal tile are staged in shared memory once; each of
// the 256 threads accumulates a 4-walker x 4-row register tile over the F features (two
// 16-byte shared loads per 16 FMAs), applies the row term with a Kahan sum, and the 16
// row-group lanes of a walker combine as compensated fp32 pairs in a fixed xor order.
#define BAY_WT 64
#define BAY_RW 4
#define BAY_RN 4
#define BAY_NG 16
#define BAY_ROWS_PER_PASS (BAY_NG * BAY_RN)
#define BAY_DPAD (DIM | 1)
#ifndef BAY_GEMM_AUX
#define BAY_GEMM_AUX 0
#endif
#define BAY_AUXS (BAY_GEMM_AUX > 0 ? BAY_GEMM_AUX : 1)

template <bool ACCU, bool LOGFN_ONLY>
__device__ __forceinline__ void bay_stretch_gemm(const bay_stretch_params& P) {
    extern __shared__ __align__(128) float bay_smem[];
    const unsigned int rows = (unsigned int)P.gemm_rows;
    const unsigned int NP = P.gemm_np;
    float* As = bay_smem;                              // [F][NP]   (the sampler's layout,
    float* Aux = As + (size_t)BAY_GEMM_F * NP;         // [NP][AUXS] copied as one block)
    float* Ys = Aux + (size_t)NP * BAY_AUXS;           // [F][BAY_WT]
    float* Yw = Ys + BAY_GEMM_F * BAY_WT;              // [BAY_WT][BAY_DPAD]
    __shared__ float sZ[BAY_WT], sU2[BAY_WT], sW[BAY_WT];
    __shared__ unsigned int sJ[BAY_WT];
    __shared__ float sPrep[BAY_WT][BAY_PREP_LEN];
    __shared__ bay_cf sSum[BAY_WT];
    __shared__ float sLx[BAY_WT];
    __shared__ __align__(8) unsigned long long sBar;

    const unsigned int kind = ACCU ? 1u : 0u;
    const unsigned int tid = threadIdx.x;
    const unsigned int k0 = blockIdx.x * BAY_WT;
    const unsigned int nk = LOGFN_ONLY ? P.W : P.K;
    const unsigned int step = P.ctl->step[kind] + P.step_off;
    const float* hyper = P.params + P.data_len;
    float* X = P.xs + (LOGFN_ONLY ? 0 : (size_t)P.half * P.K * DIM);
    const float* S = P.xs + (size_t)(1u - P.half) * P.K * DIM;

    // 1. one TMA bulk copy (cp.async.bulk, completion counted on an mbarrier) brings the
    //    laid-out matrix and aux values into shared memory; it overlaps the proposals.
    const unsigned int lay_bytes =
        (unsigned int)(((size_t)BAY_GEMM_F * NP + (size_t)NP * BAY_AUXS) * sizeof(float));
    const unsigned int bar = (unsigned int)__cvta_generic_to_shared(&sBar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                     "r"(lay_bytes) : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
            ::"r"((unsigned int)__cvta_generic_to_shared(As)), "l"(P.gemm_lay), "r"(lay_bytes),
            "r"(bar) : "memory");
    }
    // 2. proposals (Philox, z, partner) for the tile, then Y in both layouts; each thread
    //    keeps all its gather loads in flight before it uses any of them
    if (!LOGFN_ONLY && tid < BAY_WT) {
        const unsigned int k = k0 + tid;
        if (k < nk) {
            const unsigned int stream = ACCU ? (P.half ? 2222u : 1111u) : (P.half ? 4444u : 3333u);
            bay_u4 c;
            c.x = k;
            c.y = step;
            c.z = stream;
            c.w = 0xbeeff00du;
            const bay_u4 r = bay_philox4x32_10(c, P.ctl->seed[kind] + P.half, 0xdecafbadu);
            const float z = bay_stretch_z(P.ctl->a, bay_u01(r.y));
            sZ[tid] = z;
            sJ[tid] = bay_partner(bay_u01(r.x), P.K);
            sU2[tid] = bay_u01(r.z);
            sLx[tid] = P.logfn[(size_t)P.half * P.K + k];
        }
    }
    __syncthreads();
    {
        // The tile's own rows are one contiguous block of BAY_WT * DIM floats; element e is
        // (walker e / DIM, coordinate e % DIM), so a warp reads its own elements coalesced
        // and each partner row (DIM contiguous floats) in runs of consecutive coordinates.
        constexpr int NE = (BAY_WT * DIM + 255) / 256;   // elements per thread
        constexpr int CH = 16;                            // loads kept in flight per batch
        const float* Xt = X + (size_t)k0 * DIM;
        const unsigned int n_own = (nk - k0 < BAY_WT ? nk - k0 : BAY_WT) * DIM;
#pragma unroll
        for (int c0 = 0; c0 < NE; c0 += CH) {
            float xv[CH], sv[CH];
#pragma unroll
            for (int i = 0; i < CH; ++i) {
                const unsigned int e = tid + 256u * (unsigned int)(c0 + i);
                const unsigned int w = e / DIM, d = e - w * DIM;
                const bool ev = (c0 + i < NE) && e < n_own;
                xv[i] = ev ? Xt[e] : 0.0f;
                sv[i] = (!LOGFN_ONLY && ev) ? S[(size_t)sJ[w] * DIM + d] : 0.0f;
            }
#pragma unroll
            for (int i = 0; i < CH; ++i) {
                const unsigned int e = tid + 256u * (unsigned int)(c0 + i);
                if ((c0 + i < NE) && e < BAY_WT * DIM) {
                    const unsigned int w = e / DIM, d = e - w * DIM;
                    const float y = LOGFN_ONLY ? xv[i]
                        : (e < n_own ? __fmaf_rn(sZ[w], __fsub_rn(xv[i], sv[i]), sv[i]) : 0.0f);
                    Yw[w * BAY_DPAD + d] = y;
                }
            }
        }
    }
    __syncthreads();
    // feature-major copy of the coefficient block for the register tiles (bank-conflict
    // free: consecutive lanes write consecutive walkers and read rows of odd stride)
    for (unsigned int e = tid; e < BAY_GEMM_F * BAY_WT; e += blockDim.x) {
        const unsigned int f = e / BAY_WT, w = e - f * BAY_WT;
        Ys[e] = Yw[w * BAY_DPAD + BAY_GEMM_COEF + f];
    }
    // the matrix copy: bounded wait; a CTA-uniform timeout flags the sampler and exits
    {
        unsigned int done = 0;
        for (unsigned int it = 0; it < (1u << 22) && !done; ++it)
            asm volatile(
                "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                " selp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(done) : "r"(bar), "r"(0u) : "memory");
        if (__syncthreads_or(!done)) {
            if (tid == 0) atomicOr(&P.ctl->status, 1u);
            return;
        }
    }
    // 3. per-walker precompute and the terms outside the row sum
    if (tid < BAY_WT) {
        float pr[BAY_PREP_LEN];
#pragma unroll
        for (int i = 0; i < BAY_PREP_LEN; ++i) pr[i] = 0.0f;
        float wt = 0.0f;
        if (k0 + tid < nk) {
            BAY_GEMM_PREP(hyper, P.params_len, DIM, &Yw[tid * BAY_DPAD], pr);
            wt = BAY_GEMM_WALKER(P.gemm_rows, hyper, P.params_len, DIM, &Yw[tid * BAY_DPAD]);
        }
#pragma unroll
        for (int i = 0; i < BAY_PREP_LEN; ++i) sPrep[tid][i] = pr[i];
        sW[tid] = wt;
    }
    __syncthreads();
    // 4. eta tiles and row terms
    const unsigned int wg = tid / BAY_NG, rg = tid - wg * BAY_NG;
    const unsigned int w0 = wg * BAY_RW;
    float sum[BAY_RW], cmp[BAY_RW];
#pragma unroll
    for (int i = 0; i < BAY_RW; ++i) {
        sum[i] = 0.0f;
        cmp[i] = 0.0f;
    }
    for (unsigned int r0 = 0; r0 < NP; r0 += BAY_ROWS_PER_PASS) {
        const unsigned int n0 = r0 + rg * BAY_RN;
        float acc[BAY_RW][BAY_RN];
#pragma unroll
        for (int i = 0; i < BAY_RW; ++i)
#pragma unroll
            for (int j = 0; j < BAY_RN; ++j) acc[i][j] = 0.0f;
#pragma unroll 5
        for (int f = 0; f < BAY_GEMM_F; ++f) {
            const float4 y = *reinterpret_cast<const float4*>(&Ys[f * BAY_WT + w0]);
            const float4 a = *reinterpret_cast<const float4*>(&As[(size_t)f * NP + n0]);
            const float yv[4] = {y.x, y.y, y.z, y.w};
            const float av[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
            for (int i = 0; i < BAY_RW; ++i)
#pragma unroll
                for (int j = 0; j < BAY_RN; ++j) acc[i][j] = __fmaf_rn(av[j], yv[i], acc[i][j]);
        }
#pragma unroll
        for (int j = 0; j < BAY_RN; ++j) {
            const unsigned int r = n0 + j;
            if (r < rows) {
#pragma unroll
                for (int i = 0; i < BAY_RW; ++i) {
                    const float t = BAY_GEMM_TERM(acc[i][j], &Aux[(size_t)r * BAY_AUXS], (uint64_t)r,
                                                  &Yw[(w0 + i) * BAY_DPAD], sPrep[w0 + i]);
                    const float yk = __fsub_rn(t, cmp[i]);
                    const float s2 = __fadd_rn(sum[i], yk);
                    cmp[i] = __fsub_rn(__fsub_rn(s2, sum[i]), yk);
                    sum[i] = s2;
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < BAY_RW; ++i) {
        bay_cf v;
        v.hi = sum[i];
        v.lo = -cmp[i];
#pragma unroll
        for (int o = BAY_NG / 2; o > 0; o >>= 1) v = bay_cadd(v, bay_cf_shfl_xor(v, o));
        if (rg == 0) sSum[w0 + i] = v;
    }
    __syncthreads();
    // 5. accept (one thread per walker), then the tile's rows written back cooperatively
    //    (accepted walkers' proposals; for the accu statistics the rejected walkers' current
    //    rows are copied into the tile), statistics
    __shared__ unsigned char sAcc[BAY_WT];
    const unsigned int k = k0 + tid;
    const bool valid = tid < BAY_WT && k < nk;
    bool accepted = false;
    if (valid) {
        bay_cf t;
        t.hi = sW[tid];
        t.lo = 0.0f;
        t = bay_cadd(t, sSum[tid]);
        const float ly = __fadd_rn(t.hi, t.lo);
        if (LOGFN_ONLY) {
            P.logfn[k] = ly;
        } else {
            accepted = bay_accept(sU2[tid], sZ[tid], ly, sLx[tid], ACCU ? 1.0f : P.ctl->beta);
            if (accepted) P.logfn[(size_t)P.half * P.K + k] = ly;
        }
    }
    if (LOGFN_ONLY) return;
    if (tid < BAY_WT) sAcc[tid] = accepted ? 1 : 0;
    const int n_acc = __syncthreads_count(accepted);
    {
        float* Xt = X + (size_t)k0 * DIM;
        const unsigned int n_own = (nk - k0 < BAY_WT ? nk - k0 : BAY_WT) * DIM;
        for (unsigned int e = tid; e < n_own; e += blockDim.x) {
            const unsigned int w = e / DIM, d = e - w * DIM;
            if (sAcc[w]) Xt[e] = Yw[w * BAY_DPAD + d];
            else if (ACCU) Yw[w * BAY_DPAD + d] = Xt[e];
        }
    }
    if (ACCU) {
        __syncthreads();
        if (tid == 0 && n_acc) atomicAdd(&P.ctl->accepted, (unsigned long long)n_acc);
        if (P.means_cap != 0) {
            float* out = P.part + ((size_t)P.step_off * 2 + P.half) * DIM * gridDim.x
                + blockIdx.x;
            const unsigned int nv = nk - k0 < BAY_WT ? nk - k0 : BAY_WT;
            for (unsigned int d = tid; d < DIM; d += blockDim.x) {
                bay_cf s;
                s.hi = 0.0f;
                s.lo = 0.0f;
                for (unsigned int w = 0; w < nv; ++w) {
                    bay_cf y;
                    y.hi = Yw[w * BAY_DPAD + d];
                    y.lo = 0.0f;
                    s = bay_cadd(s, y);
                }
                out[(size_t)d * gridDim.x] = __fadd_rn(s.hi, s.lo);
            }
        }
    }
}

extern "C" __global__ void __launch_bounds__(256) bay_stretch_bare(bay_stretch_params P) {
    bay_stretch_gemm<false, false>(P);
}
extern "C" __global__ void __launch_bounds__(256) bay_stretch_accu(bay_stretch_params P) {
    bay_stretch_gemm<true, false>(P);
}
extern "C" __global__ void __launch_bounds__(256) bay_logfn_all(bay_stretch_params P) {
    bay_stretch_gemm<false, true>(P);
}

// ---------------------------------------------------------------- GEMM form, streaming
// For matrices too large for shared memory.  A half-step is three launches:
//   propose: one thread per walker -- Philox, stretch, partner, proposal row, prep and the
//            terms outside the row sum into per-walker scratch;
//   rows:    CTA (128-walker tile, row super-block): the tile's coefficient block stays in
//            shared memory (feature-major); for each 128-row sub-block the matrix is
//            streamed in 32-feature chunks; each thread owns 8 walkers x 8 rows (rows
//            rg + 16 j) of eta, applies the row term with Kahan sums, and the 16 row-group
//            lanes of a walker combine as compensated fp32 pairs -> s_part[sb][walker];
//            blockIdx.x runs over walker tiles so that the tiles sharing a row block run
//            together and the block is read from HBM once;
//   accept:  one thread per walker -- partials summed in super-block order, accept,
//            write-back, statistics.
#define BAY_SW 128
#define BAY_SR 128
#define BAY_SF 32
#define BAY_XS (BAY_SR + 1)   // odd row stride of the staged matrix chunk (no bank conflicts)

// bf16 of a float rounded to nearest even, as its 16 bits (NaN stays a quiet NaN)
__device__ __forceinline__ unsigned short bay_bf16_rn(float x) {
    unsigned int u = __float_as_uint(x);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (unsigned short)((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (unsigned short)(u >> 16);
}
__device__ __forceinline__ float bay_bf16_float(unsigned short h) {
    return __uint_as_float((unsigned int)h << 16);
}
// Two floats as packed bf16 hi + lo pairs (a in the low halves, b in the high halves), each
// rounded to nearest even by one cvt.rn.bf16x2.f32: hi = bf16(x), lo = bf16(x - hi).
__device__ __forceinline__ void bay_split_bf16x2(float a, float b, unsigned int& hi,
                                                 unsigned int& lo) {
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(hi) : "f"(b), "f"(a));
    const float ha = __uint_as_float(hi << 16), hb = __uint_as_float(hi & 0xffff0000u);
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(lo) : "f"(__fsub_rn(b, hb)), "f"(__fsub_rn(a, ha)));
}

template <int MODE>  // 0 bare, 1 accu, 2 log density of the current positions
__device__ __forceinline__ void bay_gemm_propose_impl(const bay_stretch_params& P) {
    const unsigned int kind = MODE == 1 ? 1u : 0u;
    const unsigned int nk = MODE == 2 ? P.W : P.K;
    const unsigned int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nk) return;
    float* y = P.s_y + (size_t)k * DIM;
    if (MODE == 2) {
        const float* x = P.xs + (size_t)k * DIM;
        for (int d = 0; d < DIM; ++d) y[d] = x[d];
    } else {
        const float* X = P.xs + (size_t)P.half * P.K * DIM + (size_t)k * DIM;
        const unsigned int stream = MODE == 1 ? (P.half ? 2222u : 1111u) : (P.half ? 4444u : 3333u);
        bay_u4 c;
        c.x = k;
        c.y = P.ctl->step[kind] + P.step_off;
        c.z = stream;
        c.w = 0xbeeff00du;
        const bay_u4 r = bay_philox4x32_10(c, P.ctl->seed[kind] + P.half, 0xdecafbadu);
        const float z = bay_stretch_z(P.ctl->a, bay_u01(r.y));
        const unsigned int j = bay_partner(bay_u01(r.x), P.K);
        const float* S = P.xs + (size_t)(1u - P.half) * P.K * DIM + (size_t)j * DIM;
        for (int d = 0; d < DIM; ++d) {
            const float s = S[d];
            y[d] = __fmaf_rn(z, __fsub_rn(X[d], s), s);
        }
        P.s_zu[2 * (size_t)k] = z;
        P.s_zu[2 * (size_t)k + 1] = bay_u01(r.z);
    }
    if (!P.s_bh) {
        for (int f = 0; f < BAY_GEMM_F; ++f) P.s_b[(size_t)k * BAY_GEMM_F + f] = y[BAY_GEMM_COEF + f];
    } else {
        // the tensor-core form's operand: coefficient = hi + lo, both bf16
        for (int f = 0; f < BAY_GEMM_F; ++f) {
            const float v = y[BAY_GEMM_COEF + f];
            const unsigned short h = bay_bf16_rn(v);
            P.s_bh[(size_t)k * P.tc_fp + f] = h;
            P.s_bl[(size_t)k * P.tc_fp + f] = bay_bf16_rn(__fsub_rn(v, bay_bf16_float(h)));
        }
    }
    const float* hyper = P.params + P.data_len;
    float pr[BAY_PREP_LEN];
#pragma unroll
    for (int i = 0; i < BAY_PREP_LEN; ++i) pr[i] = 0.0f;
    BAY_GEMM_PREP(hyper, P.params_len, DIM, y, pr);
#pragma unroll
    for (int i = 0; i < BAY_PREP_LEN; ++i) P.s_prep[(size_t)k * BAY_PREP_LEN + i] = pr[i];
    P.s_w[k] = BAY_GEMM_WALKER(P.gemm_rows, hyper, P.params_len, DIM, y);
}

template <int MODE>
__device__ __forceinline__ void bay_gemm_rows_impl(const bay_stretch_params& P) {
    extern __shared__ __align__(128) float bay_smem[];
    float* Bs = bay_smem;                              // [F][BAY_SW]
    float* Xs = Bs + (size_t)BAY_GEMM_F * BAY_SW;      // [BAY_SF][BAY_XS]
    __shared__ float sPrep[BAY_SW][BAY_PREP_LEN];
    const unsigned int nk = MODE == 2 ? P.W : P.K;
    const unsigned int tid = threadIdx.x;
    const unsigned int k0 = blockIdx.x * BAY_SW;
    const unsigned int sb = blockIdx.y;
    const unsigned int rows = (unsigned int)P.gemm_rows;
    const float* A = P.params + P.gemm_base;
    // the tile's coefficient block, feature-major (walkers past nk are zero)
    for (unsigned int e = tid; e < BAY_GEMM_F * BAY_SW; e += blockDim.x) {
        const unsigned int f = e / BAY_SW, w = e - f * BAY_SW;
        Bs[e] = (k0 + w < nk) ? P.s_b[(size_t)(k0 + w) * BAY_GEMM_F + f] : 0.0f;
    }
    for (unsigned int e = tid; e < BAY_SW * BAY_PREP_LEN; e += blockDim.x) {
        const unsigned int w = e / BAY_PREP_LEN, i = e - w * BAY_PREP_LEN;
        sPrep[w][i] = (k0 + w < nk) ? P.s_prep[(size_t)(k0 + w) * BAY_PREP_LEN + i] : 0.0f;
    }
    const unsigned int wg = tid >> 4, rg = tid & 15u;
    const unsigned int w0 = wg * 8;
    float sum[8], cmp[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        sum[i] = 0.0f;
        cmp[i] = 0.0f;
    }
    const unsigned int rb = sb * P.s_sbrows;
    const unsigned int re = rb + P.s_sbrows < rows ? rb + P.s_sbrows : rows;
    for (unsigned int r0 = rb; r0 < re; r0 += BAY_SR) {
        float acc[8][8];
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
        for (unsigned int f0 = 0; f0 < BAY_GEMM_F; f0 += BAY_SF) {
            __syncthreads();
            // chunk of rows r0..r0+127, features f0..f0+31: reads run along each row
            for (unsigned int e = tid; e < BAY_SR * BAY_SF; e += blockDim.x) {
                const unsigned int r = e / BAY_SF, fl = e - r * BAY_SF;
                const unsigned int f = f0 + fl;
                Xs[fl * BAY_XS + r] = (r0 + r < re && f < BAY_GEMM_F)
                    ? __ldg(A + (size_t)(r0 + r) * P.gemm_ld + f) : 0.0f;
            }
            __syncthreads();
            const unsigned int fe = BAY_GEMM_F - f0 < BAY_SF ? BAY_GEMM_F - f0 : BAY_SF;
#pragma unroll 4
            for (unsigned int fl = 0; fl < fe; ++fl) {
                const float4 b0 = *reinterpret_cast<const float4*>(&Bs[(f0 + fl) * BAY_SW + w0]);
                const float4 b1 = *reinterpret_cast<const float4*>(&Bs[(f0 + fl) * BAY_SW + w0 + 4]);
                const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
                float xv[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) xv[j] = Xs[fl * BAY_XS + rg + 16 * j];
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < 8; ++j) acc[i][j] = __fmaf_rn(bv[i], xv[j], acc[i][j]);
            }
        }
        // row terms of this sub-block
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const unsigned int r = r0 + rg + 16 * j;
            if (r < re) {
                float aux[BAY_AUXS];
#pragma unroll
                for (int c = 0; c < BAY_AUXS; ++c)
                    aux[c] = BAY_GEMM_AUX > 0 ? __ldg(A + (size_t)r * P.gemm_ld + BAY_GEMM_AUXCOL + c) : 0.0f;
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const unsigned int kw = k0 + w0 + i < nk ? k0 + w0 + i : nk - 1;
                    const float t = BAY_GEMM_TERM(acc[i][j], aux, (uint64_t)r,
                                                  P.s_y + (size_t)kw * DIM, sPrep[w0 + i]);
                    const float yk = __fsub_rn(t, cmp[i]);
                    const float s2 = __fadd_rn(sum[i], yk);
                    cmp[i] = __fsub_rn(__fsub_rn(s2, sum[i]), yk);
                    sum[i] = s2;
                }
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        bay_cf v;
        v.hi = sum[i];
        v.lo = -cmp[i];
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) v = bay_cadd(v, bay_cf_shfl_xor(v, o));
        const unsigned int kw = k0 + w0 + i;
        if (rg == 0 && kw < nk) {
            P.s_part[2 * ((size_t)sb * nk + kw)] = v.hi;
            P.s_part[2 * ((size_t)sb * nk + kw) + 1] = v.lo;
        }
    }
}

template <int MODE>
__device__ __forceinline__ void bay_gemm_accept_impl(const bay_stretch_params& P) {
    const unsigned int nk = MODE == 2 ? P.W : P.K;
    const unsigned int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = k < nk;
    bool accepted = false;
    if (valid) {
        bay_cf s;
        s.hi = 0.0f;
        s.lo = 0.0f;
        for (unsigned int sb = 0; sb < P.s_nsb; ++sb) {
            bay_cf p;
            p.hi = P.s_part[2 * ((size_t)sb * nk + k)];
            p.lo = P.s_part[2 * ((size_t)sb * nk + k) + 1];
            s = bay_cadd(s, p);
        }
        const float ly = bay_cf_total(P.s_w[k], s);
        if (MODE == 2) {
            P.logfn[k] = ly;
        } else {
            const float lx = P.logfn[(size_t)P.half * P.K + k];
            accepted = bay_accept(P.s_zu[2 * (size_t)k + 1], P.s_zu[2 * (size_t)k], ly, lx,
                                  MODE == 1 ? 1.0f : P.ctl->beta);
            if (accepted) {
                float* X = P.xs + (size_t)P.half * P.K * DIM + (size_t)k * DIM;
                const float* y = P.s_y + (size_t)k * DIM;
                for (int d = 0; d < DIM; ++d) X[d] = y[d];
                P.logfn[(size_t)P.half * P.K + k] = ly;
            }
        }
    }
    if (MODE != 1) return;
    // accu: acceptance count and the per-dim sums of this CTA's walkers (new positions)
    const int n_acc = __syncthreads_count(accepted);
    if (threadIdx.x == 0 && n_acc) atomicAdd(&P.ctl->accepted, (unsigned long long)n_acc);
    if (P.means_cap == 0) return;
    const unsigned int k0 = blockIdx.x * blockDim.x;
    const unsigned int nv = nk - k0 < blockDim.x ? nk - k0 : blockDim.x;
    const float* Xc = P.xs + (size_t)P.half * P.K * DIM + (size_t)k0 * DIM;
    float* out = P.part + ((size_t)P.step_off * 2 + P.half) * DIM * gridDim.x + blockIdx.x;
    for (unsigned int d = threadIdx.x; d < DIM; d += blockDim.x) {
        bay_cf s;
        s.hi = 0.0f;
        s.lo = 0.0f;
        // in walker order; unrolled so that several rows' loads are in flight
#pragma unroll 8
        for (unsigned int w = 0; w < nv; ++w) {
            bay_cf y;
            y.hi = Xc[(size_t)w * DIM + d];
            y.lo = 0.0f;
            s = bay_cadd(s, y);
        }
        out[(size_t)d * gridDim.x] = __fadd_rn(s.hi, s.lo);
    }
}

extern "C" __global__ void __launch_bounds__(256) bay_gemm_propose_bare(bay_stretch_params P) {
    bay_gemm_propose_impl<0>(P);
}
extern "C" __global__ void __launch_bounds__(256) bay_gemm_propose_accu(bay_stretch_params P) {
    bay_gemm_propose_impl<1>(P);
}
extern "C" __global__ void __launch_bounds__(256) bay_gemm_propose_logfn(bay_stretch_params P) {
    bay_gemm_propose_impl<2>(P);
}
extern "C" __global__ void __launch_bounds__(256) bay_gemm_rows_move(bay_stretch_params P) {
    bay_gemm_rows_impl<0>(P);
}
extern "C" __global__ void __launch_bounds__(256) bay_gemm_rows_logfn(bay_stretch_params P) {
    bay_gemm_rows_impl<2>(P);
}
extern "C" __global__ void __launch_bounds__(256) bay_gemm_accept_bare(bay_stretch_params P) {
    bay_gemm_accept_impl<0>(P);
}
extern "C" __global__ void __launch_bounds__(256) bay_gemm_accept_accu(bay_stretch_params P) {
    bay_gemm_accept_impl<1>(P);
}
extern "C" __global__ void __launch_bounds__(256) bay_gemm_accept_logfn(bay_stretch_params P) {
    bay_gemm_accept_impl<2>(P);
}

#if BAY_GEMM_TC
// ---------------------------------------------------------------- GEMM form, tensor cores
// The rows launch of the streaming form with eta on the 5th-generation tensor cores:
// eta[walker][row] = sum_f B[walker][f] A[row][f], A and B each split into bf16 hi + lo
// and three products (hi.hi + hi.lo + lo.hi) accumulated in fp32 in tensor memory; the
// dropped lo.lo product is below 2^-16 of each term.  tcgen05.mma kind::f16 with
// M = 128 walkers (TMEM lanes), N = 128 rows (TMEM columns), K = 16 per instruction,
// both operands K-major in shared memory with the 128-byte swizzle TMA writes.
// CTA roles: warp 0 -- TMA producer (the CTA's walker operand once, then each 128-row
// tile in 64-feature chunks through a ring of BAY_TC_STAGES stages); warp 1 -- TMEM
// allocation and the MMA issue (one thread); warps 2 .. 17 -- epilogue, a thread per
// walker and share of a tile's rows: tcgen05.ld of its TMEM lane, the model's row terms,
// a compensated sum over the super-block's rows.  Two accumulator buffers in TMEM let the MMAs of
// tile t + 1 run under the epilogue of tile t.  Every wait is bounded in time; a wait
// that gives up sets the sampler's status word and the CTA's abort flag, and the CTA
// drains its own copies and MMAs, frees its TMEM and exits.
#ifndef BAY_TC_G
#define BAY_TC_G 1
#endif
#ifndef BAY_TC_STAGES
#define BAY_TC_STAGES 2
#endif
#define BAY_TC_FP ((BAY_GEMM_F + 63) / 64 * 64)
#define BAY_TC_KC (BAY_TC_FP / 64)
#define BAY_TC_TILE 16384u                      // one 128 x 64 bf16 operand chunk
#define BAY_TC_WBYTES ((unsigned int)BAY_TC_G * BAY_TC_KC * 2u * BAY_TC_TILE)
#define BAY_TC_SBYTES (2u * BAY_TC_TILE)        // a stage: rows hi + lo chunk
#define BAY_TC_AUXF (128u * BAY_AUXS)
#define BAY_TC_NEPI 512u                        // epilogue threads (16 warps)
#define BAY_TC_THREADS 576
#define BAY_TC_COLS (BAY_TC_G == 2 ? 512u : 256u)
#define BAY_TC_WAIT_NS 2000000000ull
// instruction descriptor: fp32 accumulator, bf16 A and B, both K-major, N = 128, M = 128
#define BAY_TC_IDESC ((1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24))

// the four TMA tensor maps (CUtensorMap, 128 bytes each), a __grid_constant__ parameter
struct __align__(64) bay_tmaps {
    unsigned long long xh[16];   // matrix rows, bf16 hi: dims {tc_fp, rows_pad}, box {64, 128}
    unsigned long long xl[16];   // matrix rows, bf16 lo
    unsigned long long bh[16];   // coefficient block, bf16 hi: dims {tc_fp, walkers_pad}
    unsigned long long bl[16];   // coefficient block, bf16 lo
};

__device__ __forceinline__ unsigned long long bay_globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for the completion of the phase of parity `par` of the mbarrier at shared address
// `bar`.  Gives up after BAY_TC_WAIT_NS, or as soon as another role has given up (abort
// flag set; pass abort = nullptr for a wait that must not be cut short).  Giving up on
// time sets the abort flag and the sampler's status word.
__device__ __forceinline__ bool bay_tc_wait(unsigned int bar, unsigned int par,
                                            volatile unsigned int* abort, unsigned int* status) {
    unsigned long long t0 = 0;
    for (unsigned int it = 0;; ++it) {
        unsigned int ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok) : "r"(bar), "r"(par) : "memory");
        if (ok) return true;
        if ((it & 15u) == 0u) {
            if (abort && *abort) return false;
            const unsigned long long t = bay_globaltimer();
            if (it == 0u) {
                t0 = t;
            } else if (t - t0 > BAY_TC_WAIT_NS) {
                if (abort) *abort = 1u;
                atomicOr(status, 2u);
                return false;
            }
        }
    }
}

__device__ __forceinline__ void bay_mbar_init(unsigned int bar, unsigned int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void bay_expect_tx(unsigned int bar, unsigned int bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bay_tma2d(unsigned int dst, const void* map, int c0, int c1,
                                          unsigned int bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"((unsigned long long)map), "r"(c0), "r"(c1), "r"(bar) : "memory");
}
// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ unsigned long long bay_sdesc(unsigned int saddr) {
    return (unsigned long long)((saddr & 0x3FFFFu) >> 4)
         | (1ull << 16)                                    // leading offset (unused here)
         | ((unsigned long long)(1024u >> 4) << 32)        // stride offset
         | (1ull << 46)                                    // tcgen05 descriptor version
         | (2ull << 61);                                   // 128-byte swizzle
}
__device__ __forceinline__ void bay_mma(unsigned int d, unsigned long long a, unsigned long long b,
                                        unsigned int acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(d), "l"(a), "l"(b), "r"(BAY_TC_IDESC), "r"(acc) : "memory");
}
__device__ __forceinline__ void bay_mma_commit(unsigned int bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(bar) : "memory");
}
__device__ __forceinline__ void bay_tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void bay_tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// 16 consecutive TMEM columns of this thread's lane
__device__ __forceinline__ void bay_tmem_ld16(unsigned int ta, float (&v)[16]) {
    unsigned int r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
        "%11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(ta));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <int MODE>  // 0: move (K walkers of the moving half), 2: log density of all W
__device__ __forceinline__ void bay_gemm_rows_tc_impl(const bay_stretch_params& P,
                                                      const bay_tmaps& T) {
    extern __shared__ __align__(1024) unsigned char bay_smem_tc[];
    const unsigned int raw = (unsigned int)__cvta_generic_to_shared(bay_smem_tc);
    const unsigned int pad = ((raw + 1023u) & ~1023u) - raw;
    unsigned char* sm = bay_smem_tc + pad;
    const unsigned int s_wop = raw + pad;                    // walker operand [G][KC][hi,lo]
    const unsigned int s_stg = s_wop + BAY_TC_WBYTES;        // row stages [S][hi,lo]
    float* saux = (float*)(sm + BAY_TC_WBYTES + BAY_TC_STAGES * BAY_TC_SBYTES);  // [2][AUXF]
    unsigned long long* bars = (unsigned long long*)(saux + 2 * BAY_TC_AUXF);
    volatile unsigned int* flags = (volatile unsigned int*)(bars + 2 * BAY_TC_STAGES + 6);
    const unsigned int bar0 = (unsigned int)__cvta_generic_to_shared(bars);
    // barriers: full[S], empty[S], tmem full[2], tmem empty[2], walker operand, drain
    const unsigned int b_full = bar0, b_empty = bar0 + 8u * BAY_TC_STAGES;
    const unsigned int b_tfull = bar0 + 16u * BAY_TC_STAGES, b_tempty = b_tfull + 16u;
    const unsigned int b_wop = b_tempty + 16u, b_drain = b_wop + 8u;
    // flags: [0] TMEM base, [1] abort, [2], [3] epilogue go flags of the two buffers
    volatile unsigned int* abort = flags + 1;
    unsigned int* status = &P.ctl->status;

    const unsigned int warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const unsigned int nk = MODE == 2 ? P.W : P.K;
    const unsigned int k0 = blockIdx.x * (128u * BAY_TC_G);
    const unsigned int rows = (unsigned int)P.gemm_rows;
    const unsigned int rb = blockIdx.y * P.s_sbrows;
    const unsigned long long re64 = (unsigned long long)rb + P.s_sbrows;
    const unsigned int re = re64 < rows ? (unsigned int)re64 : rows;
    const unsigned int ntile = (re - rb + 127u) / 128u;

    if (threadIdx.x == 0) {
        for (unsigned int s = 0; s < BAY_TC_STAGES; ++s) {
            bay_mbar_init(b_full + 8u * s, 1u);
            bay_mbar_init(b_empty + 8u * s, 1u);
        }
        for (unsigned int b = 0; b < 2; ++b) {
            bay_mbar_init(b_tfull + 8u * b, 1u);
            bay_mbar_init(b_tempty + 8u * b, BAY_TC_NEPI / 32u);
        }
        bay_mbar_init(b_wop, 1u);
        bay_mbar_init(b_drain, 1u);
        flags[1] = 0u;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        const unsigned int dst = (unsigned int)__cvta_generic_to_shared((const void*)flags);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(dst), "r"(BAY_TC_COLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    bay_tc_fence_before();
    __syncthreads();
    bay_tc_fence_after();
    const unsigned int tmem = flags[0];

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer
            bay_expect_tx(b_wop, BAY_TC_WBYTES);
            for (unsigned int g = 0; g < BAY_TC_G; ++g)
                for (unsigned int c = 0; c < BAY_TC_KC; ++c) {
                    const unsigned int dst = s_wop + ((g * BAY_TC_KC + c) * 2u) * BAY_TC_TILE;
                    bay_tma2d(dst, T.bh, (int)(c * 64u), (int)(k0 + g * 128u), b_wop);
                    bay_tma2d(dst + BAY_TC_TILE, T.bl, (int)(c * 64u), (int)(k0 + g * 128u), b_wop);
                }
            unsigned int issued = 0;
            bool ok = true;
            for (unsigned int t = 0; t < ntile && ok; ++t) {
                for (unsigned int c = 0; c < BAY_TC_KC; ++c) {
                    const unsigned int s = issued % BAY_TC_STAGES, u = issued / BAY_TC_STAGES;
                    if (u > 0u && !bay_tc_wait(b_empty + 8u * s, (u - 1u) & 1u, abort, status)) {
                        ok = false;
                        break;
                    }
                    const unsigned int dst = s_stg + s * BAY_TC_SBYTES;
                    bay_expect_tx(b_full + 8u * s, BAY_TC_SBYTES);
                    bay_tma2d(dst, T.xh, (int)(c * 64u), (int)(rb + t * 128u), b_full + 8u * s);
                    bay_tma2d(dst + BAY_TC_TILE, T.xl, (int)(c * 64u), (int)(rb + t * 128u),
                              b_full + 8u * s);
                    ++issued;
                }
            }
            // drain: every copy issued here has landed before the CTA may exit
            bay_tc_wait(b_wop, 0u, nullptr, status);
            for (unsigned int i = issued > BAY_TC_STAGES ? issued - BAY_TC_STAGES : 0u; i < issued; ++i)
                bay_tc_wait(b_full + 8u * (i % BAY_TC_STAGES), (i / BAY_TC_STAGES) & 1u, nullptr, status);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issue
            bool ok = bay_tc_wait(b_wop, 0u, abort, status);
            bay_tc_fence_after();
            unsigned int i = 0;
            for (unsigned int t = 0; t < ntile && ok; ++t) {
                const unsigned int b = t & 1u, ub = t >> 1;
                if (ub > 0u && !(ok = bay_tc_wait(b_tempty + 8u * b, (ub - 1u) & 1u, abort, status)))
                    break;
                bay_tc_fence_after();
                const unsigned int d0 = tmem + b * (128u * BAY_TC_G);
                for (unsigned int c = 0; c < BAY_TC_KC; ++c, ++i) {
                    const unsigned int s = i % BAY_TC_STAGES, u = i / BAY_TC_STAGES;
                    if (!(ok = bay_tc_wait(b_full + 8u * s, u & 1u, abort, status))) break;
                    bay_tc_fence_after();
                    const unsigned int xs = s_stg + s * BAY_TC_SBYTES;
#pragma unroll
                    for (unsigned int g = 0; g < BAY_TC_G; ++g) {
                        const unsigned int wa = s_wop + ((g * BAY_TC_KC + c) * 2u) * BAY_TC_TILE;
#pragma unroll
                        for (unsigned int ks = 0; ks < 4u; ++ks) {
                            const unsigned long long ah = bay_sdesc(wa + 32u * ks);
                            const unsigned long long al = bay_sdesc(wa + BAY_TC_TILE + 32u * ks);
                            const unsigned long long xh = bay_sdesc(xs + 32u * ks);
                            const unsigned long long xl = bay_sdesc(xs + BAY_TC_TILE + 32u * ks);
                            const unsigned int d = d0 + g * 128u;
                            bay_mma(d, ah, xh, (c | ks) != 0u ? 1u : 0u);
                            bay_mma(d, ah, xl, 1u);
                            bay_mma(d, al, xh, 1u);
                        }
                    }
                    bay_mma_commit(b_empty + 8u * s);  // the stage is free once these finish
                }
                if (!ok) break;
                bay_mma_commit(b_tfull + 8u * b);
            }
            // drain: every MMA issued here has finished before TMEM is released
            bay_mma_commit(b_drain);
            bay_tc_wait(b_drain, 0u, nullptr, status);
        }
    } else {
        // ---- epilogue, 16 warps in 4 groups of 4 (a group covers the 128 TMEM lanes).
        //      G = 2: group e takes walker sub-tile e / 2, rows 64 (e % 2) .. + 63 of a tile;
        //      G = 1: group e takes sub-tile 0, rows 32 e .. 32 e + 31.  A thread owns one
        //      walker (its TMEM lane): per 16-row batch it evaluates the row terms, sums them
        //      pairwise and adds the batch sum to a Kahan-compensated running sum; the
        //      groups' partial sums of a walker are combined at the end in group order.
        constexpr unsigned int GPS = 4u / BAY_TC_G;        // groups per walker sub-tile
        constexpr unsigned int NCOL = 128u / GPS;          // rows of a tile per group
        const unsigned int et = threadIdx.x - 64u;
        const unsigned int grp = (warp - 2u) >> 2, q = warp & 3u;
        const unsigned int g = grp / GPS;
        const unsigned int c0 = NCOL * (grp % GPS);
        const unsigned int wl = 32u * q + lane;
        const unsigned int kw = k0 + g * 128u + wl;
        const bool wv = kw < nk;
        const unsigned int kc = wv ? kw : nk - 1u;
        float prep[BAY_PREP_LEN];
#pragma unroll
        for (int i = 0; i < BAY_PREP_LEN; ++i) prep[i] = P.s_prep[(size_t)kc * BAY_PREP_LEN + i];
        const float* xw = P.s_y + (size_t)kc * DIM;
        const float* auxg = P.gemm_lay + (size_t)rb * BAY_AUXS;   // [rows_pad][AUXS]
        constexpr unsigned int MA = (BAY_TC_AUXF + BAY_TC_NEPI - 1u) / BAY_TC_NEPI;
        float apre[MA];
#pragma unroll
        for (unsigned int m = 0; m < MA; ++m) {
            const unsigned int j = et + m * BAY_TC_NEPI;
            apre[m] = (j < BAY_TC_AUXF && ntile > 0u) ? __ldg(auxg + j) : 0.0f;
        }
        float sum = 0.0f, cmp = 0.0f;
        bool ok = true;
        for (unsigned int t = 0; t < ntile; ++t) {
            const unsigned int b = t & 1u;
            float* sa = saux + b * BAY_TC_AUXF;
#pragma unroll
            for (unsigned int m = 0; m < MA; ++m) {
                const unsigned int j = et + m * BAY_TC_NEPI;
                if (j < BAY_TC_AUXF) sa[j] = apre[m];
            }
            // next tile's aux values, in flight during this tile
#pragma unroll
            for (unsigned int m = 0; m < MA; ++m) {
                const unsigned int j = et + m * BAY_TC_NEPI;
                apre[m] = (j < BAY_TC_AUXF && t + 1u < ntile)
                    ? __ldg(auxg + (size_t)(t + 1u) * BAY_TC_AUXF + j) : 0.0f;
            }
            // one thread waits for the accumulator; the decision is shared so that every
            // epilogue thread leaves the loop together (the named barrier is not bounded)
            if (et == 0u) flags[2 + b] = bay_tc_wait(b_tfull + 8u * b, (t >> 1) & 1u, abort, status) ? 1u : 0u;
            asm volatile("bar.sync 1, %0;" ::"r"(BAY_TC_NEPI) : "memory");
            if (!flags[2 + b]) {
                ok = false;
                break;
            }
            bay_tc_wait(b_tfull + 8u * b, (t >> 1) & 1u, nullptr, status);  // already complete
            bay_tc_fence_after();
            const unsigned int r0 = rb + t * 128u;
            const unsigned int nrow = re - r0 < 128u ? re - r0 : 128u;
            const unsigned int ta = tmem + ((32u * q) << 16) + b * (128u * BAY_TC_G) + g * 128u + c0;
#pragma unroll 1
            for (unsigned int j0 = 0; j0 < NCOL; j0 += 16u) {
                float v[16];
                bay_tmem_ld16(ta + j0, v);
                const unsigned int jb = c0 + j0;   // the batch's first row within the tile
                // the batch's aux values: 16 * AUXS consecutive floats, 16-byte aligned
                float av[16 * BAY_AUXS];
#pragma unroll
                for (unsigned int i = 0; i < 4u * BAY_AUXS; ++i) {
                    const float4 a4 = reinterpret_cast<const float4*>(sa + jb * BAY_AUXS)[i];
                    av[4 * i] = a4.x;
                    av[4 * i + 1] = a4.y;
                    av[4 * i + 2] = a4.z;
                    av[4 * i + 3] = a4.w;
                }
                if (jb + 16u <= nrow) {
#pragma unroll
                    for (unsigned int jj = 0; jj < 16u; ++jj)
                        v[jj] = BAY_GEMM_TERM(v[jj], &av[jj * BAY_AUXS], (uint64_t)(r0 + jb + jj),
                                              xw, prep);
                } else {
#pragma unroll
                    for (unsigned int jj = 0; jj < 16u; ++jj)
                        v[jj] = jb + jj < nrow
                            ? BAY_GEMM_TERM(v[jj], &av[jj * BAY_AUXS], (uint64_t)(r0 + jb + jj), xw, prep)
                            : 0.0f;
                }
#pragma unroll
                for (unsigned int w = 8u; w >= 1u; w >>= 1)
#pragma unroll
                    for (unsigned int i = 0; i < w; ++i) v[i] = __fadd_rn(v[i], v[i + w]);
                const float yk = __fsub_rn(v[0], cmp);
                const float s2 = __fadd_rn(sum, yk);
                cmp = __fsub_rn(__fsub_rn(s2, sum), yk);
                sum = s2;
            }
            bay_tc_fence_before();
            __syncwarp();
            if (lane == 0u)
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(b_tempty + 8u * b) : "memory");
        }
        // the groups' partial sums of each walker, combined as compensated pairs in group
        // order; stage 0 is free once the last tile's MMAs (hence its copies) are complete
        float* xchg = (float*)(sm + BAY_TC_WBYTES);        // [4 groups][128 lanes][hi, lo]
        if (ok) {
            xchg[2 * (grp * 128u + wl)] = sum;
            xchg[2 * (grp * 128u + wl) + 1] = -cmp;
        }
        asm volatile("bar.sync 1, %0;" ::"r"(BAY_TC_NEPI) : "memory");
        if (ok && grp % GPS == 0u && wv) {
            bay_cf a;
            a.hi = sum;
            a.lo = -cmp;
#pragma unroll
            for (unsigned int o = 1; o < GPS; ++o) {
                bay_cf p;
                p.hi = xchg[2 * ((grp + o) * 128u + wl)];
                p.lo = xchg[2 * ((grp + o) * 128u + wl) + 1];
                a = bay_cadd(a, p);
            }
            P.s_part[2 * ((size_t)blockIdx.y * nk + kw)] = a.hi;
            P.s_part[2 * ((size_t)blockIdx.y * nk + kw) + 1] = a.lo;
        }
    }
    bay_tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        bay_tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(BAY_TC_COLS) : "memory");
    }
}

extern "C" __global__ void __launch_bounds__(BAY_TC_THREADS, 1)
bay_gemm_rows_tc_move(bay_stretch_params P, const __grid_constant__ bay_tmaps T) {
    bay_gemm_rows_tc_impl<0>(P, T);
}
extern "C" __global__ void __launch_bounds__(BAY_TC_THREADS, 1)
bay_gemm_rows_tc_logfn(bay_stretch_params P, const __grid_constant__ bay_tmaps T) {
    bay_gemm_rows_tc_impl<2>(P, T);
}

// ---------------------------------------------------------------- GEMM form, tensor cores,
// resident matrix.  For matrices of at most 256 rows that fit in shared memory with the
// walker operand (e.g. a precision matrix): one launch per half-step, a CTA per 64
// walkers (M = 128 MMAs of which lanes 0..63 are read back: small CTAs, four per SM).  The sampler keeps an image of the matrix as the MMA's B operand -- bf16 hi
// and lo, rows padded to gemm_np (a multiple of 16), K-major in 128-byte-swizzled
// 64-feature atoms -- followed by the rows' aux values; one bulk copy brings it into
// shared memory while the CTA draws its proposals.  The proposals' coefficient blocks are
// split into bf16 hi + lo and written in the same swizzled layout as the A operand; one
// thread issues the 3 x (features / 16) MMAs (N = gemm_np rows, fp32 accumulators in
// TMEM); then each walker's row terms are read back from its TMEM lane (two warps per
// lane group, half of the rows each), summed pairwise with a Kahan carry and combined,
// and the accept step and write-back follow as in the SIMT form.
#ifndef BAY_TR_W
#define BAY_TR_W 64u                                    // walkers per CTA: 64 or 128
#endif
#define BAY_TR_ATOM (BAY_TR_W * 128u)                   // BAY_TR_W walkers x 64 bf16 (one atom)
#define BAY_TR_DPAD (DIM | 1)

__device__ __forceinline__ void bay_tmem_ld8(unsigned int ta, float (&v)[8]) {
    unsigned int r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                   "=r"(r[6]), "=r"(r[7])
                 : "r"(ta));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// n8 (1..4, warp-uniform) loads of 8 TMEM columns each from ta, ta + 8, ..., then one wait:
// the loads' latencies overlap.  v[8 q + i] = column ta + 8 q + i of the thread's lane.
__device__ __forceinline__ void bay_tmem_ld32(unsigned int ta, unsigned int n8, float (&v)[32]) {
    unsigned int r[32];
#pragma unroll
    for (unsigned int q = 0; q < 4u; ++q) {
        if (q < n8)
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                         : "=r"(r[8 * q]), "=r"(r[8 * q + 1]), "=r"(r[8 * q + 2]), "=r"(r[8 * q + 3]),
                           "=r"(r[8 * q + 4]), "=r"(r[8 * q + 5]), "=r"(r[8 * q + 6]), "=r"(r[8 * q + 7])
                         : "r"(ta + 8u * q));
        else
#pragma unroll
            for (int i = 0; i < 8; ++i) r[8 * q + i] = 0u;
    }
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void bay_mma_n(unsigned int d, unsigned long long a, unsigned long long b,
                                          unsigned int idesc, unsigned int acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(d), "l"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
}

// 8 consecutive floats (dims 8u .. 8u + 7) of a walker row: float4 loads when rows are
// 16-byte aligned (DIM % 4 == 0), float2 when 8-byte aligned, else scalar; zero past DIM
// or when !ok (no access at all).  In the persistent form other CTAs rewrote the rows
// since this SM last read them: the grid barrier's acquire orders these loads after those
// writes.
__device__ __forceinline__ void bay_tr_ld8(const float* row, unsigned int u, bool ok, float (&v)[8]) {
    const unsigned int d0 = 8u * u;
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = 0.0f;
    if (!ok) return;
    if (d0 + 8u <= DIM && DIM % 4u == 0u) {
        const float4 a = *(const float4*)(row + d0), b = *(const float4*)(row + d0 + 4u);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    } else if (d0 + 8u <= DIM && DIM % 2u == 0u) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 a = *(const float2*)(row + d0 + 2u * i);
            v[2 * i] = a.x;
            v[2 * i + 1] = a.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < 8; ++i)
            if (d0 + i < DIM) v[i] = row[d0 + i];
    }
}

// the store counterpart of bay_tr_ld8 (dims past DIM are not written)
__device__ __forceinline__ void bay_tr_st8(float* row, unsigned int u, const float (&v)[8]) {
    const unsigned int d0 = 8u * u;
    if (d0 + 8u <= DIM && DIM % 4u == 0u) {
        *(float4*)(row + d0) = make_float4(v[0], v[1], v[2], v[3]);
        *(float4*)(row + d0 + 4u) = make_float4(v[4], v[5], v[6], v[7]);
    } else if (d0 + 8u <= DIM && DIM % 2u == 0u) {
#pragma unroll
        for (int i = 0; i < 4; ++i) *(float2*)(row + d0 + 2u * i) = make_float2(v[2 * i], v[2 * i + 1]);
    } else {
#pragma unroll
        for (int i = 0; i < 8; ++i)
            if (d0 + i < DIM) row[d0 + i] = v[i];
    }
}

// 16-byte unit u (8 features) of walker row w in an A atom, at unit u ^ (w % 8) of its
// 128-byte row (the 128B swizzle); hi atoms first, lo atoms BAY_TC_KC atoms later
__device__ __forceinline__ void bay_tr_put_a(unsigned int s_a, unsigned int w, unsigned int u,
                                             const unsigned int (&hw)[4], const unsigned int (&lw)[4]) {
    const unsigned int off = (u >> 3) * BAY_TR_ATOM + w * 128u + (((u & 7u) ^ (w & 7u)) << 4);
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(s_a + off), "r"(hw[0]),
                 "r"(hw[1]), "r"(hw[2]), "r"(hw[3]) : "memory");
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};"
                 ::"r"(s_a + BAY_TC_KC * BAY_TR_ATOM + off), "r"(lw[0]), "r"(lw[1]), "r"(lw[2]),
                 "r"(lw[3]) : "memory");
}

// Grid barrier k (k = 1, 2, ... within a launch) of a cooperative launch (every CTA
// resident): each CTA adds 1 to the arrival count (a release reduction, no reply awaited)
// and waits until the count reaches k * nblocks; the count only grows during a launch.
// Bounded: a CTA that waits longer than BAY_TC_WAIT_NS raises ctl->abort and status bit 4;
// a raised abort ends every wait at once.  Returns false when the launch is being
// abandoned.  The count and the abort word are cleared before each launch.  `extra`
// arrivals beyond the grid (nonzero only in tests) make every barrier run out.
__device__ __forceinline__ bool bay_grid_barrier(bay_ctl* ctl, unsigned int nblocks, unsigned int k,
                                                 unsigned int extra) {
    __shared__ unsigned int s_go;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int go = 1u;
        volatile unsigned int* ab = &ctl->abort;
        if (*ab) {
            go = 0u;
        } else {
            const unsigned int target = k * nblocks + extra;
            __threadfence();                               // the CTA's writes before its arrival
            asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(&ctl->gbar_count) : "memory");
            unsigned long long t0 = bay_globaltimer();
            for (unsigned int it = 0;; ++it) {
                unsigned int c;
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(&ctl->gbar_count) : "memory");
                if (c >= target) break;
                __nanosleep(32);
                if ((it & 63u) == 63u) {
                    if (*ab) {
                        go = 0u;
                        break;
                    }
                    if (bay_globaltimer() - t0 > BAY_TC_WAIT_NS) {
                        *ab = 1u;
                        atomicOr(&ctl->status, 4u);
                        go = 0u;
                        break;
                    }
                }
            }
            __threadfence();
        }
        s_go = go;
    }
    __syncthreads();
    return s_go != 0u;
}

// Named barrier of one 256-thread tile group (ids 1..4; id 0 is the CTA's __syncthreads)
__device__ __forceinline__ void bay_gsync(unsigned int g) {
    asm volatile("bar.sync %0, 256;" ::"r"(g + 1u) : "memory");
}
__device__ __forceinline__ int bay_gsync_count(unsigned int g, bool p) {
    int n;
    asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %2, 0;\n bar.red.popc.u32 %0, %1, 256, q;\n}\n"
                 : "=r"(n) : "r"(g + 1u), "r"((unsigned int)p) : "memory");
    return n;
}
__device__ __forceinline__ bool bay_gsync_and(unsigned int g, bool p) {
    unsigned int r;
    asm volatile("{\n .reg .pred q, o;\n setp.ne.u32 q, %2, 0;\n bar.red.and.pred o, %1, 256, q;\n"
                 " selp.u32 %0, 1, 0, o;\n}\n"
                 : "=r"(r) : "r"(g + 1u), "r"((unsigned int)p) : "memory");
    return r != 0u;
}

// Shared memory of one tile group after the A atoms: the proposals Yw [BAY_TR_W][DPAD] and
// 2 x 256 floats of reduction scratch, at least the 8 KB past the last atom that the
// M = 128 MMA reads (walker rows 64..127 of a 64-walker tile, never read back); 1 KB
// multiple.
#define BAY_TR_TAIL_RAW ((BAY_TR_W * BAY_TR_DPAD * 4u + 2048u) > (16384u - BAY_TR_ATOM) \
                         ? (BAY_TR_W * BAY_TR_DPAD * 4u + 2048u) : (16384u - BAY_TR_ATOM))
#define BAY_TR_TAIL ((BAY_TR_TAIL_RAW + 1023u) & ~1023u)
#define BAY_TR_GREG (2u * BAY_TC_KC * BAY_TR_ATOM + BAY_TR_TAIL)   // bytes per tile group

// The statistics of a tile: per-dim sums of its walkers' positions in a fixed order.
// BAY_TR_NG walker groups (256 / DIM, at most 8; one for DIM >= 128) of BAY_TR_WG
// consecutive walkers; thread (wg, d) sums its group in fp32 in walker order (pass 1, into
// scr[wg * DIM + d], or straight to out[d * ntiles] with one group), then thread d adds the
// groups' sums in group order (pass 2).  The per-step means add the tiles' sums in FP64.
#define BAY_TR_NG (DIM >= 128u ? 1u : (256u / DIM < 8u ? 256u / DIM : 8u))
#define BAY_TR_WG ((BAY_TR_W + BAY_TR_NG - 1u) / BAY_TR_NG)

// pass 1 over the rows in device memory (rows of DIM floats, nt walkers), threads 0..255
__device__ __forceinline__ void bay_tr_sums_pass1(const float* rows, unsigned int nt, unsigned int tid,
                                                  float* scr, float* out, unsigned int ntiles) {
    for (unsigned int t = tid; t < BAY_TR_NG * DIM; t += 256u) {
        const unsigned int wg = t / DIM, d = t - wg * DIM;
        float v = 0.0f;
#pragma unroll
        for (unsigned int i = 0; i < BAY_TR_WG; ++i) {
            const unsigned int w = wg * BAY_TR_WG + i;
            if (w < nt) v = __fadd_rn(v, rows[(size_t)w * DIM + d]);
        }
        if (BAY_TR_NG == 1u) out[(size_t)d * ntiles] = v;
        else scr[t] = v;
    }
}

// pass 2 (after a barrier that follows pass 1)
__device__ __forceinline__ void bay_tr_sums_pass2(unsigned int tid, const float* scr, float* out,
                                                  unsigned int ntiles) {
    if (BAY_TR_NG > 1u && tid < DIM) {
        float a = 0.0f;
#pragma unroll
        for (unsigned int wg = 0; wg < BAY_TR_NG; ++wg) a = __fadd_rn(a, scr[wg * DIM + tid]);
        out[(size_t)tid * ntiles] = a;
    }
}

// The resident tensor-core form.  A CTA holds G independent tile groups of 256 threads
// (G = 1: an ordinary CTA); each group has its own A operand, proposals, scratch, MMA
// barrier and TMEM columns, and syncs on its own named barrier; the matrix image is shared.
// PERSIST = false: one half-step (P.half, P.step_off), tile blockIdx.x (G = 1), launched
// with programmatic dependent launch.  PERSIST = true: a cooperative launch of m steps
// (both halves each, step offsets P.step_off .. + m - 1) over a grid of co-resident CTAs
// whose groups take tiles (g * gridDim.x + blockIdx.x) + k * gridDim.x * G of every half-step, with
// a grid barrier between half-steps; barriers, TMEM and the image are set up once.  Every
// tile computes what the per-launch form computes (same statistics slots), so the two
// forms give identical results.  A group whose bounded wait gives up raises ctl->abort
// and goes on to the next grid barrier, where the whole launch stops.
template <bool ACCU, bool LOGFN_ONLY, bool PERSIST, unsigned int G>
__device__ __forceinline__ void bay_stretch_tcr(const bay_stretch_params& P, unsigned int m) {
    // Shared memory: [matrix image][group 0: A hi atoms, lo atoms, Yw, red][group 1 ...].
    // The MMA runs M = 128 (an M = 64 form was measured no faster): with 64-walker tiles it
    // also reads the 8 KB after each atom's 64 rows (the next atom, or the group's Yw) as
    // walker rows 64..127, whose accumulator lanes are never read.
    extern __shared__ __align__(1024) unsigned char bay_smem_tr[];
    const unsigned int NP = P.gemm_np;                       // rows padded to 16
    const unsigned int rows = (unsigned int)P.gemm_rows;
    const unsigned int raw = (unsigned int)__cvta_generic_to_shared(bay_smem_tr);
    const unsigned int pad = ((raw + 1023u) & ~1023u) - raw;
    unsigned char* sm = bay_smem_tr + pad;
    const unsigned int img_bytes = 2u * BAY_TC_KC * NP * 128u + NP * BAY_AUXS * 4u;
    const unsigned int a_off0 = (img_bytes + 1023u) & ~1023u;
    const unsigned int s_img = raw + pad;
    const float* Aux = (const float*)(sm + 2u * BAY_TC_KC * NP * 128u);     // [NP][AUXS]
    __shared__ float sZ[G][BAY_TR_W], sU2[G][BAY_TR_W], sW[G][BAY_TR_W], sLx[G][BAY_TR_W];
    __shared__ unsigned int sJ[G][BAY_TR_W];
    __shared__ float sPrep[G][BAY_TR_W][BAY_PREP_LEN];
    __shared__ float sHalf[G][BAY_TR_W][2];
    __shared__ unsigned char sAcc[G][BAY_TR_W];
    __shared__ __align__(8) unsigned long long sBar[1 + G];
    __shared__ unsigned int sTmem, sOk[G];

    const unsigned int kind = ACCU ? 1u : 0u;
    const unsigned int g = G == 1u ? 0u : threadIdx.x >> 8;                // tile group
    const unsigned int tid = threadIdx.x & 255u, warp = tid >> 5, lane = tid & 31u;
    const unsigned int nk = LOGFN_ONLY ? P.W : P.K;
    const unsigned int ntiles = (nk + BAY_TR_W - 1u) / BAY_TR_W;
    const float* hyper = P.params + P.data_len;
    const unsigned int a_off = a_off0 + g * BAY_TR_GREG;
    const unsigned int s_a = s_img + a_off;
    float* Yw = (float*)(sm + a_off + 2u * BAY_TC_KC * BAY_TR_ATOM);         // [W][DPAD]
    float* red = Yw + BAY_TR_W * BAY_TR_DPAD;                                // [256]
    float* red2 = red + 256;                                                 // [256]
    const unsigned int bar_img = (unsigned int)__cvta_generic_to_shared(&sBar[0]);
    const unsigned int bar_mma = (unsigned int)__cvta_generic_to_shared(&sBar[1 + g]);
    unsigned int* status = &P.ctl->status;
    const unsigned int ncols = NP <= 32u ? 32u : (NP <= 64u ? 64u : (NP <= 128u ? 128u : 256u));

    // 1. barriers, TMEM (G x ncols columns), and the matrix image's bulk copy
    if (threadIdx.x == 0) {
        bay_mbar_init(bar_img, 1u);
        for (unsigned int q = 0; q < G; ++q)
            bay_mbar_init((unsigned int)__cvta_generic_to_shared(&sBar[1 + q]), 1u);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (threadIdx.x < 32u) {
        const unsigned int dst = (unsigned int)__cvta_generic_to_shared(&sTmem);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(dst), "r"(ncols * G) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    bay_tc_fence_before();
    __syncthreads();
    bay_tc_fence_after();
    const unsigned int tmem = sTmem + g * ncols;
    // the matrix image is written once, when the sampler is created, so its copy may start
    // before this launch's dependency on the previous kernel resolves
    if (threadIdx.x == 0) {
        bay_expect_tx(bar_img, img_bytes);
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
            ::"r"(s_img), "l"(P.gemm_lay), "r"(img_bytes), "r"(bar_img) : "memory");
    }
    unsigned int mma_par = 0u;                  // phase parity of bar_mma's next completion
    const unsigned int nsteps = PERSIST ? m : 1u;
    const unsigned int h_lo = (PERSIST && !LOGFN_ONLY) ? 0u : P.half;
    const unsigned int h_hi = (PERSIST && !LOGFN_ONLY) ? 2u : P.half + 1u;
    // control words, constant during a launch: separate kernels between chunks write them,
    // and a launch after one of those starts only once it completed
    const unsigned int step0 = P.ctl->step[kind], seed0 = P.ctl->seed[kind];
    const float a_str = P.ctl->a, beta = ACCU ? 1.0f : P.ctl->beta;
    // tiles g * gridDim.x + blockIdx.x, + G * gridDim.x, ...: consecutive tiles on
    // different SMs, every SM busy when the tiles outnumber the CTAs
    const unsigned int tile0 = g * gridDim.x + blockIdx.x;
    const unsigned int tstride = PERSIST ? gridDim.x * G : ntiles;
    constexpr unsigned int NU = (DIM + 7u) / 8u;               // 8-dim units of a row
    constexpr unsigned int NQ = BAY_TR_W * NU;                  // (walker, unit) items
    constexpr unsigned int IB = 2u;                             // items in flight per thread
    // 2. proposals (Philox, z, partner) and the current log densities of a tile's walkers
    auto proposals = [&](unsigned int tile, unsigned int half, unsigned int step) {
        const unsigned int k0 = tile * BAY_TR_W;
        const unsigned int nt = nk - k0 < BAY_TR_W ? nk - k0 : BAY_TR_W;
        if (tid < nt) {
            const unsigned int k = k0 + tid;
            const unsigned int stream = ACCU ? (half ? 2222u : 1111u) : (half ? 4444u : 3333u);
            bay_u4 c;
            c.x = k;
            c.y = step;
            c.z = stream;
            c.w = 0xbeeff00du;
            const bay_u4 r = bay_philox4x32_10(c, seed0 + half, 0xdecafbadu);
            sZ[g][tid] = bay_stretch_z(a_str, bay_u01(r.y));
            sJ[g][tid] = bay_partner(bay_u01(r.x), P.K);
            sU2[g][tid] = bay_u01(r.z);
            sLx[g][tid] = P.logfn[(size_t)half * P.K + k];
        }
    };
    // the first gather pass's own rows (the tile's walkers): kept in registers, or, in the
    // persistent form (64 registers a thread at 1,024 threads), parked in Yw by the thread
    // that later reads them back
    float xpre[IB][8];
    auto own_rows = [&](const float* Xt, unsigned int nt) {
#pragma unroll
        for (unsigned int b = 0; b < IB; ++b) {
            const unsigned int q = b * 256u + tid;
            const unsigned int w = q / NU, u = q - w * NU;
            bay_tr_ld8(Xt + (size_t)w * DIM, u, q < NQ && w < nt, xpre[b]);
            if (PERSIST && q < NQ) {
#pragma unroll
                for (unsigned int i = 0; i < 8u; ++i)
                    if (8u * u + i < DIM) Yw[w * BAY_TR_DPAD + 8u * u + i] = xpre[b][i];
            }
        }
    };
    if (!PERSIST) {
        // One launch per half-step: this half's walkers last moved two launches back, so
        // their rows and log densities, like the draws, are final once the previous launch
        // began its work -- which it did only after waiting for its own predecessor, before
        // it let this launch start.  Load them now; only the partner rows (the half the
        // previous launch moves) wait for that launch and its memory.
        if (tile0 < ntiles) {
            const unsigned int k0 = tile0 * BAY_TR_W;
            const unsigned int nt = nk - k0 < BAY_TR_W ? nk - k0 : BAY_TR_W;
            if (!LOGFN_ONLY) proposals(tile0, P.half, step0 + P.step_off);
            own_rows(P.xs + (LOGFN_ONLY ? 0 : (size_t)P.half * P.K * DIM) + (size_t)k0 * DIM, nt);
        }
        asm volatile("griddepcontrol.wait;" ::: "memory");
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    }
    bool go = true;
    for (unsigned int si = 0; si < nsteps && go; ++si) {
    for (unsigned int half = h_lo; half < h_hi && go; ++half) {
    const unsigned int step_off = P.step_off + si;
    const unsigned int step = step0 + step_off;
    float* X = P.xs + (LOGFN_ONLY ? 0 : (size_t)half * P.K * DIM);
    const float* S = P.xs + (size_t)(1u - half) * P.K * DIM;
    // persistent: the group's first tile of this half-step loads its draws, own rows and
    // log densities before the grid barrier.  The tile-to-group map is fixed, so only this
    // group wrote those rows and densities (two half-steps back, ordered by its end-of-tile
    // barrier); during the half-step the barrier closes, other CTAs only read them.
    if (PERSIST && tile0 < ntiles) {
        const unsigned int nt0 = nk - tile0 * BAY_TR_W < BAY_TR_W ? nk - tile0 * BAY_TR_W : BAY_TR_W;
        if (!LOGFN_ONLY) proposals(tile0, half, step);
        own_rows(X + (size_t)tile0 * BAY_TR_W * DIM, nt0);
    }
    if (PERSIST && (si | (half - h_lo)) != 0u)
        go = bay_grid_barrier(P.ctl, gridDim.x, 2u * si + (half - h_lo), P.gbar_extra);
    if (!go) break;
    for (unsigned int tile = tile0; tile < ntiles; tile += tstride) {
    const unsigned int k0 = tile * BAY_TR_W;
    const unsigned int nt = nk - k0 < BAY_TR_W ? nk - k0 : BAY_TR_W;
    float* const Xt = X + (size_t)k0 * DIM;
    if (PERSIST && tile != tile0) {
        if (!LOGFN_ONLY) proposals(tile, half, step);
        own_rows(Xt, nt);
    }
    bay_gsync(g);
    // 3. Y of the tile (walker-major rows of odd stride) from (walker, 8-dim unit) items:
    //    consecutive threads take consecutive units of a row (the tile's own rows are one
    //    contiguous block, a partner's row is 4 * DIM contiguous bytes), IB items' loads in
    //    flight per thread; with the coefficients at dim 0 the same thread splits its unit
    //    into bf16 hi + lo and writes it to the A operand
    for (unsigned int q0 = 0; q0 < NQ; q0 += IB * 256u) {
        float xv[IB][8], sv[IB][8];
#pragma unroll
        for (unsigned int b = 0; b < IB; ++b) {
            const unsigned int q = q0 + b * 256u + tid;
            const unsigned int w = q / NU, u = q - w * NU;
            const bool ok = q < NQ && w < nt;
            if (q0 == 0u && PERSIST) {
#pragma unroll
                for (unsigned int i = 0; i < 8u; ++i)
                    xv[b][i] = (q < NQ && 8u * u + i < DIM) ? Yw[w * BAY_TR_DPAD + 8u * u + i] : 0.0f;
            } else if (q0 == 0u) {
#pragma unroll
                for (int i = 0; i < 8; ++i) xv[b][i] = xpre[b][i];
            } else {
                bay_tr_ld8(Xt + (size_t)w * DIM, u, ok, xv[b]);
            }
            if (!LOGFN_ONLY) bay_tr_ld8(S + (size_t)sJ[g][ok ? w : 0u] * DIM, u, ok, sv[b]);
        }
#pragma unroll
        for (unsigned int b = 0; b < IB; ++b) {
            const unsigned int q = q0 + b * 256u + tid;
            if (q < NQ) {
                const unsigned int w = q / NU, u = q - w * NU;
                float y[8];
                const float z = LOGFN_ONLY ? 0.0f : sZ[g][w];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    y[i] = LOGFN_ONLY ? xv[b][i]
                                      : (w < nt ? __fmaf_rn(z, __fsub_rn(xv[b][i], sv[b][i]), sv[b][i]) : 0.0f);
                    if (8u * u + i < DIM) Yw[w * BAY_TR_DPAD + 8u * u + i] = y[i];
                }
#if BAY_GEMM_COEF == 0
                if (u < BAY_TC_KC * 8u) {
                    unsigned int hw[4], lw[4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const unsigned int f = 8u * u + 2u * i;
                        bay_split_bf16x2(f < BAY_GEMM_F ? y[2 * i] : 0.0f,
                                         f + 1u < BAY_GEMM_F ? y[2 * i + 1] : 0.0f, hw[i], lw[i]);
                    }
                    bay_tr_put_a(s_a, w, u, hw, lw);
                }
#endif
            }
        }
    }
#if BAY_GEMM_COEF == 0
    // 4. A units past the row's last unit are zero
    if (BAY_TC_KC * 8u > NU) {
        constexpr unsigned int NZ = BAY_TC_KC * 8u > NU ? BAY_TC_KC * 8u - NU : 1u;
        const unsigned int zw[4] = {0u, 0u, 0u, 0u};
        for (unsigned int q = tid; q < BAY_TR_W * NZ; q += 256u) {
            const unsigned int w = q / NZ;
            bay_tr_put_a(s_a, w, NU + (q - w * NZ), zw, zw);
        }
    }
#else
    // 4. the A operand from Yw (coefficients at dim BAY_GEMM_COEF): 16-byte units of hi, lo
    bay_gsync(g);
    for (unsigned int q = tid; q < BAY_TR_W * BAY_TC_KC * 8u; q += 256u) {
        const unsigned int w = q / (BAY_TC_KC * 8u), u = q - w * (BAY_TC_KC * 8u);
        unsigned int hw[4], lw[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const unsigned int f = u * 8u + 2u * i;
            const float v0 = f < BAY_GEMM_F ? Yw[w * BAY_TR_DPAD + BAY_GEMM_COEF + f] : 0.0f;
            const float v1 = f + 1u < BAY_GEMM_F ? Yw[w * BAY_TR_DPAD + BAY_GEMM_COEF + f + 1u] : 0.0f;
            bay_split_bf16x2(v0, v1, hw[i], lw[i]);
        }
        bay_tr_put_a(s_a, w, u, hw, lw);
    }
#endif
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // A visible to the MMAs
    bay_gsync(g);
    // 5. one thread: wait for the image, issue the MMAs, commit; the others precompute
    if (tid == 0) {
        unsigned int ok = bay_tc_wait(bar_img, 0u, nullptr, status) ? 1u : 0u;   // once done, stays
        if (ok) {
            bay_tc_fence_after();
            const unsigned int idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((NP >> 3) << 17) |
                                       ((128u >> 4) << 24);
            for (unsigned int c = 0; c < BAY_TC_KC; ++c) {
#pragma unroll
                for (unsigned int ks = 0; ks < 4u; ++ks) {
                    const unsigned int ao = c * BAY_TR_ATOM + 32u * ks;
                    const unsigned int bo = c * NP * 128u + 32u * ks;
                    const unsigned long long ah = bay_sdesc(s_a + ao);
                    const unsigned long long al = bay_sdesc(s_a + BAY_TC_KC * BAY_TR_ATOM + ao);
                    const unsigned long long bh = bay_sdesc(s_img + bo);
                    const unsigned long long bl = bay_sdesc(s_img + BAY_TC_KC * NP * 128u + bo);
                    bay_mma_n(tmem, ah, bh, idesc, (c | ks) != 0u ? 1u : 0u);
                    bay_mma_n(tmem, ah, bl, idesc, 1u);
                    bay_mma_n(tmem, al, bh, idesc, 1u);
                }
            }
        }
        bay_mma_commit(bar_mma);   // also arrives with nothing issued (a failed wait)
        sOk[g] = ok;
    }
    if (tid < BAY_TR_W) {
        float pr[BAY_PREP_LEN];
#pragma unroll
        for (int i = 0; i < BAY_PREP_LEN; ++i) pr[i] = 0.0f;
        float wt = 0.0f;
        if (tid < nt) {
            BAY_GEMM_PREP(hyper, P.params_len, DIM, &Yw[tid * BAY_TR_DPAD], pr);
            wt = BAY_GEMM_WALKER(P.gemm_rows, hyper, P.params_len, DIM, &Yw[tid * BAY_TR_DPAD]);
        }
#pragma unroll
        for (int i = 0; i < BAY_PREP_LEN; ++i) sPrep[g][tid][i] = pr[i];
        sW[g][tid] = wt;
    }
    // accu, one launch per half-step: while the MMAs run, the statistics of the previous
    // half-step -- this tile of the other half, final since the previous launch completed
    // and not written by this one: (step_off, 0) from the launch of half 1, (step_off - 1,
    // 1) from the launch of half 0 (the chunk's last one has a launch of its own)
    const bool prev_stats = ACCU && !PERSIST && P.means_cap != 0 && (half == 1u || step_off > 0u);
    float* const prev_out = prev_stats
        ? P.part + ((size_t)(half == 1u ? step_off : step_off - 1u) * 2 + (1u - half)) * DIM * ntiles + tile
        : nullptr;
    // (one launch per half-step: the statistics run on the warps idle in the epilogue)
    if (prev_stats && PERSIST)
        bay_tr_sums_pass1(P.xs + (size_t)(1u - half) * P.K * DIM + (size_t)k0 * DIM, nt, tid,
                          red2, prev_out, ntiles);
    // every thread waits for the MMAs (bounded; the commit arrives even if none were issued)
    // and observes the image copy itself before reading the aux values it brought
    const bool mma_done = bay_tc_wait(bar_mma, mma_par, nullptr, status);
    mma_par ^= 1u;
    const bool img_done = bay_tc_wait(bar_img, 0u, nullptr, status);
    // one verdict for the whole CTA (a wait that gave up in any thread fails the tile)
    const bool ok = bay_gsync_and(g, mma_done && img_done) && sOk[g] != 0u;
    bay_tc_fence_after();
    // One launch per half-step (FAST): the epilogue's warps 0 and 1 decide their walkers
    // themselves once warps 4 and 5 have handed over the other half of the rows (a 128-
    // thread named barrier), and write back their own rows; no group barrier follows.
    // Meanwhile warps 2, 3, 6 and 7 finish the previous half-step's statistics (pass 1
    // ended before the barrier above).
    constexpr bool FAST = !PERSIST && !LOGFN_ONLY;
    const unsigned int hand_id = 1u + G + g;        // named barriers 1..G are the groups'
    if (FAST && prev_stats && (warp & 2u)) {
        // warps 2, 3, 6, 7 (128 threads, idle in the epilogue): both passes of the previous
        // half-step's statistics, the same slots and order as bay_tr_sums_pass1 / pass2,
        // with a 128-thread named barrier between them
        const unsigned int i0 = (warp >> 2) * 64u + (warp & 1u) * 32u + lane;
        const float* rows = P.xs + (size_t)(1u - half) * P.K * DIM + (size_t)k0 * DIM;
        for (unsigned int t = i0; t < BAY_TR_NG * DIM; t += 128u) {
            const unsigned int wg = t / DIM, d = t - wg * DIM;
            float v = 0.0f;
#pragma unroll
            for (unsigned int i = 0; i < BAY_TR_WG; ++i) {
                const unsigned int w = wg * BAY_TR_WG + i;
                if (w < nt) v = __fadd_rn(v, rows[(size_t)w * DIM + d]);
            }
            if (BAY_TR_NG == 1u) prev_out[(size_t)d * ntiles] = v;
            else red2[t] = v;
        }
        if (BAY_TR_NG > 1u) {
            asm volatile("bar.sync %0, 128;" ::"r"(1u + 2u * G + g) : "memory");
            for (unsigned int d = i0; d < DIM; d += 128u) {
                float a = 0.0f;
#pragma unroll
                for (unsigned int wg = 0; wg < BAY_TR_NG; ++wg) a = __fadd_rn(a, red2[wg * DIM + d]);
                prev_out[(size_t)d * ntiles] = a;
            }
        }
    }
    // 6. epilogue: warps 0, 1, 4, 5 read TMEM lanes 32 (w % 4) .. + 31 (walkers 0..63),
    //    rows [NP/2 * (w / 4), + NP/2) in 8-column loads; the two halves then combine
    if (32u * (warp & 3u) < BAY_TR_W) {
        const unsigned int wl = 32u * (warp & 3u) + lane;
        const unsigned int h = warp >> 2, half_rows = NP >> 1;
        const unsigned int c0 = h * half_rows;
        const unsigned int ta = tmem + ((32u * (warp & 3u)) << 16) + c0;
        const float* xw = &Yw[wl * BAY_TR_DPAD];
        float sum = 0.0f, cmp = 0.0f;
        // up to 32 columns per batch of loads (one wait), then per 8 columns: the row terms,
        // a pairwise sum, a Kahan step (the same order as one 8-column load at a time)
        for (unsigned int j1 = 0; j1 < half_rows; j1 += 32u) {
            const unsigned int n8 = (half_rows - j1) >= 32u ? 4u : (half_rows - j1) >> 3;
            float v32[32];
            bay_tmem_ld32(ta + j1, n8, v32);
#pragma unroll
            for (unsigned int q = 0; q < 4u; ++q) {
                if (q >= n8) break;
                float v[8];
#pragma unroll
                for (unsigned int i = 0; i < 8u; ++i) {
                    const unsigned int r = c0 + j1 + 8u * q + i;
                    v[i] = r < rows ? BAY_GEMM_TERM(v32[8u * q + i], &Aux[r * BAY_AUXS], (uint64_t)r, xw,
                                                    sPrep[g][wl])
                                    : 0.0f;
                }
#pragma unroll
                for (unsigned int s2 = 4u; s2 >= 1u; s2 >>= 1)
#pragma unroll
                    for (unsigned int i = 0; i < s2; ++i) v[i] = __fadd_rn(v[i], v[i + s2]);
                const float yk = __fsub_rn(v[0], cmp);
                const float t = __fadd_rn(sum, yk);
                cmp = __fsub_rn(__fsub_rn(t, sum), yk);
                sum = t;
            }
        }
        if (FAST) {
            if (h) {                                    // hand the second half over
                sHalf[g][wl][0] = sum;
                sHalf[g][wl][1] = -cmp;
                asm volatile("bar.arrive %0, 128;" ::"r"(hand_id) : "memory");
            } else {
                asm volatile("bar.sync %0, 128;" ::"r"(hand_id) : "memory");
                // 7. accept walker wl, write back its row and log density
                bool acc = false;
                if (wl < nt && ok) {
                    const unsigned int k = k0 + wl;
                    bay_cf t, a, b;
                    t.hi = sW[g][wl];
                    t.lo = 0.0f;
                    a.hi = sum;
                    a.lo = -cmp;
                    b.hi = sHalf[g][wl][0];
                    b.lo = sHalf[g][wl][1];
                    t = bay_cadd(t, bay_cadd(a, b));
                    const float ly = __fadd_rn(t.hi, t.lo);
                    acc = bay_accept(sU2[g][wl], sZ[g][wl], ly, sLx[g][wl], beta);
                    if (acc) {
                        P.logfn[(size_t)half * P.K + k] = ly;
                        const float* yr = &Yw[wl * BAY_TR_DPAD];
#pragma unroll 1
                        for (unsigned int u = 0; u < NU; ++u) {
                            float y[8];
#pragma unroll
                            for (int i = 0; i < 8; ++i) y[i] = 8u * u + i < DIM ? yr[8u * u + i] : 0.0f;
                            bay_tr_st8(Xt + (size_t)wl * DIM, u, y);
                        }
                    }
                }
                if (ACCU) {
                    const unsigned int bal = __ballot_sync(0xffffffffu, acc);
                    if (lane == 0 && bal) atomicAdd(&P.ctl->accepted, (unsigned long long)__popc(bal));
                }
            }
        } else if (h) {                                 // second half of the rows
            sHalf[g][wl][0] = sum;
            sHalf[g][wl][1] = -cmp;
        } else {                                        // first half: red[wl], red[W + wl]
            red[wl] = sum;
            red[BAY_TR_W + wl] = -cmp;
        }
    }
    if (FAST) {
        if (!ok) break;
        continue;                                       // the tile is done (one per launch)
    }
    bay_tc_fence_before();
    bay_gsync(g);
    if (prev_stats) bay_tr_sums_pass2(tid, red2, prev_out, ntiles);
    // 7. accept (one thread per walker), write-back, statistics
    bool accepted = false;
    if (tid < nt && ok) {
        const unsigned int k = k0 + tid;
        bay_cf t, a, b;
        t.hi = sW[g][tid];
        t.lo = 0.0f;
        a.hi = red[tid];
        a.lo = red[BAY_TR_W + tid];
        b.hi = sHalf[g][tid][0];
        b.lo = sHalf[g][tid][1];
        t = bay_cadd(t, bay_cadd(a, b));
        const float ly = __fadd_rn(t.hi, t.lo);
        if (LOGFN_ONLY) {
            P.logfn[k] = ly;
        } else {
            accepted = bay_accept(sU2[g][tid], sZ[g][tid], ly, sLx[g][tid], beta);
            if (accepted) P.logfn[(size_t)half * P.K + k] = ly;
        }
    }
    if (!LOGFN_ONLY) {
        if (tid < BAY_TR_W) sAcc[g][tid] = accepted ? 1 : 0;
        const int n_acc = bay_gsync_count(g, accepted);
        if (ACCU && PERSIST) {
            // the statistics need every walker's new position in Yw: the rejected walkers'
            // current rows are loaded (IB units in flight per thread), the accepted ones
            // stored
            for (unsigned int q0 = 0; q0 < NQ; q0 += IB * 256u) {
                float xv[IB][8];
#pragma unroll
                for (unsigned int b = 0; b < IB; ++b) {
                    const unsigned int q = q0 + b * 256u + tid;
                    const unsigned int w = q / NU, u = q - w * NU;
                    bay_tr_ld8(Xt + (size_t)w * DIM, u, q < NQ && w < nt && !sAcc[g][w < BAY_TR_W ? w : 0u],
                               xv[b]);
                }
#pragma unroll
                for (unsigned int b = 0; b < IB; ++b) {
                    const unsigned int q = q0 + b * 256u + tid;
                    const unsigned int w = q / NU, u = q - w * NU;
                    if (q < NQ && w < nt) {
                        float* yr = &Yw[w * BAY_TR_DPAD + 8u * u];
                        if (sAcc[g][w]) {
                            float y[8];
#pragma unroll
                            for (int i = 0; i < 8; ++i) y[i] = 8u * u + i < DIM ? yr[i] : 0.0f;
                            bay_tr_st8(Xt + (size_t)w * DIM, u, y);
                        } else {
#pragma unroll
                            for (int i = 0; i < 8; ++i)
                                if (8u * u + i < DIM) yr[i] = xv[b][i];
                        }
                    }
                }
            }
        } else {
            // accepted walkers' rows to device memory
            for (unsigned int q = tid; q < NQ; q += 256u) {
                const unsigned int w = q / NU, u = q - w * NU;
                if (w < nt && sAcc[g][w]) {
                    const float* yr = &Yw[w * BAY_TR_DPAD + 8u * u];
                    float y[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) y[i] = 8u * u + i < DIM ? yr[i] : 0.0f;
                    bay_tr_st8(Xt + (size_t)w * DIM, u, y);
                }
            }
        }
        if (ACCU) {
            if (tid == 0 && n_acc) atomicAdd(&P.ctl->accepted, (unsigned long long)n_acc);
            if (PERSIST && P.means_cap != 0) {
                // the statistics of the tile's new positions (Yw) at the end of the tile
                bay_gsync(g);
                float* out = P.part + ((size_t)step_off * 2 + half) * DIM * ntiles + tile;
                for (unsigned int t = tid; t < BAY_TR_NG * DIM; t += 256u) {
                    const unsigned int wg = t / DIM, d = t - wg * DIM;
                    float v = 0.0f;
#pragma unroll
                    for (unsigned int i = 0; i < BAY_TR_WG; ++i) {
                        const unsigned int w = wg * BAY_TR_WG + i;
                        if (w < nt) v = __fadd_rn(v, Yw[w * BAY_TR_DPAD + d]);
                    }
                    if (BAY_TR_NG == 1u) out[(size_t)d * ntiles] = v;
                    else red[t] = v;
                }
                bay_gsync(g);
                bay_tr_sums_pass2(tid, red, out, ntiles);
            }
        }
    }
    if (PERSIST) {
        // the next tile rewrites Yw, red and the A operand, and its MMAs the accumulator
        bay_tc_fence_before();
        bay_gsync(g);
    }
    if (!ok) {
        // a bounded wait gave up: no more tiles; the persistent form raises the abort flag
        // and still meets the next grid barrier, which then stops the whole launch
        if (PERSIST && tid == 0) *(volatile unsigned int*)&P.ctl->abort = 1u;
        break;
    }
    }   // tiles
    }   // halves
    }   // steps
    // 8. release TMEM (every MMA completed before the epilogue read it); the image copy has
    //    landed (a group waited for it, or the bounded wait here)
    if (threadIdx.x == 0) bay_tc_wait(bar_img, 0u, nullptr, status);
    bay_tc_fence_before();
    __syncthreads();
    if (threadIdx.x < 32u) {
        bay_tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(sTmem),
                     "r"(ncols * G) : "memory");
    }
}

// The per-launch move kernels hold BAY_TR_G tile groups per CTA (1 or 2): one matrix-image
// copy and one TMEM allocation serve BAY_TR_G tiles; group g takes tile g * gridDim.x +
// blockIdx.x.  Same results for either.
#ifndef BAY_TR_G
#define BAY_TR_G 1u
#endif
extern "C" __global__ void __launch_bounds__(256 * BAY_TR_G) bay_tcr_bare(bay_stretch_params P) {
    bay_stretch_tcr<false, false, false, BAY_TR_G>(P, 1u);
}
extern "C" __global__ void __launch_bounds__(256 * BAY_TR_G) bay_tcr_accu(bay_stretch_params P) {
    bay_stretch_tcr<true, false, false, BAY_TR_G>(P, 1u);
}
extern "C" __global__ void __launch_bounds__(256) bay_tcr_logfn(bay_stretch_params P) {
    bay_stretch_tcr<false, true, false, 1u>(P, 1u);
}
// the statistics of the last half-step of a chunk (half P.half, step P.step_off): one CTA
// per tile, the same sums as the stretch launches
extern "C" __global__ void __launch_bounds__(256) bay_tcr_stats(bay_stretch_params P) {
    __shared__ float scr[256];
    const unsigned int tile = blockIdx.x, ntiles = gridDim.x, k0 = tile * BAY_TR_W;
    const unsigned int nt = P.K - k0 < BAY_TR_W ? P.K - k0 : BAY_TR_W;
    float* out = P.part + ((size_t)P.step_off * 2 + P.half) * DIM * ntiles + tile;
    bay_tr_sums_pass1(P.xs + (size_t)P.half * P.K * DIM + (size_t)k0 * DIM, nt, threadIdx.x, scr,
                      out, ntiles);
    __syncthreads();
    bay_tr_sums_pass2(threadIdx.x, scr, out, ntiles);
}
// persistent: one CTA of 4 tile groups per SM (1,024 threads, 64 registers each)
extern "C" __global__ void __launch_bounds__(1024, 1) bay_tcr_run_bare(bay_stretch_params P, unsigned int m) {
    bay_stretch_tcr<false, false, true, 4u>(P, m);
}
extern "C" __global__ void __launch_bounds__(1024, 1) bay_tcr_run_accu(bay_stretch_params P, unsigned int m) {
    bay_stretch_tcr<true, false, true, 4u>(P, m);
}
#endif  // BAY_GEMM_TC

#elif !BAY_TILED
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
    float* X = P.xs + (size_t)P.half * P.K * DIM;
    const float* S = P.xs + (size_t)(1u - P.half) * P.K * DIM;
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
            const float s = bay_partner_coord(S, P.K, j, i);
            Y[i] = __fmaf_rn(z, __fsub_rn(X[(size_t)k * DIM + i], s), s);
        }
        const float ly = BAY_LOGFN((unsigned int)P.data_len, P.params_len, P.params, DIM, Y);
        const float lx = P.logfn[(size_t)P.half * P.K + k];
        accepted = bay_accept(u2, z, ly, lx, beta);
        if (accepted) {
#pragma unroll
            for (int i = 0; i < DIM; ++i) X[(size_t)k * DIM + i] = Y[i];
            P.logfn[(size_t)P.half * P.K + k] = ly;
        } else if (ACCU) {
#pragma unroll
            for (int i = 0; i < DIM; ++i) Y[i] = X[(size_t)k * DIM + i];
        }
    }
    if (ACCU) {
        __shared__ float red[BAY_CTA / 32][BAY_SUM_CHUNK];
        bay_accu_epilogue(P, accepted, valid, Y, red, blockIdx.x, gridDim.x);
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
    for (int i = 0; i < DIM; ++i) x[i] = P.xs[(size_t)k * DIM + i];
    P.logfn[k] = BAY_LOGFN((unsigned int)P.data_len, P.params_len, P.params, DIM, x);
}

// Density engines (reference cuda/engines/nvidia-gtx-distribution.cu logpdf/pdf and
// nvidia-gtx-likelihood.cu loglik/lik): the model's density at n points, x dim x n
// column-major (point i's coordinates contiguous); exp_out selects the density itself.
extern "C" __global__ void __launch_bounds__(BAY_CTA)
bay_points_logfn(unsigned long long n, unsigned int data_len, unsigned int params_len,
                 const float* params, const float* x, float* out, unsigned int exp_out) {
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        float p[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) p[d] = x[i * DIM + d];
        const float v = BAY_LOGFN(data_len, params_len, params, DIM, p);
        out[i] = exp_out ? expf(v) : v;
    }
}

// Evidence (nvidia-gtx-likelihood.cu evidence_reduce): per-CTA FP64 sums of exp(density)
// over the points, each thread's points in order, then a fixed-order tree -> part[cta].
extern "C" __global__ void __launch_bounds__(BAY_CTA)
bay_points_evidence(unsigned long long n, unsigned int data_len, unsigned int params_len,
                    const float* params, const float* x, double* part) {
    __shared__ double red[BAY_CTA];
    double s = 0.0;
    for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
         i += (unsigned long long)gridDim.x * blockDim.x) {
        float p[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) p[d] = x[i * DIM + d];
        s += (double)expf(BAY_LOGFN(data_len, params_len, params, DIM, p));
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (unsigned int o = 512; o > 0; o >>= 1) {   // BAY_CTA: any multiple of 32 <= 1024
        if (o < BAY_CTA) {
            if (threadIdx.x < o && threadIdx.x + o < BAY_CTA) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

#else
// ---------------------------------------------------------------- tiled form
// A CTA owns BAY_WPC walkers (a power of two, at most 32) and BAY_CTA threads.  The data
// rows reach shared memory by TMA bulk copies (cp.async.bulk, completion counted on an
// mbarrier; the wait is bounded) in chunks of at most BAY_TILE_CHUNK floats, two chunk
// buffers in flight when the data span more than one.  Thread t works for walker
// t % BAY_WPC on row group t / BAY_WPC: walkers are fastest across lanes, so the lanes of
// one row group read the same row (a shared-memory broadcast), and each thread sums its rows
// in batches of 8 (pairwise) added with a Kahan carry.  The lanes and warps of a walker
// then combine as compensated pairs in a fixed order (deterministic for a given shape).
#ifndef BAY_WPC
#define BAY_WPC 8
#endif
#ifndef BAY_TILE_CHUNK
#define BAY_TILE_CHUNK 12288u                     // floats per staged chunk (48 KB)
#endif
#define BAY_TILE_CHUNK_ROWS ((BAY_TILE_CHUNK / BAY_ROW_LEN) & ~3u)   // 16-byte chunk starts
#define BAY_TILE_WAIT_NS 2000000000ull

__device__ __forceinline__ unsigned long long bay_tile_timer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for phase `par` of the mbarrier at shared address `bar`: gives up after
// BAY_TILE_WAIT_NS and sets status bit 1 (the host reports the shared-memory copy).
__device__ __forceinline__ bool bay_tile_wait(unsigned int bar, unsigned int par,
                                              unsigned int* status) {
    unsigned long long t0 = 0;
    for (unsigned int it = 0;; ++it) {
        unsigned int ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok) : "r"(bar), "r"(par) : "memory");
        if (ok) return true;
        if ((it & 15u) == 0u) {
            const unsigned long long t = bay_tile_timer();
            if (it == 0u) {
                t0 = t;
            } else if (t - t0 > BAY_TILE_WAIT_NS) {
                atomicOr(status, 1u);
                return false;
            }
        }
    }
}

// Chunk c of the rows [rb, rb + n_rows) (rb a multiple of 4) -> buffer `buf` (floats): the
// 16-byte-aligned prefix by one bulk copy completing on `bar`, issued by the calling
// thread.  Returns the chunk's floats.
__device__ __forceinline__ unsigned int bay_tile_issue(const bay_stretch_params& P, unsigned long long c,
                                                       float* buf, unsigned int bar,
                                                       unsigned long long rb, unsigned long long n_rows) {
    const unsigned long long r0 = c * BAY_TILE_CHUNK_ROWS;
    const unsigned long long nr = n_rows - r0 < BAY_TILE_CHUNK_ROWS ? n_rows - r0 : BAY_TILE_CHUNK_ROWS;
    const unsigned int nf = (unsigned int)(nr * BAY_ROW_LEN);
    const unsigned int bytes = (nf * 4u) & ~15u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
    if (bytes)
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
            ::"r"((unsigned int)__cvta_generic_to_shared(buf)), "l"(P.params + (rb + r0) * BAY_ROW_LEN),
            "r"(bytes), "r"(bar) : "memory");
    return nf;
}

// The chunk buffers' barriers and the CTA's verdict on its copies.
struct bay_tile_sync {
    unsigned long long bar[2];
    unsigned int ok;
};

// Thread 0: the chunk barriers and the first two chunks' copies.  The data never change
// while a sampler runs, so this may run before the launch waits for its predecessor.  The
// CTA's threads wait on the barriers only after a __syncthreads that follows this.
__device__ __forceinline__ void bay_tile_begin(const bay_stretch_params& P, bay_tile_sync* sy,
                                               unsigned long long rb, unsigned long long n_rows) {
    extern __shared__ __align__(128) float bay_tsm[];
    if (threadIdx.x != 0) return;
    const unsigned long long nch = (n_rows + BAY_TILE_CHUNK_ROWS - 1) / BAY_TILE_CHUNK_ROWS;
    const unsigned int bar0 = (unsigned int)__cvta_generic_to_shared(&sy->bar[0]);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8u) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    sy->ok = 1u;
    for (unsigned long long c = 0; c < 2 && c < nch; ++c)
        bay_tile_issue(P, c, bay_tsm + (unsigned int)c * BAY_TILE_CHUNK, bar0 + 8u * (unsigned int)c,
                       rb, n_rows);
}

// Sum over all data rows of BAY_TILE_TERM(row, prep of walker w) for the CTA's walkers
// w < BAY_WPC (prep: [BAY_WPC][BAY_PREP_LEN] in shared memory) -> out[w] (compensated
// pairs), the copies begun by bay_tile_begin.  Every thread of the CTA calls it.  Returns
// false (and sets the status) when a bounded wait for a copy gave up; out is then
// incomplete.
// With BAY_TILE_TERM4 (the model's row term over bay_v4) and BAY_WPC a multiple of 4, a
// thread serves the four walkers 4 s .. 4 s + 3 of walker slot s = t % (BAY_WPC / 4) on row
// group t / (BAY_WPC / 4): one row load per four walkers, four times the row groups.
#if defined(BAY_TILE_TERM4) && (BAY_WPC % 4 == 0)
#define BAY_TILE_VEC 1
typedef bay_v4 bay_tval;
#define BAY_TVAL_ZERO {0.0f, 0.0f, 0.0f, 0.0f}
#define BAY_TVAL_ADD(a, b) bay_v4_add_rn(a, b)
#define BAY_TVAL_SUB(a, b) bay_v4_sub_rn(a, b)
#define BAY_TVAL_TERM(row, pv) BAY_TILE_TERM4(row, pv)
#else
#define BAY_TILE_VEC 0
typedef float bay_tval;
#define BAY_TVAL_ZERO 0.0f
#define BAY_TVAL_ADD(a, b) __fadd_rn(a, b)
#define BAY_TVAL_SUB(a, b) __fsub_rn(a, b)
#define BAY_TVAL_TERM(row, pv) BAY_TILE_TERM(row, pv)
#endif
__device__ __forceinline__ bool bay_tiled_logfn_rows(const bay_stretch_params& P,
                                                    const float (*prep)[BAY_PREP_LEN],
                                                    bay_cf (*red)[BAY_WPC], bay_cf* out,
                                                    bay_tile_sync* sy, unsigned long long rb,
                                                    unsigned long long n_rows) {
    extern __shared__ __align__(128) float bay_tsm[];
    unsigned int& sOk = sy->ok;
    constexpr unsigned int WV = BAY_TILE_VEC ? 4u : 1u;     // walkers per thread
    constexpr unsigned int WS = BAY_WPC / WV;               // walker slots
    constexpr unsigned int L = BAY_CTA / WS;                // row groups
    const unsigned int tid = threadIdx.x, w = tid % WS, l = tid / WS;
    const unsigned long long nch = (n_rows + BAY_TILE_CHUNK_ROWS - 1) / BAY_TILE_CHUNK_ROWS;
    const unsigned int bar0 = (unsigned int)__cvta_generic_to_shared(&sy->bar[0]);
#if BAY_TILE_VEC
    bay_v4 pv[BAY_PREP_LEN];
#pragma unroll
    for (int i = 0; i < BAY_PREP_LEN; ++i)
        pv[i] = {prep[4u * w][i], prep[4u * w + 1u][i], prep[4u * w + 2u][i], prep[4u * w + 3u][i]};
#else
    float pv[BAY_PREP_LEN];
#pragma unroll
    for (int i = 0; i < BAY_PREP_LEN; ++i) pv[i] = prep[w][i];
#endif
    bay_tval sum = BAY_TVAL_ZERO, cmp = BAY_TVAL_ZERO;
    for (unsigned long long c = 0; c < nch; ++c) {
        const unsigned int b = (unsigned int)(c & 1ull);
        float* R = bay_tsm + b * BAY_TILE_CHUNK;
        const unsigned long long r0 = c * BAY_TILE_CHUNK_ROWS;
        const unsigned int nr = (unsigned int)(n_rows - r0 < BAY_TILE_CHUNK_ROWS ? n_rows - r0
                                                                              : BAY_TILE_CHUNK_ROWS);
        const unsigned int nf = nr * BAY_ROW_LEN, nb = ((nf * 4u) & ~15u) / 4u;
        const bool done = bay_tile_wait(bar0 + 8u * b, (unsigned int)((c >> 1) & 1ull), &P.ctl->status);
        if (!done) sOk = 0u;
        if (nb < nf) {   // the chunk's last floats past its 16-byte-aligned prefix
            for (unsigned int e = nb + tid; e < nf; e += BAY_CTA) R[e] = P.params[(rb + r0) * BAY_ROW_LEN + e];
        }
        __syncthreads();
        if (sOk == 0u) break;
        unsigned int r = l;
        for (; r + 7u * L < nr; r += 8u * L) {
            bay_tval t[8];
#pragma unroll
            for (unsigned int i = 0; i < 8u; ++i) t[i] = BAY_TVAL_TERM(R + (r + i * L) * BAY_ROW_LEN, pv);
#pragma unroll
            for (unsigned int h = 4u; h >= 1u; h >>= 1)
#pragma unroll
                for (unsigned int i = 0; i < h; ++i) t[i] = BAY_TVAL_ADD(t[i], t[i + h]);
            const bay_tval y = BAY_TVAL_SUB(t[0], cmp);
            const bay_tval s2 = BAY_TVAL_ADD(sum, y);
            cmp = BAY_TVAL_SUB(BAY_TVAL_SUB(s2, sum), y);
            sum = s2;
        }
        for (; r < nr; r += L) {
            const bay_tval y = BAY_TVAL_SUB(BAY_TVAL_TERM(R + r * BAY_ROW_LEN, pv), cmp);
            const bay_tval s2 = BAY_TVAL_ADD(sum, y);
            cmp = BAY_TVAL_SUB(BAY_TVAL_SUB(s2, sum), y);
            sum = s2;
        }
        __syncthreads();                                // buffer b is free again
        if (tid == 0 && c + 2 < nch) bay_tile_issue(P, c + 2, R, bar0 + 8u * b, rb, n_rows);
    }
    const bool ok = sOk != 0u;
    // the lanes of a walker slot (lane bits above the slot bits) by an xor butterfly, then
    // the warps in order; walker 4 s + j of slot s at red[warp][4 s + j] (vector path)
    const unsigned int lane = tid & 31u, warp = tid >> 5;
#pragma unroll
    for (unsigned int j = 0; j < WV; ++j) {
        bay_cf v;
#if BAY_TILE_VEC
        v.hi = j == 0u ? sum.x : j == 1u ? sum.y : j == 2u ? sum.z : sum.w;
        v.lo = -(j == 0u ? cmp.x : j == 1u ? cmp.y : j == 2u ? cmp.z : cmp.w);
#else
        v.hi = sum;
        v.lo = -cmp;
#endif
#pragma unroll
        for (unsigned int o = 16u; o >= WS && o >= 1u; o >>= 1) v = bay_cadd(v, bay_cf_shfl_xor(v, o));
        if (lane < WS) red[warp][WV * lane + j] = v;
    }
    __syncthreads();
    if (tid < BAY_WPC) {
        bay_cf s = red[0][tid];
        for (unsigned int i = 1; i < BAY_CTA / 32u; ++i) s = bay_cadd(s, red[i][tid]);
        out[tid] = s;
    }
    __syncthreads();
    return ok;
}

template <bool ACCU>
__device__ __forceinline__ void bay_stretch_tiled(const bay_stretch_params& P) {
    const unsigned int kind = ACCU ? 1u : 0u;
    __shared__ float sY[BAY_WPC][DIM];
    __shared__ float sPrep[BAY_WPC][BAY_PREP_LEN];
    __shared__ float sW[BAY_WPC], sZ[BAY_WPC], sU2[BAY_WPC];
    __shared__ bay_cf sRed[BAY_CTA / 32][BAY_WPC];
    __shared__ bay_cf sSum[BAY_WPC];
    __shared__ float red1[BAY_CTA / 32][BAY_SUM_CHUNK];
    const unsigned int step = P.ctl->step[kind] + P.step_off;
    const unsigned int seed = P.ctl->seed[kind] + P.half;
    const float a = P.ctl->a;
    const float beta = ACCU ? 1.0f : P.ctl->beta;
    const unsigned int stream = ACCU ? (P.half ? 2222u : 1111u) : (P.half ? 4444u : 3333u);
    float* X = P.xs + (size_t)P.half * P.K * DIM;
    const float* S = P.xs + (size_t)(1u - P.half) * P.K * DIM;
    const float* hyper = P.params + P.data_len;
    // walker group g and row slice sl (slice-major CTAs); slices start on 4-row boundaries
    const unsigned int NS = P.t_slices, groups = gridDim.x / NS;
    const unsigned int g = blockIdx.x % groups, sl = blockIdx.x / groups;
    const unsigned int k0 = g * BAY_WPC;
    const unsigned long long n_rows = P.data_len / BAY_ROW_LEN;
    const unsigned long long rps = NS > 1u ? (((n_rows + NS - 1u) / NS + 3ull) & ~3ull) : n_rows;
    const unsigned long long rb = (unsigned long long)sl * rps < n_rows ? (unsigned long long)sl * rps : n_rows;
    const unsigned long long rn = n_rows - rb < rps ? n_rows - rb : rps;
    __shared__ bay_tile_sync sSync;
    bay_tile_begin(P, &sSync, rb, rn);
    // Launched with programmatic dependent launch: the draws, the walker's own row and log
    // density (this half last moved two launches back, final once the previous launch began
    // its work, which it did only after waiting for its own predecessor) come before the
    // wait for the previous launch; the partner row, from the half that launch moves, after.
    const unsigned int t0 = threadIdx.x, kk = k0 + t0;
    const bool mine_ok = t0 < BAY_WPC && kk < P.K;
    float xr[DIM], z = 0.0f, u2 = 0.0f;
    unsigned int j = 0;
    if (mine_ok) {
        bay_u4 c;
        c.x = kk;
        c.y = step;
        c.z = stream;
        c.w = 0xbeeff00du;
        const bay_u4 r = bay_philox4x32_10(c, seed, 0xdecafbadu);
        z = bay_stretch_z(a, bay_u01(r.y));
        j = bay_partner(bay_u01(r.x), P.K);
        u2 = bay_u01(r.z);
#pragma unroll
        for (int i = 0; i < DIM; ++i) xr[i] = X[(size_t)kk * DIM + i];
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

    if (threadIdx.x < BAY_WPC) {
        const unsigned int t = threadIdx.x, k = k0 + t;
        if (k < P.K) {
            float Y[DIM];
#pragma unroll
            for (int i = 0; i < DIM; ++i) {
                const float s = bay_partner_coord(S, P.K, j, i);
                Y[i] = __fmaf_rn(z, __fsub_rn(xr[i], s), s);
                sY[t][i] = Y[i];
            }
            float pr[BAY_PREP_LEN];
            BAY_TILE_PREP(hyper, P.params_len, DIM, Y, pr);
#pragma unroll
            for (int i = 0; i < BAY_PREP_LEN; ++i) sPrep[t][i] = pr[i];
            sW[t] = BAY_TILE_WALKER(n_rows, hyper, P.params_len, DIM, Y);
            sZ[t] = z;
            sU2[t] = u2;
        } else {
#pragma unroll
            for (int i = 0; i < BAY_PREP_LEN; ++i) sPrep[t][i] = 0.0f;
            sW[t] = 0.0f;
        }
    }
    __syncthreads();
    bool ok = bay_tiled_logfn_rows(P, sPrep, sRed, sSum, &sSync, rb, rn);
    bool accepted = false;
    const unsigned int t = threadIdx.x, k = k0 + t;
    const bool valid = t < BAY_WPC && k < P.K;
    if (NS > 1u) {
        // leave this slice's partials (NaN after a failed copy: the walker is then
        // rejected), take the group's ticket; the last slice combines them in slice order
        __shared__ unsigned int sLast;
        float2* part = reinterpret_cast<float2*>(P.t_part);
        if (valid) part[(size_t)k * NS + sl] = ok ? make_float2(sSum[t].hi, sSum[t].lo)
                                                 : make_float2(__int_as_float(0x7fc00000), 0.0f);
        __threadfence();
        __syncthreads();
        if (t == 0) sLast = atomicAdd(&P.t_ticket[g], 1u) == NS - 1u ? 1u : 0u;
        __syncthreads();
        if (sLast == 0u) return;
        __threadfence();
        if (t == 0) P.t_ticket[g] = 0u;             // for the next launch
        if (valid) {
            bay_cf a;
            a.hi = 0.0f;
            a.lo = 0.0f;
            for (unsigned int q = 0; q < NS; ++q) {
                const float2 v = __ldcg(&part[(size_t)k * NS + q]);
                bay_cf b;
                b.hi = v.x;
                b.lo = v.y;
                a = bay_cadd(a, b);
            }
            sSum[t] = a;
        }
        ok = true;
        __syncthreads();
    }
    float mine[DIM];
    if (valid) {
        if (ok) {
            const float ly = bay_cf_total(sW[t], sSum[t]);
            const float lx = P.logfn[(size_t)P.half * P.K + k];
            accepted = bay_accept(sU2[t], sZ[t], ly, lx, beta);
            if (accepted) {
#pragma unroll
                for (int i = 0; i < DIM; ++i) X[(size_t)k * DIM + i] = sY[t][i];
                P.logfn[(size_t)P.half * P.K + k] = ly;
            }
        }
        if (ACCU) {
#pragma unroll
            for (int i = 0; i < DIM; ++i) mine[i] = accepted ? sY[t][i] : X[(size_t)k * DIM + i];
        }
    }
    if (ACCU) bay_accu_epilogue(P, accepted, valid, mine, red1, g, groups);
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
    __shared__ bay_cf sRed[BAY_CTA / 32][BAY_WPC];
    __shared__ bay_cf sSum[BAY_WPC];
    const float* hyper = P.params + P.data_len;
    const unsigned long long n_rows = P.data_len / BAY_ROW_LEN;
    const unsigned int k0 = blockIdx.x * BAY_WPC;
    __shared__ bay_tile_sync sSync;
    bay_tile_begin(P, &sSync, 0ull, n_rows);
    if (threadIdx.x < BAY_WPC) {
        const unsigned int t = threadIdx.x, k = k0 + t;
        if (k < P.W) {
            float x[DIM];
#pragma unroll
            for (int i = 0; i < DIM; ++i) x[i] = P.xs[(size_t)k * DIM + i];
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
    const bool ok = bay_tiled_logfn_rows(P, sPrep, sRed, sSum, &sSync, 0ull, n_rows);
    const unsigned int t = threadIdx.x, k = k0 + t;
    if (ok && t < BAY_WPC && k < P.W) P.logfn[k] = bay_cf_total(sW[t], sSum[t]);
}
#endif
