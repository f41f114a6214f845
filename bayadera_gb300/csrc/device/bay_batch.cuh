// bay_batch.cuh -- batched stretch moves: many independent models of one model family
// (one NVRTC compile), each member with its own dimension, walkers, data, hyperparameters
// and seed, advanced together.  Compiled by NVRTC per model family with bay_rng.cuh and
// the model source in front.
//
// A half-step of every member is three launches over work lists the host builds once:
//   propose: CTA = (member, 256-walker tile): Philox draw with the member's seed and the
//            single-sampler counter {k, step, stream, 0xbeeff00d}, stretch factor, partner
//            from the member's other half, the proposal y -> scratch (coalesced over the
//            tile's contiguous block), per-walker prep and the terms outside the row sum;
//   rows:    CTA = (member, tile of wpc walkers, chunk of rows): the chunk of rows and the
//            walkers' proposals are staged in shared memory, then each of 256 / wpc lanes
//            per walker sums the row terms of its rows (walkers fastest, so a warp reads
//            one row as a broadcast) in pairwise batches with a Kahan carry; lanes combine
//            by an xor butterfly and in warp order -> a compensated partial per (walker,
//            chunk).  wpc and the chunk size are chosen per member so that every item
//            carries about the same work, which balances members whose data differ by
//            orders of magnitude;
//   accept:  CTA = (member, 256-walker tile): partials summed in chunk order, log-space
//            accept (bay_accept_log), write-back; accu: accepted count per member, per-CTA per-dim sums.
// Counter and key words per member are those of a single sampler with the member's seed,
// so a member's trajectory is the trajectory that sampler would take (up to the order of
// the log-density sums).
//
// Model ABI (row form, runtime dimension):
//   void BAY_TILE_PREP(const REAL* hyper, uint32_t hyper_len, uint32_t dim, const REAL* x,
//                      REAL* prep)                          BAY_PREP_LEN values per walker
//   REAL BAY_TILE_TERM(const REAL* row, const REAL* x, const REAL* prep)    one data row
//   REAL BAY_TILE_WALKER(uint64_t n_rows, const REAL* hyper, uint32_t hyper_len,
//                        uint32_t dim, const REAL* x)       every term not summed over rows
// log density = walker(x) + sum over the member's rows of term(row, x, prep(x)); a member's
// params are rows (BAY_ROW_LEN floats each) followed by hyper_len hyperparameters.

#ifndef BAY_PREP_LEN
#define BAY_PREP_LEN 1
#endif
// staged rows: BAY_ROW_LEN floats padded to a 16-byte stride, one vector load per row
#define BAY_ROW_STRIDE ((BAY_ROW_LEN + 3) & ~3)

struct bay_ctl {
    unsigned int step[2];
    unsigned int seed[2];
    float a;
    float beta;
    unsigned int ticket[2];
    unsigned long long accepted;
    unsigned int status;
    unsigned int pad0[21];
    unsigned int gbar_count;   // byte 128
    unsigned int pad1[31];
    unsigned int abort;        // byte 256
    unsigned int pad2[31];
};

// per member (host-built, read-only on the device)
struct bay_bmember {
    unsigned long long xs;        // float offset of the member's positions, W x dim
    unsigned long long params;    // float offset of its rows || hyperparameters
    unsigned long long rows;      // data rows
    unsigned long long part;      // float offset of its partials, W x chunks x 2
    unsigned long long dsum;      // float offset of its per-CTA dim sums, tiles x dim
    unsigned long long means;     // float offset of its per-step means, cap x dim
    unsigned int dim, W, K, hyper_len;
    unsigned int walker0;         // first walker of the member in the per-walker arrays
    unsigned int chunks, chunk_rows;
    unsigned int tile0;           // first move tile (accept CTA) of the member
    unsigned int ntiles;          // move tiles of the member
    unsigned int pad[3];
};
struct bay_bitem { unsigned int m, k0, c, wpc; };   // rows work item
struct bay_btile { unsigned int m, k0; };           // propose / accept CTA

struct bay_batch_params {
    const bay_bmember* mem;
    const bay_bitem* items;
    const bay_btile* tiles;
    const unsigned int* seeds;    // [member][2]: bare, accu
    const float* params;
    float* xs;
    float* y;                     // proposals, laid out like xs
    float* logfn;                 // [walker0 + w]
    float* prep;                  // [walker0 + k][BAY_PREP_LEN]
    float* wterm;                 // [walker0 + k]
    float* zu;                    // [walker0 + k][2]
    float* part;
    unsigned long long* accepted; // [member]
    float* dsum;                  // [step_off * 2 + half][dsum_stride]
    float* means;
    bay_ctl* ctl;
    unsigned long long dsum_stride;
    unsigned int half, step_off, means_cap, n_members;
    unsigned int n_tiles, n_items;  // move tiles and rows work items (the persistent launch)
    unsigned int gbar_extra;        // persistent launch: extra arrivals its barriers wait for
                                    // (0; 1 makes them run out, for tests)
    unsigned int pad;
};

// log u <= (dim - 1) log z + beta (ly - lx) in fp32 with bay_log_det (bay_accept_log); a
// non-finite proposal is rejected
__device__ __forceinline__ bool bay_batch_accept(float u2, float z, float ly, float lx,
                                                 float beta, unsigned int dim) {
    return bay_accept_log(u2, z, ly, lx, beta, dim - 1);
}

struct bay_bcf {
    float hi, lo;
};
__device__ __forceinline__ bay_bcf bay_bcadd(bay_bcf a, bay_bcf b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    const float lo = __fadd_rn(__fadd_rn(a.lo, b.lo), e);
    const float hi = __fadd_rn(s, lo);
    bay_bcf r;
    r.hi = hi;
    r.lo = __fsub_rn(lo, __fsub_rn(hi, s));
    return r;
}

#ifndef BAY_STRETCH_REF
#define BAY_STRETCH_REF 0
#endif
__device__ __forceinline__ float bay_stretch_z(float a, float u1) {
    // the stretch kernels' form (device/bay_stretch.cuh): fixed operation order, 1/a IEEE
    // or, with BAY_STRETCH_REF, the fast division of the reference's build
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
    unsigned int j = __float2uint_rz(__fmul_rn(u0, (float)K));
    return j < K ? j : K - 1;
}

// e / dim for e < 2^24 from a float reciprocal, corrected to the exact quotient (the float
// product is within 1 of it): a few instructions instead of an integer division.
__device__ __forceinline__ unsigned int bay_div_dim(unsigned int e, unsigned int dim, float inv_dim) {
    unsigned int q = __float2uint_rz(__fmul_rn((float)e, inv_dim));
    if (q * dim > e) --q;
    else if ((q + 1u) * dim <= e) ++q;
    return q;
}

template <int MODE>  // 0 bare, 1 accu, 2 log density of the current positions (all W)
__device__ __forceinline__ void bay_batch_propose_impl(const bay_batch_params& P, unsigned int idx) {
    __shared__ float sZ[256];
    __shared__ unsigned int sJ[256];
    const bay_btile T = P.tiles[idx];
    const bay_bmember& M = P.mem[T.m];
    const unsigned int nk = MODE == 2 ? M.W : M.K;
    const unsigned int dim = M.dim;
    const unsigned int tid = threadIdx.x;
    const unsigned int k = T.k0 + tid;
    const unsigned int nt = nk - T.k0 < 256u ? nk - T.k0 : 256u;   // walkers of the tile
    const unsigned int kind = MODE == 1 ? 1u : 0u;
    if (MODE != 2 && tid < nt) {
        const unsigned int stream = MODE == 1 ? (P.half ? 2222u : 1111u) : (P.half ? 4444u : 3333u);
        bay_u4 c;
        c.x = k;
        c.y = P.ctl->step[kind] + P.step_off;
        c.z = stream;
        c.w = 0xbeeff00du;
        const bay_u4 r = bay_philox4x32_10(c, P.seeds[2 * T.m + kind] + P.half, 0xdecafbadu);
        const float z = bay_stretch_z(P.ctl->a, bay_u01(r.y));
        sZ[tid] = z;
        sJ[tid] = bay_partner(bay_u01(r.x), M.K);
        P.zu[2 * ((size_t)M.walker0 + k)] = z;
        P.zu[2 * ((size_t)M.walker0 + k) + 1] = bay_u01(r.z);
    }
    __syncthreads();
    // the tile's proposals: one contiguous block of nt * dim floats, element-wise
    // (plain loads, not the read-only path: the persistent launch rewrites the positions
    // between its phases; the proposals are a separate buffer, hence __restrict__)
    float* __restrict__ Y = P.y + M.xs + (size_t)T.k0 * dim;
    const float* __restrict__ X = P.xs + M.xs + (MODE == 2 ? 0 : (size_t)P.half * M.K * dim) + (size_t)T.k0 * dim;
    const float* __restrict__ S = P.xs + M.xs + (size_t)(1u - P.half) * M.K * dim;
    const unsigned int ne = nt * dim;
    const float inv_dim = __frcp_rn((float)dim);
    // 8 elements per thread per pass, all their loads issued before any is used
    for (unsigned int e0 = tid; e0 < ne; e0 += 8u * blockDim.x) {
        float xv[8], sv[8], zv[8];
#pragma unroll
        for (unsigned int i = 0; i < 8u; ++i) {
            const unsigned int e = e0 + i * blockDim.x;
            xv[i] = 0.0f;
            sv[i] = 0.0f;
            zv[i] = 0.0f;
            if (e < ne) {
                xv[i] = X[e];
                if (MODE != 2) {
                    const unsigned int w = bay_div_dim(e, dim, inv_dim), d = e - w * dim;
                    sv[i] = S[(size_t)sJ[w] * dim + d];
                    zv[i] = sZ[w];
                }
            }
        }
#pragma unroll
        for (unsigned int i = 0; i < 8u; ++i) {
            const unsigned int e = e0 + i * blockDim.x;
            if (e < ne) Y[e] = MODE == 2 ? xv[i] : __fmaf_rn(zv[i], __fsub_rn(xv[i], sv[i]), sv[i]);
        }
    }
    __syncthreads();
    if (tid < nt) {
        const float* y = Y + (size_t)tid * dim;
        const float* hyper = P.params + M.params + M.rows * BAY_ROW_LEN;
        float pr[BAY_PREP_LEN];
#pragma unroll
        for (int i = 0; i < BAY_PREP_LEN; ++i) pr[i] = 0.0f;
        BAY_TILE_PREP(hyper, M.hyper_len, dim, y, pr);
#pragma unroll
        for (int i = 0; i < BAY_PREP_LEN; ++i) P.prep[((size_t)M.walker0 + k) * BAY_PREP_LEN + i] = pr[i];
        P.wterm[(size_t)M.walker0 + k] = BAY_TILE_WALKER(M.rows, hyper, M.hyper_len, dim, y);
    }
}

// WPT walkers per thread (1, 2 or 4): thread t serves walkers tw, tw + TPR, ..., tw + (WPT -
// 1) TPR of the item (TPR = wpc / WPT threads per row group, tw = t % TPR) on row group
// t / TPR, so one staged row -- one broadcast load, and whatever the model derives from the
// row alone -- serves WPT walkers.  Each walker's sum has the same structure for any WPT
// (its rows split over L = 256 / TPR row groups, batches of 8 pairwise with a Kahan carry,
// the row groups combined in xor-butterfly then warp order), so results depend on WPT only
// through L.
// With 4 walkers per thread and a model that also writes its row term over bay_v4
// (BAY_BATCH_TERM4), the thread's walkers are 4 tw .. 4 tw + 3 instead, stored interleaved
// ([wpc / 4][dpad][4]: coordinate i of the four at one 16-byte address), and the term runs
// once per row for all four -- one coordinate load where the scalar path makes four.  Each
// walker's operations and sum order are those of the scalar path.
#ifdef BAY_BATCH_TERM4
#define BAY_HAS_TERM4 1
#else
#define BAY_HAS_TERM4 0
#endif
template <int MODE, unsigned int WPT>  // MODE 0: move (K walkers), 2: log density of all W
__device__ __forceinline__ void bay_batch_rows_impl(const bay_batch_params& P, unsigned int idx) {
    extern __shared__ __align__(16) float bay_bsm[];
    const bay_bitem I = P.items[idx];
    const bay_bmember& M = P.mem[I.m];
    const unsigned int nk = MODE == 2 ? M.W : M.K;
    const unsigned int dim = M.dim, wpc = I.wpc, tid = threadIdx.x;
    const unsigned long long r0 = (unsigned long long)I.c * M.chunk_rows;
    const unsigned int nr = (unsigned int)(r0 + M.chunk_rows < M.rows ? M.chunk_rows : M.rows - r0);
    const unsigned int dpad = dim | 1u;   // odd walker stride: the lanes' x[j] hit distinct banks
    constexpr bool VEC = WPT == 4u && BAY_HAS_TERM4;
    float* Ys = bay_bsm;                                    // [wpc][dpad] or [wpc / 4][dpad][4]
    float* Pr = Ys + ((wpc * dpad + 3u) & ~3u);                        // [wpc][BAY_PREP_LEN]
    float* Rs = Pr + ((wpc * BAY_PREP_LEN + 3u) & ~3u);                // [nr][BAY_ROW_STRIDE]
    float* red = Rs + M.chunk_rows * BAY_ROW_STRIDE;                   // [256][WPT][2]
    const unsigned int nv = nk - I.k0 < wpc ? nk - I.k0 : wpc;   // walkers of the item
    // stage the item's walkers, their prep values and its chunk of rows (coalesced,
    // every load issued before any is used)
    const float* Yg = P.y + M.xs + (size_t)I.k0 * dim;
    {
        // warp by warp, no division by the runtime dimension: one walker per warp pass
        // (lanes over its coordinates), or on the vector path four walkers per pass (lanes
        // over (coordinate, walker): consecutive shared-memory words, four row segments)
        const unsigned int lane = tid & 31u, nw = blockDim.x >> 5;
        if (VEC) {
            for (unsigned int G = tid >> 5; G < (wpc >> 2); G += nw)
                for (unsigned int e = lane; e < 4u * dim; e += 32u) {
                    const unsigned int d = e >> 2, ww = 4u * G + (e & 3u);
                    Ys[(G * dpad + d) * 4u + (e & 3u)] = ww < nv ? Yg[(size_t)ww * dim + d] : 0.0f;
                }
        } else {
            for (unsigned int ww = tid >> 5; ww < wpc; ww += nw)
                for (unsigned int d = lane; d < dim; d += 32u)
                    Ys[ww * dpad + d] = ww < nv ? Yg[(size_t)ww * dim + d] : 0.0f;
        }
    }
    for (unsigned int e = tid; e < wpc * BAY_PREP_LEN; e += blockDim.x) {
        const float v = e < nv * BAY_PREP_LEN ? P.prep[((size_t)M.walker0 + I.k0) * BAY_PREP_LEN + e] : 0.0f;
        const unsigned int ww = e / BAY_PREP_LEN, i = e - ww * BAY_PREP_LEN;
        if (VEC) Pr[((ww >> 2) * BAY_PREP_LEN + i) * 4u + (ww & 3u)] = v;
        else Pr[e] = v;
    }
    const float* Rg = P.params + M.params + r0 * BAY_ROW_LEN;
    // a row per thread: its BAY_ROW_LEN floats (adjacent lanes, adjacent rows: every byte
    // of the loaded sectors used), stored as 16-byte words (padding zero)
#pragma unroll 2
    for (unsigned int rr = tid; rr < nr; rr += blockDim.x) {
        const float* src = Rg + (size_t)rr * BAY_ROW_LEN;
        float v[BAY_ROW_STRIDE];
#pragma unroll
        for (int i = 0; i < BAY_ROW_STRIDE; ++i) v[i] = i < BAY_ROW_LEN ? __ldg(src + i) : 0.0f;
#pragma unroll
        for (int q = 0; q < BAY_ROW_STRIDE / 4; ++q)
            *reinterpret_cast<float4*>(Rs + rr * BAY_ROW_STRIDE + 4 * q) =
                make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    }
    __syncthreads();
    // walkers fastest: a warp's lanes are up to 32 walkers on the same row (a broadcast)
    const unsigned int TPR = wpc / WPT;                 // threads per row group
    const unsigned int L = blockDim.x / TPR, tw = tid % TPR, l = tid / TPR;
    float sum[WPT], cmp[WPT];
    const float* xw[WPT];
    const float* pw[WPT];
#pragma unroll
    for (unsigned int j = 0; j < WPT; ++j) {
        sum[j] = 0.0f;
        cmp[j] = 0.0f;
        xw[j] = Ys + (tw + j * TPR) * dpad;
        pw[j] = Pr + (tw + j * TPR) * BAY_PREP_LEN;
    }
#if BAY_HAS_TERM4
    if constexpr (VEC) {
        // the four walkers 4 tw .. 4 tw + 3 (zero rows past nv, their sums dropped)
        const bay_v4* x4 = reinterpret_cast<const bay_v4*>(Ys) + tw * dpad;
        const bay_v4* p4 = reinterpret_cast<const bay_v4*>(Pr) + tw * BAY_PREP_LEN;
        bay_v4 s4 = {0.0f, 0.0f, 0.0f, 0.0f}, c4 = {0.0f, 0.0f, 0.0f, 0.0f};
        if (4u * tw < nv) {
            unsigned int r = l;
            for (; r + 7u * L < nr; r += 8u * L) {
                bay_v4 t[8];
#pragma unroll
                for (unsigned int i = 0; i < 8u; ++i) {
                    float rv[BAY_ROW_STRIDE];
                    const float4* rp = reinterpret_cast<const float4*>(Rs + (r + i * L) * BAY_ROW_STRIDE);
#pragma unroll
                    for (int q = 0; q < BAY_ROW_STRIDE / 4; ++q) {
                        const float4 v4 = rp[q];
                        rv[4 * q] = v4.x;
                        rv[4 * q + 1] = v4.y;
                        rv[4 * q + 2] = v4.z;
                        rv[4 * q + 3] = v4.w;
                    }
                    t[i] = BAY_BATCH_TERM4(rv, x4, p4);
                }
#pragma unroll
                for (unsigned int h = 4u; h >= 1u; h >>= 1)
#pragma unroll
                    for (unsigned int i = 0; i < h; ++i) t[i] = bay_v4_add_rn(t[i], t[i + h]);
                const bay_v4 yk = bay_v4_sub_rn(t[0], c4);
                const bay_v4 s2 = bay_v4_add_rn(s4, yk);
                c4 = bay_v4_sub_rn(bay_v4_sub_rn(s2, s4), yk);
                s4 = s2;
            }
            for (; r < nr; r += L) {
                const bay_v4 yk = bay_v4_sub_rn(BAY_BATCH_TERM4(Rs + r * BAY_ROW_STRIDE, x4, p4), c4);
                const bay_v4 s2 = bay_v4_add_rn(s4, yk);
                c4 = bay_v4_sub_rn(bay_v4_sub_rn(s2, s4), yk);
                s4 = s2;
            }
        }
        sum[0] = s4.x; sum[1 % WPT] = s4.y; sum[2 % WPT] = s4.z; sum[3 % WPT] = s4.w;
        cmp[0] = c4.x; cmp[1 % WPT] = c4.y; cmp[2 % WPT] = c4.z; cmp[3 % WPT] = c4.w;
    } else
#endif
    if (tw < nv) {      // walkers past nv are zero rows in Ys/Pr: their sums are dropped
        unsigned int r = l;
        // batches of 8 rows summed pairwise per walker, each batch added with Kahan
        // compensation; a row comes to registers as BAY_ROW_STRIDE / 4 vector loads
        for (; r + 7u * L < nr; r += 8u * L) {
            float t[WPT][8];
#pragma unroll
            for (unsigned int i = 0; i < 8u; ++i) {
                float rv[BAY_ROW_STRIDE];
                const float4* rp = reinterpret_cast<const float4*>(Rs + (r + i * L) * BAY_ROW_STRIDE);
#pragma unroll
                for (int q = 0; q < BAY_ROW_STRIDE / 4; ++q) {
                    const float4 v4 = rp[q];
                    rv[4 * q] = v4.x;
                    rv[4 * q + 1] = v4.y;
                    rv[4 * q + 2] = v4.z;
                    rv[4 * q + 3] = v4.w;
                }
#pragma unroll
                for (unsigned int j = 0; j < WPT; ++j) t[j][i] = BAY_TILE_TERM(rv, xw[j], pw[j]);
            }
#pragma unroll
            for (unsigned int j = 0; j < WPT; ++j) {
#pragma unroll
                for (unsigned int h = 4u; h >= 1u; h >>= 1)
#pragma unroll
                    for (unsigned int i = 0; i < h; ++i) t[j][i] = __fadd_rn(t[j][i], t[j][i + h]);
                const float yk = __fsub_rn(t[j][0], cmp[j]);
                const float s2 = __fadd_rn(sum[j], yk);
                cmp[j] = __fsub_rn(__fsub_rn(s2, sum[j]), yk);
                sum[j] = s2;
            }
        }
        for (; r < nr; r += L) {
#pragma unroll
            for (unsigned int j = 0; j < WPT; ++j) {
                const float yk = __fsub_rn(BAY_TILE_TERM(Rs + r * BAY_ROW_STRIDE, xw[j], pw[j]), cmp[j]);
                const float s2 = __fadd_rn(sum[j], yk);
                cmp[j] = __fsub_rn(__fsub_rn(s2, sum[j]), yk);
                sum[j] = s2;
            }
        }
    }
    // combine the lanes of each walker: inside a warp by an xor butterfly over the lane
    // bits above the walker bits (bay_bcadd is symmetric, so every lane of a walker ends
    // with the same bits), then across warps in warp order
    const unsigned int lane = tid & 31u, warp = tid >> 5;
    const unsigned int tpw = TPR < 32u ? TPR : 32u;   // walker slots per warp
#pragma unroll
    for (unsigned int j = 0; j < WPT; ++j) {
        bay_bcf v;
        v.hi = sum[j];
        v.lo = -cmp[j];
        for (unsigned int o = 16u; o >= TPR && o >= 1u; o >>= 1) {
            bay_bcf u;
            u.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
            u.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
            v = bay_bcadd(v, u);
        }
        if (lane < tpw) {
            red[2 * ((warp * 32u + lane) * WPT + j)] = v.hi;
            red[2 * ((warp * 32u + lane) * WPT + j) + 1] = v.lo;
        }
    }
    __syncthreads();
    if (tid < nv) {
        // walker tid = tw' + j' TPR (4 tw' + j' on the vector path): its partials sit at lane
        // tw' % 32 of the warps holding tw'
        const unsigned int twp = VEC ? tid >> 2 : tid % TPR, jp = VEC ? tid & 3u : tid / TPR;
        const unsigned int stride = TPR < 32u ? 1u : TPR / 32u;   // warps between its copies
        bay_bcf a;
        a.hi = 0.0f;
        a.lo = 0.0f;
        for (unsigned int wq = twp / 32u; wq < blockDim.x / 32u; wq += stride) {
            bay_bcf b;
            b.hi = red[2 * ((wq * 32u + (twp & 31u)) * WPT + jp)];
            b.lo = red[2 * ((wq * 32u + (twp & 31u)) * WPT + jp) + 1];
            a = bay_bcadd(a, b);
        }
        float* out = P.part + M.part + 2 * ((size_t)(I.k0 + tid) * M.chunks + I.c);
        out[0] = a.hi;
        out[1] = a.lo;
    }
}

template <int MODE>  // 0 bare, 1 accu, 2 log density of the current positions
__device__ __forceinline__ void bay_batch_accept_impl(const bay_batch_params& P, unsigned int idx) {
    const bay_btile T = P.tiles[idx];
    const bay_bmember& M = P.mem[T.m];
    const unsigned int nk = MODE == 2 ? M.W : M.K;
    const unsigned int dim = M.dim, tid = threadIdx.x;
    const unsigned int k = T.k0 + tid;
    const bool valid = k < nk;
    bool accepted = false;
    if (valid) {
        const size_t wk = (size_t)M.walker0 + k;
        bay_bcf s;
        s.hi = P.wterm[wk];
        s.lo = 0.0f;
        const float2* pp = reinterpret_cast<const float2*>(P.part + M.part) + (size_t)k * M.chunks;
        // in chunk order; unrolled so that several partials' loads are in flight
#pragma unroll 4
        for (unsigned int c = 0; c < M.chunks; ++c) {
            const float2 v = pp[c];
            bay_bcf p;
            p.hi = v.x;
            p.lo = v.y;
            s = bay_bcadd(s, p);
        }
        const float ly = __fadd_rn(s.hi, s.lo);
        if (MODE == 2) {
            P.logfn[wk] = ly;
        } else {
            const size_t lk = (size_t)M.walker0 + (size_t)P.half * M.K + k;
            accepted = bay_batch_accept(P.zu[2 * wk + 1], P.zu[2 * wk], ly, P.logfn[lk],
                                        MODE == 1 ? 1.0f : P.ctl->beta, dim);
            if (accepted) P.logfn[lk] = ly;
        }
    }
    if (MODE == 2) return;
    // the accepted walkers' rows, element-wise over the tile (coalesced, many in flight)
    __shared__ unsigned char sAcc[256];
    sAcc[tid] = accepted ? 1 : 0;
    __syncthreads();
    {
        const unsigned int nt = nk - T.k0 < blockDim.x ? nk - T.k0 : blockDim.x;
        float* __restrict__ Xt = P.xs + M.xs + ((size_t)P.half * M.K + T.k0) * dim;
        const float* __restrict__ Yt = P.y + M.xs + (size_t)T.k0 * dim;
        const float inv_dim = __frcp_rn((float)dim);
#pragma unroll 4
        for (unsigned int e = tid; e < nt * dim; e += blockDim.x)
            if (sAcc[bay_div_dim(e, dim, inv_dim)]) Xt[e] = Yt[e];
    }
    // the persistent launch runs the next tile's accept in this CTA: sAcc is rewritten
    // there only after every thread has read it here
    __syncthreads();
    if (MODE != 1) return;
    // accu: the member's accepted count and this CTA's per-dim sums of the moved walkers
    const int n_acc = __syncthreads_count(accepted);
    if (tid == 0 && n_acc) atomicAdd(&P.accepted[T.m], (unsigned long long)n_acc);
    if (P.means_cap == 0) return;
    const unsigned int nt = nk - T.k0 < blockDim.x ? nk - T.k0 : blockDim.x;
    const float* Xc = P.xs + M.xs + ((size_t)P.half * M.K + T.k0) * dim;
    float* out = P.dsum + ((size_t)P.step_off * 2 + P.half) * P.dsum_stride + M.dsum
        + (size_t)(idx - M.tile0) * dim;
    for (unsigned int d = tid; d < dim; d += blockDim.x) {
        bay_bcf s;
        s.hi = 0.0f;
        s.lo = 0.0f;
        // in walker order; unrolled so that several rows' loads are in flight
#pragma unroll 8
        for (unsigned int w = 0; w < nt; ++w) {
            bay_bcf y;
            y.hi = Xc[(size_t)w * dim + d];
            y.lo = 0.0f;
            s = bay_bcadd(s, y);
        }
        out[d] = __fadd_rn(s.hi, s.lo);
    }
}

// Per-step ensemble means of each member from the accu launches' per-CTA sums:
// grid (members, steps); means[M.means + (step[1] + t) * dim + d] = sum / W in FP64.
__device__ __forceinline__ void bay_batch_means_impl(const bay_batch_params& P) {
    const unsigned int m = blockIdx.x, t = blockIdx.y;
    const bay_bmember& M = P.mem[m];
    const unsigned int step = P.ctl->step[1] + t;
    if (step >= P.means_cap) return;
    for (unsigned int d = threadIdx.x; d < M.dim; d += blockDim.x) {
        double s = 0.0;
        for (unsigned int h = 0; h < 2; ++h) {
            const float* src = P.dsum + ((size_t)t * 2 + h) * P.dsum_stride + M.dsum + d;
            for (unsigned int c = 0; c < M.ntiles; ++c) s += (double)src[(size_t)c * M.dim];
        }
        P.means[M.means + (size_t)step * M.dim + d] = (float)(s / (double)M.W);
    }
}

extern "C" __global__ void __launch_bounds__(256) bay_batch_propose_bare(bay_batch_params P) {
    bay_batch_propose_impl<0>(P, blockIdx.x);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_propose_accu(bay_batch_params P) {
    bay_batch_propose_impl<1>(P, blockIdx.x);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_propose_logfn(bay_batch_params P) {
    bay_batch_propose_impl<2>(P, blockIdx.x);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_rows_move(bay_batch_params P) {
    bay_batch_rows_impl<0, 1u>(P, blockIdx.x);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_rows_logfn(bay_batch_params P) {
    bay_batch_rows_impl<2, 1u>(P, blockIdx.x);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_rows_move2(bay_batch_params P) {
    bay_batch_rows_impl<0, 2u>(P, blockIdx.x);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_rows_logfn2(bay_batch_params P) {
    bay_batch_rows_impl<2, 2u>(P, blockIdx.x);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_rows_move4(bay_batch_params P) {
    bay_batch_rows_impl<0, 4u>(P, blockIdx.x);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_rows_logfn4(bay_batch_params P) {
    bay_batch_rows_impl<2, 4u>(P, blockIdx.x);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_accept_bare(bay_batch_params P) {
    bay_batch_accept_impl<0>(P, blockIdx.x);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_accept_accu(bay_batch_params P) {
    bay_batch_accept_impl<1>(P, blockIdx.x);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_accept_logfn(bay_batch_params P) {
    bay_batch_accept_impl<2>(P, blockIdx.x);
}
extern "C" __global__ void __launch_bounds__(128) bay_batch_means(bay_batch_params P) {
    bay_batch_means_impl(P);
}

// One persistent cooperative launch of m steps (both halves each) of every member.  Each
// half-step's three phases -- proposals over the move tiles, row terms over the work items,
// accept over the tiles -- run with a bounded grid barrier between them; CTA b takes work
// b, b + gridDim.x, ... of every phase.  The same functions on the same work as the three
// launches per half-step, so the results are identical.  A barrier that runs out (status
// bit 4) ends the launch.
template <int MODE, unsigned int WPT>
__device__ __forceinline__ void bay_batch_run_impl(bay_batch_params P, unsigned int m) {
    unsigned int k = 0;   // grid barriers passed
    for (unsigned int si = 0; si < m; ++si) {
        for (unsigned int half = 0; half < 2u; ++half) {
            P.half = half;
            P.step_off = si;
            if ((si | half) != 0u &&
                !bay_grid_sync(&P.ctl->gbar_count, &P.ctl->abort, &P.ctl->status, gridDim.x, ++k,
                               P.gbar_extra))
                return;
            for (unsigned int t = blockIdx.x; t < P.n_tiles; t += gridDim.x)
                bay_batch_propose_impl<MODE>(P, t);
            if (!bay_grid_sync(&P.ctl->gbar_count, &P.ctl->abort, &P.ctl->status, gridDim.x, ++k,
                               P.gbar_extra))
                return;
            for (unsigned int i = blockIdx.x; i < P.n_items; i += gridDim.x)
                bay_batch_rows_impl<0, WPT>(P, i);
            if (!bay_grid_sync(&P.ctl->gbar_count, &P.ctl->abort, &P.ctl->status, gridDim.x, ++k,
                               P.gbar_extra))
                return;
            for (unsigned int t = blockIdx.x; t < P.n_tiles; t += gridDim.x)
                bay_batch_accept_impl<MODE>(P, t);
        }
    }
}

extern "C" __global__ void __launch_bounds__(256) bay_batch_run_bare(bay_batch_params P, unsigned int m) {
    bay_batch_run_impl<0, 1u>(P, m);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_run_accu(bay_batch_params P, unsigned int m) {
    bay_batch_run_impl<1, 1u>(P, m);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_run_bare2(bay_batch_params P, unsigned int m) {
    bay_batch_run_impl<0, 2u>(P, m);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_run_accu2(bay_batch_params P, unsigned int m) {
    bay_batch_run_impl<1, 2u>(P, m);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_run_bare4(bay_batch_params P, unsigned int m) {
    bay_batch_run_impl<0, 4u>(P, m);
}
extern "C" __global__ void __launch_bounds__(256) bay_batch_run_accu4(bay_batch_params P, unsigned int m) {
    bay_batch_run_impl<1, 4u>(P, m);
}
