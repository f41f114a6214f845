// bay_rng.cuh -- counter-based random numbers for the stretch-move engine.
//
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As Easy
// as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies, key bumped by the
// Weyl constants between rounds.  The reference draws its numbers from Random123's
// philox.h; the counter/key words each kernel uses are listed beside the kernels.
//
// bay_u01: the reference's u01fpt_oo_32_24 (cuda/rng/uniform-sampler.cu:11-13),
// (0.5 + (i >> 9)) * 2^-23, an exactly representable value in (0, 1).
//
// bay_accept_log: the stretch move's accept test, shared by every kernel form, with
// bay_log_det, a logarithm whose bits a CPU restatement reproduces.
// bay_grid_sync: a bounded grid barrier for persistent cooperative launches.
//
// This header is compiled both by nvcc (into libbayadera_gb300.so) and by NVRTC
// (prepended to every fused stretch kernel), so it uses no host headers.
#pragma once

#ifndef BAY_RNG_CUH
#define BAY_RNG_CUH

struct bay_u4 {
    unsigned int x, y, z, w;
};

__device__ __forceinline__ bay_u4 bay_philox4x32_10(bay_u4 c, unsigned int k0, unsigned int k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const unsigned int lo0 = 0xD2511F53u * c.x;
        const unsigned int hi0 = __umulhi(0xD2511F53u, c.x);
        const unsigned int lo1 = 0xCD9E8D57u * c.z;
        const unsigned int hi1 = __umulhi(0xCD9E8D57u, c.z);
        bay_u4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

__device__ __forceinline__ float bay_u01(unsigned int i) {
    // (0.5 + (i >> 9)) * 2^-23: both steps are exact in fp32.
    return __fmul_rn(__fadd_rn(0.5f, (float)(i >> 9)), 1.1920928955078125E-7f);
}

// Natural logarithm of a positive normal float in fp32, every operation rounded on its own
// (no fast-math approximation, no FP64), so that a CPU restatement with the same
// operations gives the same bits.  x = m 2^e with m in [sqrt(1/2), sqrt(2)); log m =
// 2 atanh(s), s = (m - 1) / (m + 1), |s| <= 0.1716, by its series to s^11 (the first
// omitted term is below 2^-28 of the result); e ln 2 with ln 2 split into a 16-bit head
// and a tail.  About 1 ulp.
__device__ __forceinline__ float bay_log_det(float x) {
    const unsigned int b = __float_as_uint(x);
    int e = (int)(b >> 23) - 127;
    float m = __uint_as_float((b & 0x007fffffu) | 0x3f800000u);
    if (m > 1.41421354f) {
        m = __fmul_rn(m, 0.5f);
        e += 1;
    }
    const float f = __fsub_rn(m, 1.0f);
    const float s = __fdiv_rn(f, __fadd_rn(2.0f, f));
    const float w = __fmul_rn(s, s);
    float p = __fmaf_rn(w, 0.181818187f, 0.222222224f);      // 2/11, 2/9
    p = __fmaf_rn(w, p, 0.285714298f);                         // 2/7
    p = __fmaf_rn(w, p, 0.400000006f);                         // 2/5
    p = __fmaf_rn(w, p, 0.666666687f);                         // 2/3
    const float lm = __fmaf_rn(__fmul_rn(s, w), p, __fadd_rn(s, s));
    const float fe = (float)e;
    return __fmaf_rn(fe, 0.693145752f, __fmaf_rn(fe, 1.42860677e-06f, lm));
}

// The stretch move's Metropolis test (Goodman & Weare 2010, eq. 7) in log space:
// accept iff log u <= dm1 log z + beta (ly - lx), dm1 = dimension - 1; a non-finite
// proposal density is rejected.  fp32 throughout with bay_log_det, each operation rounded
// on its own: the decision is a fixed function of (u, z, ly, lx, beta), which the CPU
// restatement reproduces bit for bit, and it needs neither fast-math logs nor FP64.
__device__ __forceinline__ bool bay_accept_log(float u2, float z, float ly, float lx, float beta,
                                               unsigned int dm1) {
    if (!isfinite(ly)) return false;
    const float dl = __fmul_rn(beta, __fsub_rn(ly, lx));
    const float rhs = __fmaf_rn((float)dm1, bay_log_det(z), dl);
    return bay_log_det(u2) <= rhs;
}

// Grid barrier k (k = 1, 2, ... within a launch) of a cooperative launch (every CTA
// resident): each CTA adds 1 to *count (a release reduction) and waits until it reaches
// k * nblocks + extra; the count only grows during a launch and is cleared before it.
// Bounded: a CTA that waits longer than 2 s raises *abort and status bit 4, and a raised
// abort ends every wait at once.  Returns false when the launch is being abandoned.
// `extra` arrivals beyond the grid (nonzero only in tests) make every barrier run out.
__device__ __forceinline__ bool bay_grid_sync(unsigned int* count, unsigned int* abort_flag,
                                              unsigned int* status, unsigned int nblocks,
                                              unsigned int k, unsigned int extra) {
    __shared__ unsigned int s_go;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int go = 1u;
        volatile unsigned int* ab = abort_flag;
        if (*ab) {
            go = 0u;
        } else {
            const unsigned int target = k * nblocks + extra;
            __threadfence();
            asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(count) : "memory");
            unsigned long long t0;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
            for (unsigned int it = 0;; ++it) {
                unsigned int c;
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(count) : "memory");
                if (c >= target) break;
                if ((it & 63u) == 63u) {
                    if (*ab) {
                        go = 0u;
                        break;
                    }
                    unsigned long long t;
                    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
                    if (t - t0 > 2000000000ull) {
                        *ab = 1u;
                        atomicOr(status, 4u);
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

// bay_v4: the values of four walkers, for row terms written over their number type (the
// batched engine's 4-walker path).  Each operator applies the scalar operator lane by lane,
// so a term gives every walker the bits its scalar form gives.
struct __align__(16) bay_v4 {
    float x, y, z, w;
};
__device__ __forceinline__ bay_v4 operator+(bay_v4 a, bay_v4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
__device__ __forceinline__ bay_v4 operator-(bay_v4 a, bay_v4 b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
__device__ __forceinline__ bay_v4 operator*(bay_v4 a, bay_v4 b) { return {a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
__device__ __forceinline__ bay_v4 operator+(float a, bay_v4 b) { return {a + b.x, a + b.y, a + b.z, a + b.w}; }
__device__ __forceinline__ bay_v4 operator-(float a, bay_v4 b) { return {a - b.x, a - b.y, a - b.z, a - b.w}; }
__device__ __forceinline__ bay_v4 operator*(float a, bay_v4 b) { return {a * b.x, a * b.y, a * b.z, a * b.w}; }
__device__ __forceinline__ bay_v4 operator+(bay_v4 a, float b) { return {a.x + b, a.y + b, a.z + b, a.w + b}; }
__device__ __forceinline__ bay_v4 operator-(bay_v4 a, float b) { return {a.x - b, a.y - b, a.z - b, a.w - b}; }
__device__ __forceinline__ bay_v4 operator*(bay_v4 a, float b) { return {a.x * b, a.y * b, a.z * b, a.w * b}; }
// lane-wise IEEE add and subtract, never contracted (the engine's sums)
__device__ __forceinline__ bay_v4 bay_v4_add_rn(bay_v4 a, bay_v4 b) {
    return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w)};
}
__device__ __forceinline__ bay_v4 bay_v4_sub_rn(bay_v4 a, bay_v4 b) {
    return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z), __fsub_rn(a.w, b.w)};
}

#endif
