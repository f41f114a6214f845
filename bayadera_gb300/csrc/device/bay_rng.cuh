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
// bay_accept_log: the stretch move's accept test, shared by every kernel form.
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

// The stretch move's Metropolis test (Goodman & Weare 2010, eq. 7) in log space:
// accept iff log u <= dm1 log z + beta (ly - lx), dm1 = dimension - 1; a non-finite
// proposal density is rejected.  The decision is that of the test in FP64 with FP64 logs.
// An fp32 evaluation with the fast logs decides whenever its two sides differ by more than
// a bound on its error; inside that band (a few walkers in 10^5) the FP64 logs decide.  So
// the decision does not depend on the fast logs' rounding (a CPU restatement with FP64 logs
// reproduces it), and the common path has no FP64 arithmetic.
//   fp32 errors: __logf at most 2^-21.41 absolute on [0.5, 2] and 3 ulp elsewhere, i.e.
//   below 2^-21.41 (1 + |log|); ly - lx and the product with beta each rounded once, below
//   2^-23 |beta| (|ly| + |lx|); the fma and the subtraction of tol below 2^-23 of |rhs| and
//   tol.  tol is at least twice their sum.  Non-finite sides make the band test false
//   (inf - inf), so those cases go to the FP64 comparison too.
__device__ __forceinline__ bool bay_accept_log(float u2, float z, float ly, float lx, float beta,
                                               unsigned int dm1) {
    if (!isfinite(ly)) return false;
    const float fd = (float)dm1;
    const float lz = __logf(z);
    const float lhs = __logf(u2);
    const float dl = beta * (ly - lx);
    const float rhs = fmaf(fd, lz, dl);
    const float tol = 0x1p-20f * (1.0f + fabsf(lhs) + fd * (1.0f + fabsf(lz)) + fabsf(rhs))
        + 0x1p-21f * fabsf(beta) * (fabsf(ly) + fabsf(lx));
    if (lhs < rhs - tol) return true;
    if (lhs > rhs + tol) return false;
    const double dl64 = (double)beta * ((double)ly - (double)lx);
    return log((double)u2) <= (double)dm1 * log((double)z) + dl64;
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

#endif
