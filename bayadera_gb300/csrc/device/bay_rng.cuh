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

#endif
