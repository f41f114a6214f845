// bay_direct.cuh -- direct samplers of the built-in distributions, compiled by NVRTC with
// -use_fast_math (as the reference compiles cuda/rng/*-sampler.cu) after bay_rng.cuh.
//
// Four samples per Philox call: key {seed, 0xdecafaaa}, counter {i, 0xf00dcafe,
// 0xdeadbeef, 0xbeeff00d} for the i-th group of four (erlang: the last word is the
// draw index 0..k-1).  kind 0 uniform(lower, upper), 1 gaussian(mu, sigma) by the
// Box-Muller transform, 2 exponential(lambda) by inversion, 3 erlang(lambda, k) as the
// sum of k exponential logs.  The stream and the expressions follow the reference's
// uniform-, gaussian-, exponential- and erlang-sampler.cu, so a seed gives the
// reference's samples (bit for bit where no transcendental is involved).

#define BAY_2PI_F 6.2831855f

extern "C" __global__ void __launch_bounds__(256)
bay_direct_sample(unsigned int kind, unsigned long long n4, const float* params, unsigned int seed,
                  float4* out) {
    for (unsigned long long g = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; g < n4;
         g += (unsigned long long)gridDim.x * blockDim.x) {
        bay_u4 c;
        c.x = (unsigned int)g;
        c.y = 0xf00dcafeu;
        c.z = 0xdeadbeefu;
        c.w = 0xbeeff00du;
        float4 res;
        if (kind == 3u) {
            const float lambda = -params[0];
            const float k = params[1];
            res.x = 0.0f;
            res.y = 0.0f;
            res.z = 0.0f;
            res.w = 0.0f;
            for (unsigned int i = 0; i < k; i++) {
                c.w = i;
                const bay_u4 r = bay_philox4x32_10(c, seed, 0xdecafaaau);
                res.x += logf(bay_u01(r.x));
                res.y += logf(bay_u01(r.y));
                res.z += logf(bay_u01(r.z));
                res.w += logf(bay_u01(r.w));
            }
            res.x /= lambda;
            res.y /= lambda;
            res.z /= lambda;
            res.w /= lambda;
        } else {
            const bay_u4 r = bay_philox4x32_10(c, seed, 0xdecafaaau);
            const float u0 = bay_u01(r.x), u1 = bay_u01(r.y), u2 = bay_u01(r.z), u3 = bay_u01(r.w);
            if (kind == 0u) {
                const float lower = params[0];
                const float range = params[1] - lower;
                res.x = __fmaf_rn(u0, range, lower);   // the reference's contracted u*range + lower
                res.y = __fmaf_rn(u1, range, lower);
                res.z = __fmaf_rn(u2, range, lower);
                res.w = __fmaf_rn(u3, range, lower);
            } else if (kind == 1u) {
                const float mu = params[0], sigma = params[1];
                res.x = sinf(BAY_2PI_F * u0) * sqrtf(-2.0f * logf(u1));
                res.y = cosf(BAY_2PI_F * u0) * sqrtf(-2.0f * logf(u1));
                res.z = sinf(BAY_2PI_F * u2) * sqrtf(-2.0f * logf(u3));
                res.w = cosf(BAY_2PI_F * u2) * sqrtf(-2.0f * logf(u3));
                res.x = __fmaf_rn(res.x, sigma, mu);
                res.y = __fmaf_rn(res.y, sigma, mu);
                res.z = __fmaf_rn(res.z, sigma, mu);
                res.w = __fmaf_rn(res.w, sigma, mu);
            } else {
                const float lambda = params[0];
                res.x = -1.0f / lambda * logf(1.0f - u0);
                res.y = -1.0f / lambda * logf(1.0f - u1);
                res.z = -1.0f / lambda * logf(1.0f - u2);
                res.w = -1.0f / lambda * logf(1.0f - u3);
            }
        }
        out[g] = res;
    }
}
