// bay_hist_fastdiv.cuh -- histogram bin counts with the reference's division flavour.
//
// The reference builds its estimate kernels with NVRTC and -use_fast_math, the bin count
// being the compile-time WGS (nvidia_gtx.clj:614-616), and bins a value by
// (uint)((x - lo) / (hi - lo) * WGS) clamped to WGS - 1 (nvidia-gtx-estimate.cu:22-23):
// the division there is the compiler's fast division.  The library compiles this file the
// same way (-use_fast_math, BAY_HIST_BINS a compile-time constant) so the same expression
// gets the same division; bay_kernels.cu's hist_count is the IEEE-division default.
//
// Layout and counting as hist_count: values dimension-major (xs[d * W + w]), blockIdx.y
// the dimension, per-CTA shared-memory counts, one global atomic per non-empty bin.

extern "C" __global__ void __launch_bounds__(256)
bay_hist_count_fastdiv(const float* xs, unsigned int D, unsigned long long W,
                       const float* limits, unsigned int* counts) {
    __shared__ unsigned int h[BAY_HIST_BINS];
    const unsigned int d = blockIdx.y;
    for (unsigned int b = threadIdx.x; b < BAY_HIST_BINS; b += blockDim.x) h[b] = 0u;
    __syncthreads();
    const float lower = limits[2 * d];
    const float upper = limits[2 * d + 1];
    const float* row = xs + (unsigned long long)d * W;
    for (unsigned long long w = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; w < W;
         w += (unsigned long long)gridDim.x * blockDim.x) {
        const float x = row[w];
        unsigned int bin = (unsigned int)((x - lower) / (upper - lower) * BAY_HIST_BINS);
        bin = (bin < BAY_HIST_BINS) ? bin : BAY_HIST_BINS - 1;
        atomicAdd(&h[bin], 1u);
    }
    __syncthreads();
    for (unsigned int b = threadIdx.x; b < BAY_HIST_BINS; b += blockDim.x)
        if (h[b]) atomicAdd(&counts[(unsigned long long)d * BAY_HIST_BINS + b], h[b]);
}
