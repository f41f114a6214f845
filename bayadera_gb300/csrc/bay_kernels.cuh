// bay_kernels.cuh -- host-visible declarations of the nvcc-compiled kernels of
// libbayadera_gb300.so (everything except the per-model fused stretch kernels,
// which NVRTC builds at model-compile time from device/bay_stretch.cuh).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

// Must match struct bay_ctl in device/bay_stretch.cuh (the NVRTC side).
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

// Must match struct bay_stretch_params in device/bay_stretch.cuh.
struct bay_stretch_params {
    const float* params;
    float* xs;
    float* logfn;
    bay_ctl* ctl;
    float* part;
    float* means;
    unsigned long long data_len;
    unsigned int params_len;
    unsigned int W, K;
    unsigned int half;
    unsigned int step_off;
    unsigned int means_cap;
    float inv_W;
    unsigned long long gemm_base;
    unsigned long long gemm_rows;
    unsigned int gemm_ld;
    unsigned int gemm_np;
    const float* gemm_lay;
    float* s_y;
    float* s_b;
    float* s_prep;
    float* s_w;
    float* s_zu;
    float* s_part;
    unsigned int s_nsb;
    unsigned int s_sbrows;
    unsigned short* s_bh;
    unsigned short* s_bl;
    unsigned int tc_fp;
    unsigned int gbar_extra;
    unsigned int t_slices;
    unsigned int pad_t;
    float* t_part;
    unsigned int* t_ticket;
};

enum {
    BAY_CTL_SET_STEP0 = 1u << 0,
    BAY_CTL_SET_STEP1 = 1u << 1,
    BAY_CTL_SET_SEED0 = 1u << 2,
    BAY_CTL_SET_SEED1 = 1u << 3,
    BAY_CTL_SET_A = 1u << 4,
    BAY_CTL_SET_BETA = 1u << 5,
    BAY_CTL_ADD_STEP0 = 1u << 6,
    BAY_CTL_ADD_STEP1 = 1u << 7,
    BAY_CTL_RESET_ACCEPTED = 1u << 8,
    BAY_CTL_RESET_TICKETS = 1u << 9,
};

struct bay_ctl_op {
    unsigned int mask;
    unsigned int step[2];
    unsigned int seed[2];
    float a;
    float beta;
};

// Device state of mix!'s a-adaptation loop (bay_adapt_a): the current a (FP64, as the
// host loop keeps it), the last acceptance rate, the loop index i of mcmc.clj's loop, the
// number of acc-rate! probes run, and bad = 1 when the rule took a to 1 or below (the next
// probe would be refused, as bay_acc_rate refuses it).
struct bay_mix_state {
    double a;
    double rate;
    unsigned int i;
    unsigned int probes;
    unsigned int bad;
    unsigned int pad;
};

namespace bay {

cudaError_t launch_ctl_apply(bay_ctl* ctl, const bay_ctl_op& op, cudaStream_t s);
cudaError_t launch_init_uniform(float* xs, uint32_t D, uint64_t W, uint32_t seed,
                                const float* limits, cudaStream_t s);
cudaError_t launch_init_normal(float* xs, uint32_t D, uint64_t W, uint32_t seed, float mean,
                               float sd, cudaStream_t s);
// SoA xs[d*W + w] <-> AoS out[w*D + d] (dim x W column-major), for walkers [w0, w0+n).
cudaError_t launch_soa_to_aos(const float* xs, uint32_t D, uint64_t W, uint64_t w0, uint64_t n,
                              float* out, cudaStream_t s);
cudaError_t launch_aos_to_soa(const float* in, uint32_t D, uint64_t W, float* xs, cudaStream_t s);
// FP64 per-dim mean and population variance over W walkers (two passes per dim).
cudaError_t launch_moments(const float* xs, uint32_t D, uint64_t W, double* mean, double* var,
                           cudaStream_t s);
// Per-dim [min, max] into limits[2*d], [2*d+1]; zero_fold folds 0.0 in (reference Q7).
cudaError_t launch_minmax(const float* xs, uint32_t D, uint64_t W, int zero_fold, float* limits,
                          cudaStream_t s);
// counts[d*bins + b] += bin counts of the walkers (bins <= 4096).
cudaError_t launch_hist_count(const float* xs, uint32_t D, uint64_t W, uint32_t bins,
                              const float* limits, uint32_t* counts, cudaStream_t s);
// pdf = (bins/n)/(hi-lo) * count, then bitonic ranks (bins a power of two <= 1024).
cudaError_t launch_hist_finish(const uint32_t* counts, const float* limits, uint32_t D,
                               uint32_t bins, uint64_t n, float* pdf, float* ranks,
                               cudaStream_t s);
cudaError_t launch_fill_u32(uint32_t* p, uint32_t v, uint64_t n, cudaStream_t s);
// The GEMM form's matrix (rows x F at A, row stride ld, aux values at column aux_col)
// laid out feature-major with rows zero-padded to NP, then the aux values [NP][auxs].
cudaError_t launch_gemm_layout(const float* A, uint64_t ld, uint32_t rows, uint32_t F, uint32_t NP,
                               uint32_t aux_col, uint32_t aux_len, uint32_t auxs, float* lay,
                               cudaStream_t s);
// Tensor-core GEMM form: bf16 hi + lo copies of the matrix, [rows_pad][Fp] row-major with
// zero padding, and the rows' aux values [rows_pad][auxs].
cudaError_t launch_gemm_split(const float* A, uint64_t ld, uint32_t rows, uint32_t F, uint32_t Fp,
                              uint64_t rows_pad, uint32_t aux_col, uint32_t aux_len, uint32_t auxs,
                              unsigned short* hi, unsigned short* lo, float* aux, cudaStream_t s);
// Resident tensor-core GEMM form: the matrix image (bf16 hi then lo 128B-swizzled
// K-major atoms [KC][NP rows][64 features], then aux [NP][auxs]); 2 KC NP 128 + 4 NP auxs
// bytes.
cudaError_t launch_gemm_tc_image(const float* A, uint64_t ld, uint32_t rows, uint32_t F,
                                 uint32_t KC, uint32_t NP, uint32_t aux_col, uint32_t aux_len,
                                 uint32_t auxs, void* img, cudaStream_t s);
// Per-step ensemble means of `nsteps` accu steps from the stretch kernels' per-CTA sums
// part[((t*2 + half)*D + d)*G + cta]: means[(ctl->step[1] + t)*D + d] = sum / W, summed
// in FP64 in (half, cta) order; steps at or past means_cap are dropped.
cudaError_t launch_reduce_means(const bay_ctl* ctl, const float* part, float* means,
                                uint32_t means_cap, uint32_t G, uint32_t D, uint32_t nsteps,
                                double inv_W, cudaStream_t s);
// acor of a D x n column-major series (series[t*D + d]); work holds D*n doubles.
cudaError_t launch_acor(const float* series, uint32_t D, uint32_t n, uint32_t wgs, uint32_t lag,
                        double* work, double* tau, double* mean, double* sigma, cudaStream_t s);
// Fixed scratch of bay_acor_noalloc: dim * n + 3 * dim doubles at most (8 MiB).
#define BAY_ACOR_NOALLOC_MAX_DOUBLES (1u << 20)
// Device address of that scratch on the current device (cudaGetSymbolAddress; loads the
// library's module on that device if it is not loaded yet).  Allocates nothing.
cudaError_t acor_noalloc_scratch(double** ptr);
// One probe of mix!'s loop on the device: mix_begin is init-move! (accu seed + 2, accu
// step 0, a = (float) st->a, acceptance count 0); after the probe's accu step, mix_end
// counts the step, computes the rate and applies the loop's rule (mcmc.clj:84-91) in FP64
// without contraction, then sets the graph's WHILE condition (cont) to go on or stop.
cudaError_t launch_mix_begin(bay_ctl* ctl, bay_mix_state* st, cudaStream_t s);
cudaError_t launch_mix_end(bay_ctl* ctl, bay_mix_state* st, unsigned long long W, unsigned int step,
                           double min_acc, double max_acc, cudaGraphConditionalHandle cont,
                           cudaStream_t s);
// Kernels enqueued through this library in this process (graph nodes counted at replay).
unsigned long long launch_count();
void count_launches(unsigned long long n);
// Flush: write n bytes (used by the bench between timed iterations).
cudaError_t launch_fill_bytes(void* p, uint64_t n, unsigned char v, cudaStream_t s);

}  // namespace bay
