// bay_api.cpp -- host side of libbayadera_gb300.so (C ABI in include/bayadera_gb300.h).
//
// Owns contexts (device + stream), models (NVRTC-compiled fused stretch kernels,
// loaded as CUDA driver-API libraries), and samplers (device-resident walker state,
// control block, captured CUDA graphs for the step loops).  Mirrors the reference's
// GTXStretch / GTXStretchFactory / GTXAcorEngine (internal/device/nvidia_gtx.clj).
#include "bayadera_gb300.h"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <nvtx3/nvToolsExt.h>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "bay_embedded.h"
#include "bay_kernels.cuh"

namespace {

thread_local std::string g_err;

struct Err {
    int code;
    std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg) { throw Err{code, msg}; }

void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        const int code = (e == cudaErrorMemoryAllocation) ? BAY_ERR_ALLOC : BAY_ERR_CUDA;
        fail(code, std::string(what) + ": " + cudaGetErrorString(e));
    }
}

// Driver-API entry points, resolved through the runtime at first context creation so
// that the library loads (and compile-checks models) on machines without a driver.
// NVTX range over a public call (header-only NVTX 3: inert unless a profiler attaches), so
// a trace shows which library call issued which kernels
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

struct DriverApi {
    PFN_cuGetErrorString_v6000 GetErrorString = nullptr;
    PFN_cuLibraryLoadData_v12000 LibraryLoadData = nullptr;
    PFN_cuLibraryUnload_v12000 LibraryUnload = nullptr;
    PFN_cuLibraryGetKernel_v12000 LibraryGetKernel = nullptr;
    PFN_cuLaunchKernel_v4000 LaunchKernel = nullptr;
    PFN_cuLaunchKernelEx_v11060 LaunchKernelEx = nullptr;
    PFN_cuKernelSetAttribute_v12000 KernelSetAttribute = nullptr;
    PFN_cuTensorMapEncodeTiled_v12000 TensorMapEncodeTiled = nullptr;
    PFN_cuKernelGetFunction_v12000 KernelGetFunction = nullptr;
    PFN_cuOccupancyMaxActiveBlocksPerMultiprocessor_v6050 OccupancyMaxActiveBlocks = nullptr;
    bool loaded = false;
};
DriverApi g_cu;
std::mutex g_cu_mu;

void cu_check(CUresult r, const char* what) {
    if (r != CUDA_SUCCESS) {
        const char* s = nullptr;
        if (g_cu.GetErrorString) g_cu.GetErrorString(r, &s);
        fail(BAY_ERR_CUDA, std::string(what) + ": " + (s ? s : "driver error " + std::to_string((int)r)));
    }
}

template <class T>
void resolve(const char* name, T& fn, unsigned version) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    const cudaError_t e = cudaGetDriverEntryPointByVersion(name, &p, version, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p) {
        cudaGetLastError();
        fail(BAY_ERR_CUDA, std::string("driver entry point not found: ") + name);
    }
    fn = reinterpret_cast<T>(p);
}

void load_driver_api() {
    std::lock_guard<std::mutex> g(g_cu_mu);
    if (g_cu.loaded) return;
    resolve("cuGetErrorString", g_cu.GetErrorString, 6000);
    resolve("cuLibraryLoadData", g_cu.LibraryLoadData, 12000);
    resolve("cuLibraryUnload", g_cu.LibraryUnload, 12000);
    resolve("cuLibraryGetKernel", g_cu.LibraryGetKernel, 12000);
    resolve("cuLaunchKernel", g_cu.LaunchKernel, 4000);
    resolve("cuLaunchKernelEx", g_cu.LaunchKernelEx, 11060);
    resolve("cuKernelSetAttribute", g_cu.KernelSetAttribute, 12000);
    resolve("cuTensorMapEncodeTiled", g_cu.TensorMapEncodeTiled, 12000);
    resolve("cuKernelGetFunction", g_cu.KernelGetFunction, 12000);
    resolve("cuOccupancyMaxActiveBlocksPerMultiprocessor", g_cu.OccupancyMaxActiveBlocks, 6050);
    g_cu.loaded = true;
}

template <class F>
int guarded(F&& f) {
    try {
        f();
        return BAY_OK;
    } catch (const Err& e) {
        g_err = e.msg;
        return e.code;
    } catch (const std::bad_alloc&) {
        g_err = "host allocation failed";
        return BAY_ERR_ALLOC;
    } catch (...) {
        g_err = "unexpected exception";
        return BAY_ERR_STATE;
    }
}

// Decides where a caller's pointer lives: device memory that the kernels of a context on
// `device` may read (true), or host memory that is staged through a copy (false).  Device
// memory of another GPU is refused with BAY_ERR_ARG before anything is launched: without
// peer access a kernel reading it faults.
bool ptr_on_device(int type, int ptr_device, int device) {
    if (type == cudaMemoryTypeDevice) {
        if (ptr_device != device)
            fail(BAY_ERR_ARG, "the array lies in device memory of device " +
                                  std::to_string(ptr_device) + ", but the context runs on device " +
                                  std::to_string(device));
        return true;
    }
    return type == cudaMemoryTypeManaged;
}

bool is_device_ptr(const void* p, int device) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return ptr_on_device((int)a.type, a.device, device);
}

// Process-wide cache of NVRTC output: identical (source, options) compile once.
std::mutex g_cache_mu;
std::map<std::string, std::vector<char>> g_cubin_cache;

constexpr uint32_t kChunk = 32;  // steps per captured graph

}  // namespace

// ============================================================================ context
struct bay_ctx {
    int device = 0;
    uint32_t wgs = 1024;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaStream_t capture = nullptr;
    uint64_t mem_limit = 0;
    uint64_t allocated = 0;
    std::recursive_mutex mu;
    std::map<void*, size_t> sizes;
    // the direct samplers' NVRTC module, compiled on first use
    CUlibrary direct_lib = nullptr;
    CUkernel k_direct = nullptr;
    // device address of bay_acor_noalloc's fixed scratch array on this context's device,
    // looked up when the context is created (the array itself is never allocated)
    double* acor_scratch = nullptr;
    // histogram bin counts with the fast division (BAY_HIST_COMPAT_FASTDIV): one NVRTC
    // module per bin count, compiled on first use
    std::map<uint32_t, std::pair<CUlibrary, CUkernel>> hist_fastdiv;

    void* alloc(size_t bytes) {
        if (bytes == 0) bytes = 16;
        if (mem_limit && allocated + bytes > mem_limit)
            fail(BAY_ERR_ALLOC, "device memory limit of the context exceeded (" +
                                    std::to_string(allocated + bytes) + " > " +
                                    std::to_string(mem_limit) + " bytes)");
        void* p = nullptr;
        cuda_check(cudaMalloc(&p, bytes), "cudaMalloc");
        allocated += bytes;
        sizes[p] = bytes;
        return p;
    }
    void release(void* p) {
        if (!p) return;
        auto it = sizes.find(p);
        if (it != sizes.end()) {
            allocated -= it->second;
            sizes.erase(it);
        }
        cudaFree(p);
    }
    void use() { cuda_check(cudaSetDevice(device), "cudaSetDevice"); }
};

// ============================================================================ model
struct bay_model {
    bay_ctx* ctx = nullptr;
    CUlibrary lib = nullptr;
    CUkernel k_bare = nullptr, k_accu = nullptr, k_logfn = nullptr;
    uint32_t dim = 0, params_size = 0, form = 0, cta = 256, wpc = 1, flags = 0;
    uint32_t tslices = 1;   // tiled form: row slices per walker group
    // GEMM form layout of A (see bay_model_desc)
    uint32_t gemm_features = 0, gemm_block = 0, gemm_ld = 0, gemm_aux_col = 0, gemm_aux_len = 0;
    uint32_t prep_len = 1;
    uint64_t gemm_offset = 0, gemm_rows = 0;
    // GEMM form, streaming kernels: propose / accept [bare, accu, logfn], rows [move, logfn]
    CUkernel k_gp[3] = {nullptr, nullptr, nullptr};
    CUkernel k_gr[2] = {nullptr, nullptr};
    CUkernel k_gr_wpt[3][2] = {};   // batch form rows kernels with 1, 2, 4 walkers per thread
    CUkernel k_brun[2][3] = {};     // batch form persistent launches [bare, accu][walkers per thread]
    CUkernel k_ga[3] = {nullptr, nullptr, nullptr};
    // GEMM form on the tensor cores: rows kernels [move, logfn], walker sub-tiles per CTA,
    // shared-memory stages, dynamic shared memory
    CUkernel k_gt[2] = {nullptr, nullptr};
    // GEMM form on the tensor cores with the matrix resident: [bare, accu, logfn]
    CUkernel k_tr[6] = {};   // bare, accu, logfn, persistent bare, persistent accu, statistics
    uint32_t tc_g = 0, tc_stages = 0;
    size_t tc_smem = 0;
    uint32_t tr_g = 1;   // resident tensor-core form: tile groups per CTA of the move kernels
    // batch form: propose / accept in k_gp / k_ga, rows in k_gr, per-step means here
    CUkernel k_bmeans = nullptr;
    uint32_t row_len = 0;
    // plain form: the density engines' point kernels
    CUkernel k_points = nullptr, k_evidence = nullptr;
};

namespace {
constexpr uint32_t kGemmWalkers = 64;             // BAY_WT in device/bay_stretch.cuh
constexpr size_t kGemmMaxSmem = 200 * 1024;       // dynamic shared memory cap per CTA

// Dynamic shared memory of the GEMM-form kernels for `rows` rows (layout in
// bay_stretch_gemm: A feature-major, Y tile twice, aux values).
size_t gemm_smem_bytes(const bay_model* m, uint64_t rows) {
    const uint64_t np = (rows + 63) & ~63ull;
    const uint64_t dpad = m->dim | 1u;
    const uint64_t auxs = m->gemm_aux_len ? m->gemm_aux_len : 1;
    return sizeof(float) * (m->gemm_features * np + m->gemm_features * kGemmWalkers +
                            kGemmWalkers * dpad + np * auxs);
}

// Tiled form: the data rows are staged in chunks of kTileChunk floats (BAY_TILE_CHUNK of
// the kernel), rounded down to whole rows, a multiple of 4; two chunk buffers when the
// data span more than one chunk, else one buffer of the data's size.
constexpr uint32_t kTileChunk = 12288;
size_t tile_smem_bytes(uint32_t row_len, uint64_t data_len) {
    const uint64_t chunk_rows = (kTileChunk / row_len) & ~3ull;
    const uint64_t n_rows = data_len / row_len;
    if (n_rows > chunk_rows) return 2ull * kTileChunk * sizeof(float);
    return ((n_rows * row_len * sizeof(float)) + 15) & ~15ull;
}

// Tensor-core rows kernel (bay_gemm_rows_tc_impl): G sub-tiles of 128 walkers per CTA
// with their bf16 hi + lo coefficient operand resident (G x ceil(F/64) x 32 KB), a ring
// of S stages of one 128-row x 64-feature hi + lo chunk (32 KB each), two aux buffers,
// the barriers and flags, and 1 KB to align the operands to the 128-byte swizzle's
// 1024-byte period.  Largest G (fewer re-reads of the matrix), then up to 6 stages.
constexpr size_t kTcSmemMax = 232448;  // opt-in dynamic shared memory per CTA, sm_100 family
constexpr size_t kBatchSmemMax = 160 * 1024;   // batched rows kernels: dynamic shared memory, at most
constexpr uint32_t kTrWalkers = 64;  // walkers per tile of the resident tensor-core form
constexpr uint32_t kTrGroups = 4;    // tile groups (256 threads each) per persistent CTA
// want_g / want_s (0 = free) ask for a shape; false when no shape fits (or the asked one
// does not).
bool tc_plan(uint32_t features, uint32_t aux_len, uint32_t* G, uint32_t* S, size_t* smem,
             uint32_t want_g = 0, uint32_t want_s = 0) {
    const size_t kc = (features + 63) / 64, auxs = aux_len ? aux_len : 1;
    for (uint32_t g = 2; g >= 1; --g) {
        if (want_g && g != want_g) continue;
        const size_t fixed = (size_t)g * kc * 32768 + 2 * 128 * auxs * sizeof(float) + 1024 + 256;
        if (fixed + 2 * 32768 > kTcSmemMax) continue;
        size_t st = std::min<size_t>(6, (kTcSmemMax - fixed) / 32768);
        if (want_s) {
            if (want_s < 2 || want_s > st) return false;
            st = want_s;
        }
        *G = g;
        *S = (uint32_t)st;
        *smem = fixed + st * 32768;
        return true;
    }
    return false;
}

// Host image of the kernel's bay_tmaps parameter.
struct TcMaps {
    CUtensorMap xh, xl, bh, bl;
};

// 2-D bf16 tensor map over a row-major [rows][cols] array, 64 x 128 boxes, 128B swizzle.
void encode_bf16_map(CUtensorMap* m, void* base, uint64_t cols, uint64_t rows) {
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)(cols * 2)};
    const cuuint32_t box[2] = {64, 128};
    const cuuint32_t estr[2] = {1, 1};
    cu_check(g_cu.TensorMapEncodeTiled(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides,
                                       box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                       CU_TENSOR_MAP_SWIZZLE_128B,
                                       CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                       CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE),
             "cuTensorMapEncodeTiled");
}
}  // namespace

namespace {

const char* kStdint =
    "#pragma once\n"
    "typedef unsigned char uint8_t; typedef signed char int8_t;\n"
    "typedef unsigned short uint16_t; typedef short int16_t;\n"
    "typedef unsigned int uint32_t; typedef int int32_t;\n"
    "typedef unsigned long long uint64_t; typedef long long int64_t;\n";

std::vector<char> nvrtc_compile(const std::string& src, const std::vector<std::string>& opts) {
    std::string key = src;
    for (auto& o : opts) key += "\n//" + o;
    {
        std::lock_guard<std::mutex> g(g_cache_mu);
        auto it = g_cubin_cache.find(key);
        if (it != g_cubin_cache.end()) return it->second;
    }
    nvrtcProgram prog;
    const char* hdr_src[] = {kStdint, kStdint};
    const char* hdr_name[] = {"stdint.h", "cstdint"};
    if (nvrtcCreateProgram(&prog, src.c_str(), "bay_model.cu", 2, hdr_src, hdr_name) !=
        NVRTC_SUCCESS)
        fail(BAY_ERR_COMPILE, "nvrtcCreateProgram failed");
    std::vector<const char*> o;
    for (auto& s : opts) o.push_back(s.c_str());
    // BAY_PTXAS_VERBOSE=1 prints ptxas' resource report (registers, spills, shared memory)
    const bool verbose = std::getenv("BAY_PTXAS_VERBOSE") != nullptr;
    if (verbose) o.push_back("--ptxas-options=-v");
    const nvrtcResult r = nvrtcCompileProgram(prog, (int)o.size(), o.data());
    if (verbose && r == NVRTC_SUCCESS) {
        size_t n = 0;
        nvrtcGetProgramLogSize(prog, &n);
        std::string log(n, '\0');
        if (n) nvrtcGetProgramLog(prog, &log[0]);
        std::fprintf(stderr, "%s\n", log.c_str());
    }
    if (r != NVRTC_SUCCESS) {
        size_t n = 0;
        nvrtcGetProgramLogSize(prog, &n);
        std::string log(n, '\0');
        if (n) nvrtcGetProgramLog(prog, &log[0]);
        nvrtcDestroyProgram(&prog);
        fail(BAY_ERR_COMPILE, std::string("model compilation failed: ") +
                                  nvrtcGetErrorString(r) + "\n" + log);
    }
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    std::vector<char> cubin(n);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    std::lock_guard<std::mutex> g(g_cache_mu);
    g_cubin_cache[key] = cubin;
    return cubin;
}

bool valid_ident(const char* s) {
    if (!s || !*s) return false;
    if (!(std::isalpha((unsigned char)s[0]) || s[0] == '_')) return false;
    for (const char* p = s; *p; ++p)
        if (!(std::isalnum((unsigned char)*p) || *p == '_')) return false;
    return true;
}

}  // namespace

// ============================================================================ sampler
struct bay_sampler {
    bay_model* model = nullptr;
    bay_ctx* ctx = nullptr;
    uint64_t W = 0, K = 0;
    uint32_t D = 0;
    float* xs = nullptr;
    float* logfn = nullptr;
    bay_ctl* ctl = nullptr;
    const float* params = nullptr;
    bool own_params = false;
    uint64_t n_params = 0, data_len = 0;
    float* part = nullptr;  // accu per-CTA sums of one chunk: kChunk x 2 x grid() x D
    float* t_part = nullptr;         // tiled form, row slices: [K][slices] (hi, lo) partials
    unsigned int* t_ticket = nullptr;  // tiled form, row slices: [grid()] slice tickets
    float* means = nullptr;
    uint64_t means_cap = 0;
    float* stage = nullptr;  // W*D floats: AoS staging
    double* stats = nullptr;  // 2*D doubles
    float* hist = nullptr;    // limits + pdf + ranks scratch
    uint32_t* counts = nullptr;
    uint64_t hist_bins = 0;
    // host mirror of the control block
    uint32_t seed_bare = 0, seed_accu = 0;
    uint32_t step_bare = 0, step_accu = 0;
    float a = 2.0f, beta = 1.0f;
    uint64_t iteration_counter = 0;
    bool positioned = false;
    bool graphs = true;
    cudaGraphExec_t g_bare = nullptr, g_accu = nullptr;
    uint64_t g_accu_cap = 0;
    bay_mix_state* mix = nullptr;   // bay_adapt_a's device state, allocated on first use

    uint64_t gemm_base = 0, gemm_rows = 0;  // GEMM form: A's row 0 and row count in params
    uint32_t gemm_np = 0;                   // rows padded to a multiple of 64
    float* gemm_lay = nullptr;              // the kernel's layout of A and the aux values
    size_t smem = 0;                        // dynamic shared memory per CTA

    // Dimension-major copy of the walker state (stage[d * W + w]) for the per-dimension
    // estimate kernels (moments, limits, histogram), which read one dimension per CTA.
    const float* dim_major() {
        if (!stage) stage = (float*)ctx->alloc(sizeof(float) * (size_t)D * W);
        cuda_check(bay::launch_aos_to_soa(xs, D, W, stage, ctx->stream), "transpose");
        return stage;
    }

    // A device-detected failure (a bounded wait that gave up) sets ctl->status.
    void check_status() {
        unsigned int st = 0;
        cuda_check(cudaMemcpyAsync(&st, &ctl->status, sizeof(st), cudaMemcpyDeviceToHost,
                                   ctx->stream),
                   "cudaMemcpy(status)");
        cuda_check(cudaStreamSynchronize(ctx->stream), "sync");
        if (st) fail(BAY_ERR_DEVICE, std::string("a kernel gave up waiting for ") +
                                         ((st & 4u) ? "the other CTAs of its launch (grid barrier)"
                                          : (st & 2u) ? "its tensor-core pipeline" : "its shared-memory copy") +
                                         " (device status " + std::to_string(st) + ")");
    }

    // GEMM form, streaming mode (matrix read from device memory in row blocks)
    bool streaming = false;
    float *s_y = nullptr, *s_b = nullptr, *s_prep = nullptr, *s_w = nullptr, *s_zu = nullptr,
          *s_part = nullptr;
    uint32_t s_nsb = 0, s_sbrows = 0;
    size_t smem_rows = 0;
    // streaming on the tensor cores: bf16 hi + lo matrix [rows_pad][tc_fp], coefficient
    // operand [tc_wpad][tc_fp] (hi, lo), the aux values in gemm_lay [rows_pad][aux]
    bool tc = false;
    bool tcr = false;   // tensor cores, matrix resident (one launch per half-step, or
                        // one persistent cooperative launch per chunk of steps)
    uint32_t tr_g = 1;          // tcr: tile groups per CTA of the per-launch move kernels
    size_t smem_move = 0;       // tcr: their dynamic shared memory; tiled: a row slice's
    bool persistent = false;    // tcr: the persistent form (when tr_smem != 0); measured
                                // slower than programmatic dependent launches, so opt-in
    uint32_t tr_grid = 0;       // tcr: CTAs of the persistent form (all co-resident)
    size_t tr_smem = 0;         // tcr: dynamic shared memory of a persistent CTA
    uint32_t gbar_extra = 0;    // tcr persistent: arrivals the grid barriers wait for beyond
                                // the grid (1 in tests of the bounded wait)
    uint32_t tc_fp = 0;
    uint64_t tc_rows_pad = 0, tc_wpad = 0;
    unsigned short *tc_xh = nullptr, *tc_xl = nullptr, *s_bh = nullptr, *s_bl = nullptr;
    TcMaps tc_maps;

    uint64_t per_cta() const {
        if (streaming) return 256;  // the accept kernel: one thread per walker
        if (tcr) return kTrWalkers;
        return model->form == BAY_FORM_PLAIN ? model->cta : model->wpc;
    }

    // CTAs of the launch that writes the accu statistics (and so of the partials)
    unsigned grid() const { return (unsigned)((K + per_cta() - 1) / per_cta()); }

    void launch(CUkernel k, unsigned gx, unsigned gy, size_t sm, bay_stretch_params& p,
                cudaStream_t st, const char* what) {
        void* args[] = {&p};
        cu_check(g_cu.LaunchKernel((CUfunction)k, gx, gy, 1, 256, 1, 1, (unsigned)sm,
                                   (CUstream)st, args, nullptr),
                 what);
    }

    // the three launches of a streaming half-step (mode 0 bare, 1 accu, 2 logfn)
    void launch_streaming(int mode, uint32_t half, uint32_t step_off, cudaStream_t st) {
        bay_stretch_params p = make_params(half, step_off);
        const uint64_t nk = mode == 2 ? W : K;
        const unsigned g1 = (unsigned)((nk + 255) / 256), gt = (unsigned)((nk + 127) / 128);
        launch(model->k_gp[mode], g1, 1, 0, p, st, "cuLaunchKernel(gemm propose)");
        if (tc) {
            const uint64_t per = 128ull * model->tc_g;
            void* args[] = {&p, &tc_maps};
            cu_check(g_cu.LaunchKernel((CUfunction)model->k_gt[mode == 2 ? 1 : 0],
                                       (unsigned)((nk + per - 1) / per), s_nsb, 1,
                                       576, 1, 1, (unsigned)model->tc_smem,
                                       (CUstream)st, args, nullptr),
                     "cuLaunchKernel(gemm rows, tensor cores)");
        } else {
            launch(model->k_gr[mode == 2 ? 1 : 0], gt, s_nsb, smem_rows, p, st,
                   "cuLaunchKernel(gemm rows)");
        }
        launch(model->k_ga[mode], g1, 1, 0, p, st, "cuLaunchKernel(gemm accept)");
        if (st == ctx->stream) bay::count_launches(3);
    }

    bay_stretch_params make_params(uint32_t half, uint32_t step_off) const {
        bay_stretch_params p;
        p.params = params;
        p.xs = xs;
        p.logfn = logfn;
        p.ctl = ctl;
        p.part = part;
        p.means = means;
        p.data_len = data_len;
        p.params_len = (unsigned)(n_params - data_len);
        p.W = (unsigned)W;
        p.K = (unsigned)K;
        p.half = half;
        p.step_off = step_off;
        p.means_cap = (unsigned)std::min<uint64_t>(means_cap, 0xffffffffull);
        p.inv_W = (float)(1.0 / (double)W);
        p.gemm_base = gemm_base;
        p.gemm_rows = gemm_rows;
        p.gemm_ld = model->gemm_ld;
        p.gemm_np = gemm_np;
        p.gemm_lay = gemm_lay;
        p.s_y = s_y;
        p.s_b = s_b;
        p.s_prep = s_prep;
        p.s_w = s_w;
        p.s_zu = s_zu;
        p.s_part = s_part;
        p.s_nsb = s_nsb;
        p.s_sbrows = s_sbrows;
        p.s_bh = s_bh;
        p.s_bl = s_bl;
        p.tc_fp = tc_fp;
        p.gbar_extra = gbar_extra;
        p.t_slices = model->form == BAY_FORM_TILED ? model->tslices : 1u;
        p.pad_t = 0;
        p.t_part = t_part;
        p.t_ticket = t_ticket;
        return p;
    }

    // pdl = false launches the resident tensor-core kernels without programmatic
    // dependent launch (the body of a conditional graph node)
    void launch_half(bool accu, uint32_t half, uint32_t step_off, cudaStream_t st, bool pdl = true) {
        if (streaming) {
            launch_streaming(accu ? 1 : 0, half, step_off, st);
            return;
        }
        if (st == ctx->stream) bay::count_launches(1);
        bay_stretch_params p = make_params(half, step_off);
        void* args[] = {&p};
        if (tcr || model->form == BAY_FORM_TILED) {
            // programmatic dependent launch: the kernel sets up its barriers (tensor memory,
            // data copies) and reads what the previous kernel of the stream does not write,
            // then waits (griddepcontrol.wait) for that kernel to complete, so all this
            // overlaps its tail
            CUlaunchAttribute at[1];
            at[0].id = CU_LAUNCH_ATTRIBUTE_PROGRAMMATIC_STREAM_SERIALIZATION;
            at[0].value.programmaticStreamSerializationAllowed = 1;
            CUlaunchConfig cfg{};
            cfg.gridDimX = tcr ? (grid() + tr_g - 1) / tr_g : grid() * model->tslices;
            cfg.gridDimY = 1;
            cfg.gridDimZ = 1;
            cfg.blockDimX = tcr ? 256 * tr_g : model->cta;
            cfg.blockDimY = 1;
            cfg.blockDimZ = 1;
            cfg.sharedMemBytes = (unsigned)smem_move;
            cfg.hStream = (CUstream)st;
            cfg.attrs = at;
            cfg.numAttrs = pdl ? 1 : 0;
            CUkernel k = tcr ? model->k_tr[accu ? 1 : 0] : (accu ? model->k_accu : model->k_bare);
            cu_check(g_cu.LaunchKernelEx(&cfg, (CUfunction)k, args, nullptr),
                     tcr ? "cuLaunchKernelEx(stretch, tensor cores)" : "cuLaunchKernelEx(stretch, tiled)");
            return;
        }
        CUkernel k = accu ? model->k_accu : model->k_bare;
        cu_check(g_cu.LaunchKernel((CUfunction)k, grid(), 1, 1, model->cta, 1, 1,
                                   (unsigned)smem, (CUstream)st, args, nullptr),
                 "cuLaunchKernel(stretch)");
    }

    void ctl_op(const bay_ctl_op& op) {
        cuda_check(bay::launch_ctl_apply(ctl, op, ctx->stream), "ctl_apply");
    }

    void launch_logfn_all() {
        if (streaming) {
            launch_streaming(2, 0, 0, ctx->stream);
            return;
        }
        bay::count_launches(1);
        bay_stretch_params p = make_params(0, 0);
        void* args[] = {&p};
        const unsigned g = (unsigned)((W + per_cta() - 1) / per_cta());
        cu_check(g_cu.LaunchKernel((CUfunction)(tcr ? model->k_tr[2] : model->k_logfn), g, 1, 1,
                                   tcr ? 256 : model->cta, 1, 1, (unsigned)smem,
                                   (CUstream)ctx->stream, args, nullptr),
                 "cuLaunchKernel(logfn)");
    }

    // m <= kChunk steps: the kernel pairs with step offsets 0..m-1, the per-step means
    // of the accu steps (from the per-CTA sums), then the device step counter += m.
    // persistent tcr: clear the grid barrier's words, then one cooperative launch of m steps
    void launch_persistent(bool accu, uint32_t m, cudaStream_t st) {
        static_assert(offsetof(bay_ctl, gbar_count) == 128 && offsetof(bay_ctl, abort) == 256,
                      "grid barrier words of bay_ctl");
        cuda_check(cudaMemsetAsync(&ctl->gbar_count, 0,
                                   offsetof(bay_ctl, abort) + sizeof(unsigned int) - offsetof(bay_ctl, gbar_count),
                                   st),
                   "memset(grid barrier)");
        if (st == ctx->stream) bay::count_launches(1);
        bay_stretch_params p = make_params(0, 0);
        void* args[] = {&p, &m};
        CUlaunchAttribute at[1];
        at[0].id = CU_LAUNCH_ATTRIBUTE_COOPERATIVE;
        at[0].value.cooperative = 1;
        CUlaunchConfig cfg{};
        cfg.gridDimX = tr_grid;
        cfg.gridDimY = 1;
        cfg.gridDimZ = 1;
        cfg.blockDimX = 256 * kTrGroups;
        cfg.blockDimY = 1;
        cfg.blockDimZ = 1;
        cfg.sharedMemBytes = (unsigned)tr_smem;
        cfg.hStream = (CUstream)st;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        cu_check(g_cu.LaunchKernelEx(&cfg, (CUfunction)model->k_tr[accu ? 4 : 3], args, nullptr),
                 "cuLaunchKernelEx(stretch, persistent)");
    }

    bool use_persistent() const { return tcr && persistent && tr_grid != 0; }

    // per-launch resident tensor-core accu steps sum each half-step's positions in the
    // next launch; the chunk's last half-step has a statistics launch of its own
    bool tail_stats(bool accu) const { return accu && means_cap && tcr && !use_persistent(); }

    // kernels one run_chunk of m steps launches
    uint32_t chunk_launches(bool accu, uint32_t m) const {
        const uint32_t moves = use_persistent() ? 1u : (streaming ? 6u : 2u) * m;
        return moves + 1u + ((accu && means_cap) ? 1u : 0u) + (tail_stats(accu) ? 1u : 0u);
    }

    void run_chunk(bool accu, uint32_t m, cudaStream_t st) {
        if (use_persistent()) {
            launch_persistent(accu, m, st);
        } else {
            for (uint32_t i = 0; i < m; ++i) {
                launch_half(accu, 0, i, st);
                launch_half(accu, 1, i, st);
            }
            if (tail_stats(accu)) {
                if (st == ctx->stream) bay::count_launches(1);
                bay_stretch_params p = make_params(1, m - 1);
                void* args[] = {&p};
                cu_check(g_cu.LaunchKernel((CUfunction)model->k_tr[5], grid(), 1, 1, 256, 1, 1, 0,
                                           (CUstream)st, args, nullptr),
                         "cuLaunchKernel(statistics)");
            }
        }
        if (accu && means_cap)
            cuda_check(bay::launch_reduce_means(ctl, part, means,
                                                (uint32_t)std::min<uint64_t>(means_cap, 0xffffffffull),
                                                grid(), D, m, 1.0 / (double)W, st),
                       "reduce_means");
        bay_ctl_op op{};
        op.mask = accu ? BAY_CTL_ADD_STEP1 : BAY_CTL_ADD_STEP0;
        op.step[accu ? 1 : 0] = m;
        cuda_check(bay::launch_ctl_apply(ctl, op, st), "ctl_apply(step)");
    }

    cudaGraphExec_t capture_chunk(bool accu) {
        cudaStream_t cs = ctx->capture;
        cuda_check(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "BeginCapture");
        try {
            run_chunk(accu, kChunk, cs);
        } catch (...) {
            cudaGraph_t g;
            cudaStreamEndCapture(cs, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        cudaGraph_t g = nullptr;
        cuda_check(cudaStreamEndCapture(cs, &g), "EndCapture");
        cudaGraphExec_t ex = nullptr;
        const cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        cuda_check(e, "cudaGraphInstantiate");
        return ex;
    }

    // n steps of the bare (accu = false) or accu kernel pair, advancing the device
    // step counter; graph replay for whole chunks.
    void steps(bool accu, uint64_t n) {
        uint64_t done = 0;
        if (graphs && n >= kChunk) {
            cudaGraphExec_t& ex = accu ? g_accu : g_bare;
            if (accu && ex && g_accu_cap != means_cap) {
                cudaGraphExecDestroy(ex);
                ex = nullptr;
            }
            if (!ex) {
                ex = capture_chunk(accu);
                if (accu) g_accu_cap = means_cap;
            }
            for (; done + kChunk <= n; done += kChunk) {
                cuda_check(cudaGraphLaunch(ex, ctx->stream), "cudaGraphLaunch");
                bay::count_launches(chunk_launches(accu, kChunk));
            }
        }
        while (done < n) {
            const uint32_t m = (uint32_t)std::min<uint64_t>(kChunk, n - done);
            run_chunk(accu, m, ctx->stream);
            done += m;
        }
        if (accu) step_accu += (uint32_t)n;
        else step_bare += (uint32_t)n;
    }

    void set_a_beta(float a_, float beta_) {
        a = a_;
        beta = beta_;
        bay_ctl_op op{};
        op.mask = BAY_CTL_SET_A | BAY_CTL_SET_BETA;
        op.a = a_;
        op.beta = beta_;
        ctl_op(op);
    }

    void ensure_means(uint64_t n) {
        if (means_cap >= n && means) return;
        ctx->release(means);
        means = nullptr;
        means_cap = 0;
        means = (float*)ctx->alloc(sizeof(float) * (size_t)D * (size_t)std::max<uint64_t>(n, 1));
        means_cap = n;
    }

    void require_positions() const {
        if (!positioned)
            fail(BAY_ERR_STATE, "the sampler has no walker positions: call init-position first");
    }

    void destroy_graphs() {
        if (g_bare) cudaGraphExecDestroy(g_bare);
        if (g_accu) cudaGraphExecDestroy(g_accu);
        g_bare = g_accu = nullptr;
    }
};

// ============================================================================ C ABI
extern "C" {

const char* bay_last_error(void) { return g_err.c_str(); }

void bay_version(int* major, int* minor) {
    if (major) *major = 0;
    if (minor) *minor = 1;
}

int bay_ctx_create(const bay_ctx_opts* opts, bay_ctx** out) {
    return guarded([&] {
        if (!out) fail(BAY_ERR_ARG, "out is NULL");
        *out = nullptr;
        bay_ctx* c = new bay_ctx();
        try {
            c->device = opts ? opts->device : 0;
            c->wgs = (opts && opts->wgs) ? opts->wgs : 1024u;
            c->mem_limit = opts ? opts->mem_limit : 0;
            if (c->wgs < 2 || c->wgs > 1024 || (c->wgs & (c->wgs - 1)))
                fail(BAY_ERR_ARG, "wgs must be a power of two in [2, 1024]");
            int n = 0;
            cuda_check(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
            if (c->device < 0 || c->device >= n) fail(BAY_ERR_ARG, "no such CUDA device");
            c->use();
            cuda_check(cudaFree(nullptr), "context init");
            load_driver_api();
            cuda_check(cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount,
                                              c->device),
                       "cudaDeviceGetAttribute");
            if (opts && opts->stream) {
                c->stream = (cudaStream_t)opts->stream;
            } else {
                cuda_check(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking),
                           "cudaStreamCreate");
                c->own_stream = true;
            }
            cuda_check(cudaStreamCreateWithFlags(&c->capture, cudaStreamNonBlocking),
                       "cudaStreamCreate(capture)");
            cuda_check(bay::acor_noalloc_scratch(&c->acor_scratch),
                       "cudaGetSymbolAddress(acor scratch)");
        } catch (...) {
            if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
            if (c->capture) cudaStreamDestroy(c->capture);
            delete c;
            throw;
        }
        *out = c;
    });
}

int bay_ctx_release(bay_ctx* c) {
    return guarded([&] {
        if (!c) return;
        c->use();
        cudaStreamSynchronize(c->stream);
        for (auto& kv : c->sizes) cudaFree(kv.first);
        if (c->direct_lib) g_cu.LibraryUnload(c->direct_lib);
        for (auto& kv : c->hist_fastdiv) g_cu.LibraryUnload(kv.second.first);
        if (c->own_stream) cudaStreamDestroy(c->stream);
        cudaStreamDestroy(c->capture);
        delete c;
    });
}

int bay_ctx_processing_elements(bay_ctx* c, uint64_t* out) {
    return guarded([&] {
        if (!c || !out) fail(BAY_ERR_ARG, "NULL argument");
        *out = (uint64_t)c->sm_count * c->wgs;
    });
}

int bay_ctx_stream(bay_ctx* c, void** s) {
    return guarded([&] {
        if (!c || !s) fail(BAY_ERR_ARG, "NULL argument");
        *s = (void*)c->stream;
    });
}

int bay_ctx_synchronize(bay_ctx* c) {
    return guarded([&] {
        if (!c) fail(BAY_ERR_ARG, "NULL context");
        c->use();
        cuda_check(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    });
}

int bay_launch_count(uint64_t* out) {
    return guarded([&] {
        if (!out) fail(BAY_ERR_ARG, "NULL argument");
        *out = bay::launch_count();
    });
}

int bay_ctx_allocated(bay_ctx* c, uint64_t* out) {
    return guarded([&] {
        if (!c || !out) fail(BAY_ERR_ARG, "NULL argument");
        *out = c->allocated;
    });
}

}  // extern "C"

namespace {
struct Codegen {
    std::string src;
    std::vector<std::string> opts;
    uint32_t cta = 256, wpc = 1;
    uint32_t tc_g = 0, tc_stages = 0;
    size_t tc_smem = 0;
    uint32_t tr_g = 1;
};

// Source and NVRTC options of a model's fused kernels (the reference's stretch-options,
// nvidia_gtx.clj:630-633, retargeted to sm_103a).
Codegen codegen(const bay_model_desc* d, uint32_t wgs) {
    if (!d) fail(BAY_ERR_ARG, "NULL model description");
    if (!d->source) fail(BAY_ERR_ARG, "model source is NULL");
    if (d->dim == 0 || d->dim > 4096) fail(BAY_ERR_ARG, "dim must be in [1, 4096]");
    Codegen g;
    uint32_t cta = d->cta_threads ? d->cta_threads : 256u;
    if (d->form == BAY_FORM_GEMM) cta = 256;  // the GEMM tile assumes 16 x 16 thread groups
    if (cta % 32 || cta > 1024) fail(BAY_ERR_ARG, "cta_threads must be a multiple of 32, <= 1024");
    std::vector<std::string>& opts = g.opts;
    opts = {"-arch=sm_103a", "-use_fast_math", "-default-device", "-std=c++17", "-DREAL=float",
            "-DREAL2=float2", "-DACCUMULATOR=float"};
    opts.push_back("-DDIM=" + std::to_string(d->dim));
    opts.push_back("-DWGS=" + std::to_string(wgs));
    opts.push_back("-DBAY_CTA=" + std::to_string(cta));
    opts.push_back(std::string("-DBAY_ACCEPT_REF=") +
                   ((d->flags & BAY_MODEL_ACCEPT_REF) ? "1" : "0"));
    opts.push_back(std::string("-DBAY_STRETCH_REF=") +
                   ((d->flags & BAY_MODEL_STRETCH_REF) ? "1" : "0"));
    if (d->flags & BAY_MODEL_PARTNER_ELEMENT) {
        if (d->form != BAY_FORM_PLAIN && d->form != BAY_FORM_TILED)
            fail(BAY_ERR_ARG, "BAY_MODEL_PARTNER_ELEMENT applies to the plain and tiled forms");
        opts.push_back("-DBAY_PARTNER_ELEMENT=1");
    }
    uint32_t wpc = 1;
    if (d->form == BAY_FORM_PLAIN) {
        if (!valid_ident(d->logfn)) fail(BAY_ERR_ARG, "logfn must name a C function");
        opts.push_back(std::string("-DBAY_LOGFN=") + d->logfn);
    } else if (d->form == BAY_FORM_TILED) {
        if (!valid_ident(d->tile_prep) || !valid_ident(d->tile_term) ||
            !valid_ident(d->tile_walker))
            fail(BAY_ERR_ARG, "tiled form needs tile_prep, tile_term and tile_walker names");
        if (d->row_len == 0 || d->row_len > 64) fail(BAY_ERR_ARG, "row_len must be in [1, 64]");
        const uint32_t pl = d->prep_len ? d->prep_len : 1u;
        if (pl > 64) fail(BAY_ERR_ARG, "prep_len must be <= 64");
        wpc = d->walkers_per_cta ? d->walkers_per_cta : 8u;
        if (wpc > 32 || wpc > cta || (wpc & (wpc - 1)))
            fail(BAY_ERR_ARG, "walkers_per_cta must be a power of two, <= 32 and <= cta_threads");
        if (d->tile_slices > 16) fail(BAY_ERR_ARG, "tile_slices must be 0..16");
        opts.push_back("-DBAY_TILED=1");
        opts.push_back("-DBAY_ROW_LEN=" + std::to_string(d->row_len));
        opts.push_back("-DBAY_PREP_LEN=" + std::to_string(pl));
        opts.push_back("-DBAY_WPC=" + std::to_string(wpc));
        opts.push_back(std::string("-DBAY_TILE_PREP=") + d->tile_prep);
        opts.push_back(std::string("-DBAY_TILE_TERM=") + d->tile_term);
        opts.push_back(std::string("-DBAY_TILE_WALKER=") + d->tile_walker);
    } else if (d->form == BAY_FORM_GEMM) {
        if (!valid_ident(d->tile_prep) || !valid_ident(d->tile_term) ||
            !valid_ident(d->tile_walker))
            fail(BAY_ERR_ARG, "GEMM form needs tile_prep, tile_term and tile_walker names");
        if (d->gemm_features == 0 || d->gemm_coef + d->gemm_features > d->dim)
            fail(BAY_ERR_ARG, "gemm_coef + gemm_features must be within the walker dimension");
        if (d->gemm_ld < d->gemm_features) fail(BAY_ERR_ARG, "gemm_ld must be >= gemm_features");
        if (d->gemm_aux_len > 8 || (d->gemm_aux_len && d->gemm_aux_col + d->gemm_aux_len > d->gemm_ld))
            fail(BAY_ERR_ARG, "aux columns must lie inside a row (at most 8)");
        const uint32_t pl = d->prep_len ? d->prep_len : 1u;
        if (pl > 64) fail(BAY_ERR_ARG, "prep_len must be <= 64");
        opts.push_back("-DBAY_GEMM=1");
        opts.push_back("-DBAY_GEMM_F=" + std::to_string(d->gemm_features));
        opts.push_back("-DBAY_GEMM_COEF=" + std::to_string(d->gemm_coef));
        opts.push_back("-DBAY_GEMM_AUX=" + std::to_string(d->gemm_aux_len));
        opts.push_back("-DBAY_GEMM_AUXCOL=" + std::to_string(d->gemm_aux_col));
        opts.push_back("-DBAY_PREP_LEN=" + std::to_string(pl));
        opts.push_back(std::string("-DBAY_GEMM_PREP=") + d->tile_prep);
        opts.push_back(std::string("-DBAY_GEMM_TERM=") + d->tile_term);
        opts.push_back(std::string("-DBAY_GEMM_WALKER=") + d->tile_walker);
        if (d->flags & BAY_MODEL_GEMM_TENSOR) {
            if (!tc_plan(d->gemm_features, d->gemm_aux_len, &g.tc_g, &g.tc_stages, &g.tc_smem))
                fail(BAY_ERR_ARG, "tensor-core GEMM form: at most 320 features");
            if ((d->tc_subtiles || d->tc_stages) &&
                !tc_plan(d->gemm_features, d->gemm_aux_len, &g.tc_g, &g.tc_stages, &g.tc_smem,
                         d->tc_subtiles, d->tc_stages))
                fail(BAY_ERR_ARG, "tensor-core GEMM form: the asked sub-tiles / stages do not fit "
                                  "in shared memory");
            if (d->tc_groups > 2) fail(BAY_ERR_ARG, "tc_groups must be 0, 1 or 2");
            g.tr_g = d->tc_groups ? d->tc_groups : 1u;
            opts.push_back("-DBAY_TR_G=" + std::to_string(g.tr_g) + "u");
            opts.push_back("-DBAY_GEMM_TC=1");
            opts.push_back("-DBAY_TC_G=" + std::to_string(g.tc_g));
            opts.push_back("-DBAY_TC_STAGES=" + std::to_string(g.tc_stages));
            opts.push_back("-DBAY_TR_W=" + std::to_string(kTrWalkers) + "u");
        }
        wpc = 64;
    } else if (d->form == BAY_FORM_BATCH) {
        if (!valid_ident(d->tile_prep) || !valid_ident(d->tile_term) ||
            !valid_ident(d->tile_walker))
            fail(BAY_ERR_ARG, "batch form needs tile_prep, tile_term and tile_walker names");
        if (d->row_len == 0 || d->row_len > 64) fail(BAY_ERR_ARG, "row_len must be in [1, 64]");
        const uint32_t pl = d->prep_len ? d->prep_len : 1u;
        if (pl > 64) fail(BAY_ERR_ARG, "prep_len must be <= 64");
        opts.push_back("-DBAY_ROW_LEN=" + std::to_string(d->row_len));
        opts.push_back("-DBAY_PREP_LEN=" + std::to_string(pl));
        opts.push_back(std::string("-DBAY_TILE_PREP=") + d->tile_prep);
        opts.push_back(std::string("-DBAY_TILE_TERM=") + d->tile_term);
        opts.push_back(std::string("-DBAY_TILE_WALKER=") + d->tile_walker);
    } else {
        fail(BAY_ERR_ARG, "unknown model form");
    }
    std::string& src = g.src;
    src += "#include <stdint.h>\n";
    src += bay_embedded_rng;
    src += "\n#line 1 \"model\"\n";
    src += d->source;
    if (d->form == BAY_FORM_BATCH) {
        src += "\n#line 1 \"bay_batch.cuh\"\n";
        src += bay_embedded_batch;
    } else {
        src += "\n#line 1 \"bay_stretch.cuh\"\n";
        src += bay_embedded_stretch;
    }
    g.cta = cta;
    g.wpc = wpc;
    return g;
}
}  // namespace

extern "C" {

int bay_model_check(const bay_model_desc* d, uint32_t wgs) {
    return guarded([&] {
        Codegen g = codegen(d, wgs ? wgs : 1024u);
        nvrtc_compile(g.src, g.opts);
    });
}

int bay_model_compile(bay_ctx* c, const bay_model_desc* d, bay_model** out) {
    NvtxRange trace_("bay_model_compile");
    return guarded([&] {
        if (!c || !d || !out) fail(BAY_ERR_ARG, "NULL argument");
        *out = nullptr;
        std::lock_guard<std::recursive_mutex> lk(c->mu);
        c->use();
        Codegen g = codegen(d, c->wgs);
        std::vector<char> cubin = nvrtc_compile(g.src, g.opts);
        bay_model* m = new bay_model();
        m->ctx = c;
        m->dim = d->dim;
        m->params_size = d->params_size;
        m->form = d->form;
        m->cta = g.cta;
        m->wpc = g.wpc;
        m->flags = d->flags;
        if (d->form == BAY_FORM_TILED) m->tslices = d->tile_slices ? d->tile_slices : 1u;
        if (d->form == BAY_FORM_TILED) m->row_len = d->row_len;
        if (d->form == BAY_FORM_GEMM) {
            m->prep_len = d->prep_len ? d->prep_len : 1u;
            m->gemm_features = d->gemm_features;
            m->gemm_block = d->gemm_block;
            m->gemm_ld = d->gemm_ld;
            m->gemm_aux_col = d->gemm_aux_col;
            m->gemm_aux_len = d->gemm_aux_len;
            m->gemm_offset = d->gemm_offset;
            m->gemm_rows = d->gemm_rows;
            m->tc_g = g.tc_g;
            m->tc_stages = g.tc_stages;
            m->tc_smem = g.tc_smem;
            m->tr_g = g.tr_g;
        }
        try {
            cu_check(g_cu.LibraryLoadData(&m->lib, cubin.data(), nullptr, nullptr, 0, nullptr,
                                       nullptr, 0),
                     "cuLibraryLoadData");
            if (d->form == BAY_FORM_BATCH) {
                const char* bp[3] = {"bay_batch_propose_bare", "bay_batch_propose_accu",
                                     "bay_batch_propose_logfn"};
                const char* ba[3] = {"bay_batch_accept_bare", "bay_batch_accept_accu",
                                     "bay_batch_accept_logfn"};
                for (int i = 0; i < 3; ++i) {
                    cu_check(g_cu.LibraryGetKernel(&m->k_gp[i], m->lib, bp[i]), "GetKernel(propose)");
                    cu_check(g_cu.LibraryGetKernel(&m->k_ga[i], m->lib, ba[i]), "GetKernel(accept)");
                }
                cu_check(g_cu.LibraryGetKernel(&m->k_gr[0], m->lib, "bay_batch_rows_move"), "GetKernel(rows)");
                cu_check(g_cu.LibraryGetKernel(&m->k_gr[1], m->lib, "bay_batch_rows_logfn"), "GetKernel(rows)");
                const char* rw[3][2] = {{"bay_batch_rows_move", "bay_batch_rows_logfn"},
                                        {"bay_batch_rows_move2", "bay_batch_rows_logfn2"},
                                        {"bay_batch_rows_move4", "bay_batch_rows_logfn4"}};
                for (int q = 0; q < 3; ++q)
                    for (int i = 0; i < 2; ++i)
                        cu_check(g_cu.LibraryGetKernel(&m->k_gr_wpt[q][i], m->lib, rw[q][i]),
                                 "GetKernel(rows)");
                const char* br[2][3] = {{"bay_batch_run_bare", "bay_batch_run_bare2", "bay_batch_run_bare4"},
                                        {"bay_batch_run_accu", "bay_batch_run_accu2", "bay_batch_run_accu4"}};
                for (int i = 0; i < 2; ++i)
                    for (int q = 0; q < 3; ++q)
                        cu_check(g_cu.LibraryGetKernel(&m->k_brun[i][q], m->lib, br[i][q]),
                                 "GetKernel(batch run)");
                // row chunks of up to kBatchSmemMax bytes of shared memory (opt-in above 48 KB)
                CUdevice dev = (CUdevice)c->device;
                for (int q = 0; q < 3; ++q)
                    for (CUkernel k : {m->k_gr_wpt[q][0], m->k_gr_wpt[q][1], m->k_brun[0][q], m->k_brun[1][q]})
                        cu_check(g_cu.KernelSetAttribute(CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES,
                                                         (int)kBatchSmemMax, k, dev),
                                 "cuKernelSetAttribute(smem)");
                cu_check(g_cu.LibraryGetKernel(&m->k_bmeans, m->lib, "bay_batch_means"), "GetKernel(means)");
                m->row_len = d->row_len;
                m->prep_len = d->prep_len ? d->prep_len : 1u;
            } else {
                cu_check(g_cu.LibraryGetKernel(&m->k_bare, m->lib, "bay_stretch_bare"), "GetKernel(bare)");
                cu_check(g_cu.LibraryGetKernel(&m->k_accu, m->lib, "bay_stretch_accu"), "GetKernel(accu)");
                cu_check(g_cu.LibraryGetKernel(&m->k_logfn, m->lib, "bay_logfn_all"), "GetKernel(logfn)");
                if (d->form == BAY_FORM_PLAIN) {
                    cu_check(g_cu.LibraryGetKernel(&m->k_points, m->lib, "bay_points_logfn"),
                             "GetKernel(points)");
                    cu_check(g_cu.LibraryGetKernel(&m->k_evidence, m->lib, "bay_points_evidence"),
                             "GetKernel(evidence)");
                }
            }
            if (d->form == BAY_FORM_TILED) {
                CUdevice dev = (CUdevice)c->device;
                for (CUkernel k : {m->k_bare, m->k_accu, m->k_logfn})
                    cu_check(g_cu.KernelSetAttribute(CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES,
                                                     (int)(2 * kTileChunk * sizeof(float)), k, dev),
                             "cuKernelSetAttribute(smem)");
            }
            if (d->form == BAY_FORM_GEMM) {
                const char* gp[3] = {"bay_gemm_propose_bare", "bay_gemm_propose_accu",
                                     "bay_gemm_propose_logfn"};
                const char* ga[3] = {"bay_gemm_accept_bare", "bay_gemm_accept_accu",
                                     "bay_gemm_accept_logfn"};
                for (int i = 0; i < 3; ++i) {
                    cu_check(g_cu.LibraryGetKernel(&m->k_gp[i], m->lib, gp[i]), "GetKernel(propose)");
                    cu_check(g_cu.LibraryGetKernel(&m->k_ga[i], m->lib, ga[i]), "GetKernel(accept)");
                }
                cu_check(g_cu.LibraryGetKernel(&m->k_gr[0], m->lib, "bay_gemm_rows_move"), "GetKernel(rows)");
                cu_check(g_cu.LibraryGetKernel(&m->k_gr[1], m->lib, "bay_gemm_rows_logfn"), "GetKernel(rows)");
                CUdevice dev = (CUdevice)c->device;
                for (CUkernel k : {m->k_bare, m->k_accu, m->k_logfn, m->k_gr[0], m->k_gr[1]})
                    cu_check(g_cu.KernelSetAttribute(CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES,
                                                     (int)kGemmMaxSmem, k, dev),
                             "cuKernelSetAttribute(smem)");
                if (m->tc_g) {
                    cu_check(g_cu.LibraryGetKernel(&m->k_gt[0], m->lib, "bay_gemm_rows_tc_move"),
                             "GetKernel(rows tc)");
                    cu_check(g_cu.LibraryGetKernel(&m->k_gt[1], m->lib, "bay_gemm_rows_tc_logfn"),
                             "GetKernel(rows tc)");
                    for (CUkernel k : {m->k_gt[0], m->k_gt[1]})
                        cu_check(g_cu.KernelSetAttribute(CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES,
                                                         (int)m->tc_smem, k, dev),
                                 "cuKernelSetAttribute(smem)");
                    const char* tr[6] = {"bay_tcr_bare", "bay_tcr_accu", "bay_tcr_logfn",
                                         "bay_tcr_run_bare", "bay_tcr_run_accu", "bay_tcr_stats"};
                    for (int i = 0; i < 6; ++i) {
                        cu_check(g_cu.LibraryGetKernel(&m->k_tr[i], m->lib, tr[i]), "GetKernel(tcr)");
                        cu_check(g_cu.KernelSetAttribute(CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES,
                                                         (int)kGemmMaxSmem, m->k_tr[i], dev),
                                 "cuKernelSetAttribute(smem)");
                        // the whole carveout as shared memory: 4 CTAs of about 50 KB per SM
                        cu_check(g_cu.KernelSetAttribute(CU_FUNC_ATTRIBUTE_PREFERRED_SHARED_MEMORY_CARVEOUT,
                                                         100, m->k_tr[i], dev),
                                 "cuKernelSetAttribute(carveout)");
                    }
                }
            }
        } catch (...) {
            if (m->lib) g_cu.LibraryUnload(m->lib);
            delete m;
            throw;
        }
        *out = m;
    });
}

int bay_model_release(bay_model* m) {
    return guarded([&] {
        if (!m) return;
        if (m->lib) g_cu.LibraryUnload(m->lib);
        delete m;
    });
}

static int sampler_create(bay_model* m, uint32_t seed, uint64_t walkers, const float* params,
                          uint64_t n_params, bool device_params, bay_sampler** out) {
    return guarded([&] {
        if (!m || !out) fail(BAY_ERR_ARG, "NULL argument");
        *out = nullptr;
        if (walkers < 4 || walkers % 2)
            fail(BAY_ERR_ARG, "Number of walkers (" + std::to_string(walkers) +
                                  ") must be even and at least 4.");
        if (walkers > 0xffffffffull / 2) fail(BAY_ERR_ARG, "too many walkers");
        if (n_params < m->params_size)
            fail(BAY_ERR_ARG, "Dimension of params must match the distribution: need at least " +
                                  std::to_string(m->params_size) + " values, got " +
                                  std::to_string(n_params));
        if (n_params && !params) fail(BAY_ERR_ARG, "params is NULL");
        bay_ctx* c = m->ctx;
        std::lock_guard<std::recursive_mutex> lk(c->mu);
        c->use();
        bay_sampler* s = new bay_sampler();
        s->model = m;
        s->ctx = c;
        s->W = walkers;
        s->K = walkers / 2;
        s->D = m->dim;
        s->n_params = n_params;
        s->data_len = n_params - m->params_size;
        if (m->form == BAY_FORM_TILED) {
            s->smem = tile_smem_bytes(m->row_len, s->data_len);   // the log-density launch
            // a move launch's CTA stages one row slice: (n / slices rounded up to 4) rows
            const uint64_t n_rows = s->data_len / m->row_len, ns = m->tslices;
            const uint64_t rps = ns > 1 ? (((n_rows + ns - 1) / ns + 3) & ~3ull) : n_rows;
            s->smem_move = tile_smem_bytes(m->row_len, std::min(rps, n_rows) * m->row_len);
        }
        if (m->form == BAY_FORM_GEMM) {
            const uint64_t block = m->gemm_block ? s->data_len : 0;
            const uint64_t block_len = m->gemm_block ? m->params_size : s->data_len;
            if (m->gemm_offset > block_len) {
                delete s;
                fail(BAY_ERR_ARG, "gemm_offset lies past the end of its params block");
            }
            s->gemm_base = block + m->gemm_offset;
            s->gemm_rows = m->gemm_rows ? m->gemm_rows : (block_len - m->gemm_offset) / m->gemm_ld;
            const uint64_t row_need = std::max<uint64_t>(m->gemm_features,
                                                         m->gemm_aux_col + m->gemm_aux_len);
            if (s->gemm_rows == 0 ||
                m->gemm_offset + (s->gemm_rows - 1) * m->gemm_ld + row_need > block_len) {
                delete s;
                fail(BAY_ERR_ARG, "the GEMM matrix does not fit its params block");
            }
            s->smem = gemm_smem_bytes(m, s->gemm_rows);
            s->tc = m->tc_g != 0;
            if (s->tc && !(m->flags & BAY_MODEL_GEMM_STREAMING) && s->gemm_rows <= 256 &&
                m->gemm_features <= 256) {
                // resident on the tensor cores when the image, the walker operand and the
                // proposals fit (layout in bay_stretch_tcr)
                const uint64_t np = (s->gemm_rows + 15) & ~15ull, kc = (m->gemm_features + 63) / 64;
                const uint64_t auxs = m->gemm_aux_len ? m->gemm_aux_len : 1;
                const uint64_t img = 2 * kc * np * 128 + np * auxs * 4;
                // image, then per tile group 2 kc atoms of kTrWalkers walker rows, the
                // proposals and the reduction scratch -- at least the part of the M = 128
                // MMA's 16 KB read that runs past the last atom (walker rows kTrWalkers..127,
                // never read back); the group stride is BAY_TR_GREG of the kernel
                const uint64_t atom = 128ull * kTrWalkers;
                const uint64_t tail = (std::max<uint64_t>(16384 - atom,
                                                          (uint64_t)kTrWalkers * (m->dim | 1u) * 4 + 2048) +
                                       1023) & ~1023ull;
                const uint64_t greg = 2 * kc * atom + tail;
                const uint64_t base = 1024 + ((img + 1023) & ~1023ull);
                if (base + greg <= kGemmMaxSmem) {
                    s->tc = false;
                    s->tcr = true;
                    s->smem = (size_t)(base + greg);
                    s->tr_g = (base + m->tr_g * greg <= kGemmMaxSmem) ? m->tr_g : 1u;
                    s->smem_move = (size_t)(base + s->tr_g * greg);
                    s->gemm_np = (uint32_t)np;
                    // persistent form: kTrGroups groups per CTA, their accumulators within
                    // the SM's 512 TMEM columns
                    const uint64_t ncols = np <= 32 ? 32 : np <= 64 ? 64 : np <= 128 ? 128 : 256;
                    const uint64_t smp = base + kTrGroups * greg;
                    if (kTrGroups * ncols <= 512 && smp <= kGemmMaxSmem) s->tr_smem = (size_t)smp;
                }
            }
            s->streaming = s->tc || (!s->tcr && ((m->flags & BAY_MODEL_GEMM_STREAMING) ||
                                                  s->smem > kGemmMaxSmem));
            if (s->tc) {
                // rows kernel on the tensor cores: one CTA per SM over (walker groups x
                // row super-blocks), one wave; super-blocks are whole 128-row tiles
                s->smem = 0;
                if (s->gemm_rows > 0x7fffff00ull) {
                    delete s;
                    fail(BAY_ERR_ARG, "tensor-core GEMM form: at most 2^31 - 256 rows");
                }
                const uint64_t n_tiles = (s->gemm_rows + 127) / 128;
                const uint64_t per = 128ull * m->tc_g;
                const uint64_t n_wg = (s->K + per - 1) / per;
                uint64_t nsb = std::max<uint64_t>(1, (uint64_t)c->sm_count / n_wg);
                nsb = std::min<uint64_t>(nsb, n_tiles);
                const uint64_t tiles = (n_tiles + nsb - 1) / nsb;
                s->s_sbrows = (uint32_t)(tiles * 128);
                s->s_nsb = (uint32_t)((s->gemm_rows + s->s_sbrows - 1) / s->s_sbrows);
                s->tc_fp = (m->gemm_features + 63) & ~63u;
                s->tc_rows_pad = n_tiles * 128;
                s->tc_wpad = (walkers + per - 1) / per * per;
            } else if (s->streaming) {
                // rows kernel: the coefficient tile (F x 128) + one 32-feature matrix chunk
                s->smem = 0;
                s->smem_rows = sizeof(float) * ((size_t)m->gemm_features * 128 + 32 * 129);
                if (s->smem_rows > kGemmMaxSmem || s->gemm_rows > 0xffffffffull) {
                    delete s;
                    fail(BAY_ERR_ARG, "GEMM form: at most 384 features and 2^32 - 1 rows");
                }
                // row super-blocks: about 8 CTAs per SM over (walker tiles x super-blocks)
                const uint64_t n_sub = (s->gemm_rows + 127) / 128;
                const uint64_t n_wt = (s->K + 127) / 128;
                const uint64_t target = 8ull * (uint64_t)c->sm_count;
                uint64_t nsb = (target + n_wt - 1) / n_wt;
                nsb = std::max<uint64_t>(1, std::min<uint64_t>(nsb, n_sub));
                const uint64_t per = (n_sub + nsb - 1) / nsb;
                s->s_sbrows = (uint32_t)(per * 128);
                s->s_nsb = (uint32_t)((s->gemm_rows + s->s_sbrows - 1) / s->s_sbrows);
            }
        }
        try {
            s->xs = (float*)c->alloc(sizeof(float) * (size_t)s->D * walkers);
            s->logfn = (float*)c->alloc(sizeof(float) * walkers);
            s->ctl = (bay_ctl*)c->alloc(sizeof(bay_ctl));
            s->part = (float*)c->alloc(sizeof(float) * kChunk * 2 * (size_t)s->grid() * s->D);
            if (m->form == BAY_FORM_TILED && m->tslices > 1) {
                s->t_part = (float*)c->alloc(sizeof(float) * 2 * (size_t)s->K * m->tslices);
                s->t_ticket = (unsigned int*)c->alloc(sizeof(unsigned int) * s->grid());
                cuda_check(cudaMemsetAsync(s->t_ticket, 0, sizeof(unsigned int) * s->grid(), c->stream),
                           "memset(tickets)");
            }
            s->stats = (double*)c->alloc(sizeof(double) * 2 * s->D);
            cuda_check(cudaMemsetAsync(s->ctl, 0, sizeof(bay_ctl), c->stream), "memset");
            cuda_check(cudaMemsetAsync(s->xs, 0, sizeof(float) * (size_t)s->D * walkers, c->stream),
                       "memset");
            cuda_check(cudaMemsetAsync(s->logfn, 0, sizeof(float) * walkers, c->stream), "memset");
            if (device_params) {
                if ((uintptr_t)params % 16) fail(BAY_ERR_ARG, "d_params must be 16-byte aligned");
                s->params = params;
            } else {
                float* p = (float*)c->alloc(sizeof(float) * std::max<uint64_t>(n_params, 1));
                if (n_params)
                    cuda_check(cudaMemcpyAsync(p, params, sizeof(float) * n_params,
                                               cudaMemcpyHostToDevice, c->stream),
                               "cudaMemcpy(params)");
                s->params = p;
                s->own_params = true;
            }
            if (s->streaming) {
                const size_t Wn = walkers;
                s->s_y = (float*)c->alloc(sizeof(float) * Wn * s->D);
                s->s_b = (float*)c->alloc(sizeof(float) * Wn * m->gemm_features);
                s->s_prep = (float*)c->alloc(sizeof(float) * Wn * m->prep_len);
                s->s_w = (float*)c->alloc(sizeof(float) * Wn);
                s->s_zu = (float*)c->alloc(sizeof(float) * Wn * 2);
                s->s_part = (float*)c->alloc(sizeof(float) * Wn * 2 * s->s_nsb);
                if (s->tc) {
                    const uint32_t auxs = m->gemm_aux_len ? m->gemm_aux_len : 1u;
                    const size_t nx = (size_t)s->tc_rows_pad * s->tc_fp;
                    const size_t nb = (size_t)s->tc_wpad * s->tc_fp;
                    s->tc_xh = (unsigned short*)c->alloc(2 * nx);
                    s->tc_xl = (unsigned short*)c->alloc(2 * nx);
                    s->gemm_lay = (float*)c->alloc(sizeof(float) * (size_t)s->tc_rows_pad * auxs);
                    s->s_bh = (unsigned short*)c->alloc(2 * nb);
                    s->s_bl = (unsigned short*)c->alloc(2 * nb);
                    cuda_check(cudaMemsetAsync(s->s_bh, 0, 2 * nb, c->stream), "memset");
                    cuda_check(cudaMemsetAsync(s->s_bl, 0, 2 * nb, c->stream), "memset");
                    cuda_check(bay::launch_gemm_split(s->params + s->gemm_base, m->gemm_ld,
                                                      (uint32_t)s->gemm_rows, m->gemm_features,
                                                      s->tc_fp, s->tc_rows_pad, m->gemm_aux_col,
                                                      m->gemm_aux_len, auxs, s->tc_xh, s->tc_xl,
                                                      s->gemm_lay, c->stream),
                               "gemm_split");
                    encode_bf16_map(&s->tc_maps.xh, s->tc_xh, s->tc_fp, s->tc_rows_pad);
                    encode_bf16_map(&s->tc_maps.xl, s->tc_xl, s->tc_fp, s->tc_rows_pad);
                    encode_bf16_map(&s->tc_maps.bh, s->s_bh, s->tc_fp, s->tc_wpad);
                    encode_bf16_map(&s->tc_maps.bl, s->s_bl, s->tc_fp, s->tc_wpad);
                }
            } else if (s->tcr) {
                // persistent form: one CTA of kTrGroups tile groups per SM (all co-resident:
                // a cooperative launch), no more CTAs than tiles
                if (s->tr_smem) {
                    CUfunction f = nullptr;
                    cu_check(g_cu.KernelGetFunction(&f, m->k_tr[3]), "cuKernelGetFunction(tcr)");
                    int per_sm = 0;
                    cu_check(g_cu.OccupancyMaxActiveBlocks(&per_sm, f, 256 * kTrGroups, s->tr_smem),
                             "cuOccupancy(tcr)");
                    int n_sm = 0;
                    cuda_check(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, c->device),
                               "cudaDeviceGetAttribute(SMs)");
                    // one CTA per SM: its TMEM columns are the only ones a resident CTA holds
                    if (per_sm >= 1)
                        s->tr_grid = (uint32_t)std::min<uint64_t>(s->grid(), (uint64_t)n_sm);
                }
                const uint32_t auxs = m->gemm_aux_len ? m->gemm_aux_len : 1u;
                const uint32_t kc = (m->gemm_features + 63) / 64;
                const size_t img = 2ull * kc * s->gemm_np * 128 + (size_t)s->gemm_np * auxs * 4;
                s->gemm_lay = (float*)c->alloc(img);
                cuda_check(bay::launch_gemm_tc_image(s->params + s->gemm_base, m->gemm_ld,
                                                     (uint32_t)s->gemm_rows, m->gemm_features, kc,
                                                     s->gemm_np, m->gemm_aux_col, m->gemm_aux_len,
                                                     auxs, s->gemm_lay, c->stream),
                           "gemm_tc_image");
            } else if (m->form == BAY_FORM_GEMM) {
                s->gemm_np = (uint32_t)((s->gemm_rows + 63) & ~63ull);
                const uint32_t auxs = m->gemm_aux_len ? m->gemm_aux_len : 1u;
                s->gemm_lay = (float*)c->alloc(
                    sizeof(float) * ((size_t)m->gemm_features * s->gemm_np + (size_t)s->gemm_np * auxs));
                cuda_check(bay::launch_gemm_layout(s->params + s->gemm_base, m->gemm_ld,
                                                   (uint32_t)s->gemm_rows, m->gemm_features,
                                                   s->gemm_np, m->gemm_aux_col, m->gemm_aux_len,
                                                   auxs, s->gemm_lay, c->stream),
                           "gemm_layout");
            }
            s->ensure_means(1);
            // init! (nvidia_gtx.clj:391-400)
            s->seed_bare = seed;
            s->seed_accu = seed;
            bay_ctl_op op{};
            op.mask = BAY_CTL_SET_STEP0 | BAY_CTL_SET_STEP1 | BAY_CTL_SET_SEED0 | BAY_CTL_SET_SEED1 |
                      BAY_CTL_SET_A | BAY_CTL_SET_BETA | BAY_CTL_RESET_ACCEPTED |
                      BAY_CTL_RESET_TICKETS;
            op.seed[0] = seed;
            op.seed[1] = seed;
            op.a = 2.0f;
            op.beta = 1.0f;
            s->ctl_op(op);
        } catch (...) {
            c->release(s->xs);
            c->release(s->logfn);
            c->release(s->ctl);
            c->release(s->part);
            c->release(s->stats);
            c->release(s->means);
            c->release(s->gemm_lay);
            c->release(s->t_part);
            c->release(s->t_ticket);
            for (float* q : {s->s_y, s->s_b, s->s_prep, s->s_w, s->s_zu, s->s_part}) c->release(q);
            for (unsigned short* q : {s->tc_xh, s->tc_xl, s->s_bh, s->s_bl}) c->release(q);
            if (s->own_params) c->release((void*)s->params);
            delete s;
            throw;
        }
        *out = s;
    });
}

int bay_sampler_create(bay_model* m, uint32_t seed, uint64_t walkers, const float* params,
                       uint64_t n_params, bay_sampler** out) {
    NvtxRange trace_("bay_sampler_create");
    return sampler_create(m, seed, walkers, params, n_params, false, out);
}

int bay_sampler_create_device(bay_model* m, uint32_t seed, uint64_t walkers, const float* d_params,
                              uint64_t n_params, bay_sampler** out) {
    NvtxRange trace_("bay_sampler_create_device");
    return sampler_create(m, seed, walkers, d_params, n_params, true, out);
}

int bay_sampler_release(bay_sampler* s) {
    return guarded([&] {
        if (!s) return;
        bay_ctx* c = s->ctx;
        std::lock_guard<std::recursive_mutex> lk(c->mu);
        c->use();
        cudaStreamSynchronize(c->stream);
        s->destroy_graphs();
        c->release(s->xs);
        c->release(s->logfn);
        c->release(s->ctl);
        c->release(s->part);
        c->release(s->stats);
        c->release(s->means);
        c->release(s->stage);
        c->release(s->hist);
        c->release(s->counts);
        c->release(s->mix);
        c->release(s->gemm_lay);
        c->release(s->t_part);
        c->release(s->t_ticket);
        for (float* q : {s->s_y, s->s_b, s->s_prep, s->s_w, s->s_zu, s->s_part}) c->release(q);
        for (unsigned short* q : {s->tc_xh, s->tc_xl, s->s_bh, s->s_bl}) c->release(q);
        if (s->own_params) c->release((void*)s->params);
        delete s;
    });
}

int bay_sampler_info_get(bay_sampler* s, bay_sampler_info* out) {
    return guarded([&] {
        if (!s || !out) fail(BAY_ERR_ARG, "NULL argument");
        out->walkers = s->W;
        out->dim = s->D;
        out->wgs = s->ctx->wgs;
        out->iteration_counter = s->iteration_counter;
        out->data_len = s->data_len;
    });
}

int bay_sampler_set_graphs(bay_sampler* s, int enabled) {
    return guarded([&] {
        if (!s) fail(BAY_ERR_ARG, "NULL sampler");
        s->graphs = enabled != 0;
    });
}

int bay_sampler_test_barrier_timeout(bay_sampler* s, int enabled) {
    return guarded([&] {
        if (!s) fail(BAY_ERR_ARG, "NULL sampler");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        const uint32_t extra = enabled ? 1u : 0u;
        if (s->gbar_extra == extra) return;
        s->gbar_extra = extra;
        // the captured chunks hold the old parameter: capture again
        for (cudaGraphExec_t* g : {&s->g_bare, &s->g_accu})
            if (*g) {
                cuda_check(cudaStreamSynchronize(s->ctx->stream), "sync");
                cudaGraphExecDestroy(*g);
                *g = nullptr;
            }
    });
}

int bay_sampler_set_persistent(bay_sampler* s, int enabled) {
    return guarded([&] {
        if (!s) fail(BAY_ERR_ARG, "NULL sampler");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        if (s->persistent == (enabled != 0)) return;
        s->persistent = enabled != 0;
        // the captured chunks launch the other form's kernels: capture again
        for (cudaGraphExec_t* g : {&s->g_bare, &s->g_accu})
            if (*g) {
                cuda_check(cudaStreamSynchronize(s->ctx->stream), "sync");
                cudaGraphExecDestroy(*g);
                *g = nullptr;
            }
    });
}

int bay_init(bay_sampler* s, uint32_t seed) {
    return guarded([&] {
        if (!s) fail(BAY_ERR_ARG, "NULL sampler");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        s->seed_bare = seed;
        s->seed_accu = seed;
        s->step_bare = 0;
        s->a = 2.0f;
        s->beta = 1.0f;
        bay_ctl_op op{};
        op.mask = BAY_CTL_SET_SEED0 | BAY_CTL_SET_SEED1 | BAY_CTL_SET_STEP0 | BAY_CTL_SET_A |
                  BAY_CTL_SET_BETA;
        op.seed[0] = seed;
        op.seed[1] = seed;
        op.a = 2.0f;
        op.beta = 1.0f;
        s->ctl_op(op);
    });
}

int bay_init_position_limits(bay_sampler* s, uint32_t seed, const float* limits) {
    NvtxRange trace_("bay_init_position_limits");
    return guarded([&] {
        if (!s || !limits) fail(BAY_ERR_ARG, "NULL argument");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        float* dl = (float*)s->ctx->alloc(sizeof(float) * 2 * s->D);
        try {
            cuda_check(cudaMemcpyAsync(dl, limits, sizeof(float) * 2 * s->D, cudaMemcpyDefault,
                                       s->ctx->stream),
                       "cudaMemcpy(limits)");
            cuda_check(bay::launch_init_uniform(s->xs, s->D, s->W, seed, dl, s->ctx->stream),
                       "init_walkers");
            s->launch_logfn_all();
            cuda_check(cudaStreamSynchronize(s->ctx->stream), "sync");
        } catch (...) {
            s->ctx->release(dl);
            throw;
        }
        s->ctx->release(dl);
        s->positioned = true;
        s->iteration_counter = 0;
    });
}

int bay_init_position_normal(bay_sampler* s, uint32_t seed, float mean, float sd) {
    NvtxRange trace_("bay_init_position_normal");
    return guarded([&] {
        if (!s) fail(BAY_ERR_ARG, "NULL sampler");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        cuda_check(bay::launch_init_normal(s->xs, s->D, s->W, seed, mean, sd, s->ctx->stream),
                   "init_normal");
        s->launch_logfn_all();
        s->positioned = true;
        s->iteration_counter = 0;
    });
}

int bay_init_position_copy(bay_sampler* s, const bay_sampler* src) {
    NvtxRange trace_("bay_init_position_copy");
    return guarded([&] {
        if (!s || !src) fail(BAY_ERR_ARG, "NULL argument");
        if (src->D != s->D || src->W != s->W)
            fail(BAY_ERR_ARG, "source sampler has a different dimension or walker count");
        if (!src->positioned) fail(BAY_ERR_STATE, "source sampler has no positions");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        if (src->ctx != s->ctx) cuda_check(cudaStreamSynchronize(src->ctx->stream), "sync(src)");
        cuda_check(cudaMemcpyAsync(s->xs, src->xs, sizeof(float) * (size_t)s->D * s->W,
                                   cudaMemcpyDeviceToDevice, s->ctx->stream),
                   "cudaMemcpy(positions)");
        s->launch_logfn_all();
        s->positioned = true;
        s->iteration_counter = 0;
    });
}

int bay_init_position_host(bay_sampler* s, const float* positions) {
    NvtxRange trace_("bay_init_position_host");
    return guarded([&] {
        if (!s || !positions) fail(BAY_ERR_ARG, "NULL argument");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        cuda_check(cudaMemcpyAsync(s->xs, positions, sizeof(float) * (size_t)s->D * s->W,
                                   cudaMemcpyDefault, s->ctx->stream),
                   "cudaMemcpy(positions)");
        s->launch_logfn_all();
        cuda_check(cudaStreamSynchronize(s->ctx->stream), "sync");
        s->positioned = true;
        s->iteration_counter = 0;
    });
}

int bay_burn_in(bay_sampler* s, uint64_t n, float a) {
    NvtxRange trace_("bay_burn_in");
    return guarded([&] {
        if (!s) fail(BAY_ERR_ARG, "NULL sampler");
        if (!(a > 1.0f)) fail(BAY_ERR_ARG, "the stretch parameter a must be > 1");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        s->require_positions();
        s->set_a_beta(a, 1.0f);
        s->steps(false, n);
        s->iteration_counter += n;
    });
}

int bay_anneal(bay_sampler* s, const float* temps, uint64_t n, float a) {
    NvtxRange trace_("bay_anneal");
    return guarded([&] {
        if (!s || (n && !temps)) fail(BAY_ERR_ARG, "NULL argument");
        if (!(a > 1.0f)) fail(BAY_ERR_ARG, "the stretch parameter a must be > 1");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        s->require_positions();
        for (uint64_t i = 0; i < n; ++i) {
            s->set_a_beta(a, (float)(1.0 / (double)temps[i]));
            s->steps(false, 1);
        }
        s->iteration_counter += n;
    });
}

namespace {
// init-move! (nvidia_gtx.clj:340-350): accu seeds advance by 2, move counter and the
// acceptance count restart.  Counts start at 0 (the OpenCL engine's choice; the CUDA
// engine memsets them to 1 per block).
void init_move(bay_sampler* s, float a) {
    s->seed_accu += 2;
    s->step_accu = 0;
    s->a = a;
    bay_ctl_op op{};
    op.mask = BAY_CTL_SET_SEED1 | BAY_CTL_SET_STEP1 | BAY_CTL_SET_A | BAY_CTL_RESET_ACCEPTED |
              BAY_CTL_RESET_TICKETS;
    op.seed[1] = s->seed_accu;
    op.a = a;
    s->ctl_op(op);
}

uint64_t read_accepted(bay_sampler* s) {
    unsigned long long v = 0;
    cuda_check(cudaMemcpyAsync(&v, &s->ctl->accepted, sizeof(v), cudaMemcpyDeviceToHost,
                               s->ctx->stream),
               "cudaMemcpy(accepted)");
    cuda_check(cudaStreamSynchronize(s->ctx->stream), "sync");
    s->check_status();
    return v;
}

// Bin counts of dimension-major values (dm[d * W + w]) into counts[d * bins + b]: the
// IEEE-division kernel, or with BAY_HIST_COMPAT_FASTDIV the reference's expression under
// -use_fast_math (device/bay_hist_fastdiv.cuh; one NVRTC module per bin count and
// context, compiled on first use).
void hist_count(bay_ctx* c, uint32_t flags, const float* dm, uint32_t D, uint64_t W,
                uint32_t bins, const float* lim, uint32_t* counts) {
    if (D > 65535) fail(BAY_ERR_ARG, "histograms of at most 65535 dimensions");
    if (!(flags & BAY_HIST_COMPAT_FASTDIV)) {
        cuda_check(bay::launch_hist_count(dm, D, W, bins, lim, counts, c->stream), "histogram");
        return;
    }
    CUkernel k = nullptr;
    auto it = c->hist_fastdiv.find(bins);
    if (it != c->hist_fastdiv.end()) {
        k = it->second.second;
    } else {
        std::string src = "\n#line 1 \"bay_hist_fastdiv.cuh\"\n";
        src += bay_embedded_hist_fastdiv;
        const std::vector<std::string> opts = {"-arch=sm_103a", "-use_fast_math", "-default-device",
                                               "-std=c++17",
                                               "-DBAY_HIST_BINS=" + std::to_string(bins)};
        std::vector<char> cubin = nvrtc_compile(src, opts);
        CUlibrary lib = nullptr;
        cu_check(g_cu.LibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0),
                 "cuLibraryLoadData(histogram)");
        const CUresult r = g_cu.LibraryGetKernel(&k, lib, "bay_hist_count_fastdiv");
        if (r != CUDA_SUCCESS) {
            g_cu.LibraryUnload(lib);
            cu_check(r, "GetKernel(histogram)");
        }
        c->hist_fastdiv[bins] = std::make_pair(lib, k);
    }
    const float* xp = dm;
    unsigned int dd = D;
    unsigned long long ww = W;
    const float* lp = lim;
    unsigned int* cp = counts;
    void* args[] = {&xp, &dd, &ww, &lp, &cp};
    const unsigned gx = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(64, (W + 255) / 256));
    cu_check(g_cu.LaunchKernel((CUfunction)k, gx, D, 1, 256, 1, 1, 0, (CUstream)c->stream, args,
                               nullptr),
             "cuLaunchKernel(histogram, fast division)");
    bay::count_launches(1);
}

uint32_t acor_lag(uint64_t n, uint32_t wgs) {
    uint64_t l = n / 5;
    if (wgs < l) l = wgs;
    if (64 < l) l = 64;
    return (uint32_t)(l < 10 ? 10 : l);
}

// acor of a device-resident series; results to host or device arrays.
int acor_device(bay_ctx* c, const float* d_series, uint32_t D, uint64_t n, double* tau,
                double* mean, double* sigma, uint32_t* lag_out) {
    const uint32_t lag = acor_lag(n, c->wgs);
    if (lag_out) *lag_out = lag;
    if ((uint64_t)lag * 5 > n) {
        g_err = "The autocorrelation time is too long relative to the variance. Number of steps (" +
                std::to_string(n) + ") must not be less than " + std::to_string(lag * 5) + ".";
        return BAY_ERR_ARG;
    }
    if (n > 0xffffffffull) fail(BAY_ERR_ARG, "series too long");
    double* work = (double*)c->alloc(sizeof(double) * ((size_t)D * n + 3 * D));
    try {
        double* res = work + (size_t)D * n;
        cuda_check(bay::launch_acor(d_series, D, (uint32_t)n, c->wgs, lag, work, res, res + D,
                                    res + 2 * D, c->stream),
                   "acor");
        if (tau) cuda_check(cudaMemcpyAsync(tau, res, sizeof(double) * D, cudaMemcpyDefault, c->stream), "copy");
        if (mean) cuda_check(cudaMemcpyAsync(mean, res + D, sizeof(double) * D, cudaMemcpyDefault, c->stream), "copy");
        if (sigma) cuda_check(cudaMemcpyAsync(sigma, res + 2 * D, sizeof(double) * D, cudaMemcpyDefault, c->stream), "copy");
        cuda_check(cudaStreamSynchronize(c->stream), "sync");
    } catch (...) {
        c->release(work);
        throw;
    }
    c->release(work);
    return BAY_OK;
}
}  // namespace

int bay_acc_rate(bay_sampler* s, float a, double* rate) {
    NvtxRange trace_("bay_acc_rate");
    return guarded([&] {
        if (!s || !rate) fail(BAY_ERR_ARG, "NULL argument");
        if (!(a > 1.0f)) fail(BAY_ERR_ARG, "the stretch parameter a must be > 1");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        s->require_positions();
        init_move(s, a);
        const uint64_t cap = s->means_cap;
        s->means_cap = 0;  // no per-step means for a single acceptance probe
        try {
            s->steps(true, 1);
        } catch (...) {
            s->means_cap = cap;
            throw;
        }
        s->means_cap = cap;
        s->iteration_counter += 1;
        *rate = (double)read_accepted(s) / (double)s->W;
    });
}

int bay_adapt_a(bay_sampler* s, uint32_t step, double a, double min_acc, double max_acc,
                bay_adapt_result* out) {
    NvtxRange trace_("bay_adapt_a");
    return guarded([&] {
        if (!s || !out) fail(BAY_ERR_ARG, "NULL argument");
        if (!((float)a > 1.0f)) fail(BAY_ERR_ARG, "the stretch parameter a must be > 1");
        if (!(0.0 <= min_acc && min_acc < max_acc && max_acc <= 1.0))
            fail(BAY_ERR_ARG, "the acceptance window must satisfy 0 <= min < max <= 1");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        bay_ctx* c = s->ctx;
        c->use();
        s->require_positions();
        if (!s->mix) s->mix = (bay_mix_state*)c->alloc(sizeof(bay_mix_state));
        bay_mix_state h0{};
        h0.a = a;
        cuda_check(cudaMemcpyAsync(s->mix, &h0, sizeof(h0), cudaMemcpyHostToDevice, c->stream),
                   "cudaMemcpy(mix state)");
        // one graph: a WHILE node whose body is one probe (init-move!, the accu step's two
        // half-step launches, the loop's rule); mix_end sets the condition, so the loop runs
        // on the device with no host readback per probe
        const uint64_t cap = s->means_cap;
        s->means_cap = 0;  // acc-rate! probes record no per-step means
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ex = nullptr;
        auto cleanup = [&] {
            s->means_cap = cap;
            if (ex) cudaGraphExecDestroy(ex);
            if (g) cudaGraphDestroy(g);
        };
        try {
            cuda_check(cudaGraphCreate(&g, 0), "cudaGraphCreate");
            cudaGraphConditionalHandle cond;
            cuda_check(cudaGraphConditionalHandleCreate(&cond, g, 1u, cudaGraphCondAssignDefault),
                       "cudaGraphConditionalHandleCreate");
            cudaGraphNodeParams np{};
            np.type = cudaGraphNodeTypeConditional;
            np.conditional.handle = cond;
            np.conditional.type = cudaGraphCondTypeWhile;
            np.conditional.size = 1;
            cudaGraphNode_t node;
            cuda_check(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np), "cudaGraphAddNode(while)");
            cudaGraph_t body = np.conditional.phGraph_out[0];
            cudaStream_t cs = c->capture;
            cuda_check(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0,
                                                     cudaStreamCaptureModeThreadLocal),
                       "cudaStreamBeginCaptureToGraph");
            try {
                cuda_check(bay::launch_mix_begin(s->ctl, s->mix, cs), "mix_begin");
                s->launch_half(true, 0, 0, cs, false);
                s->launch_half(true, 1, 0, cs, false);
                cuda_check(bay::launch_mix_end(s->ctl, s->mix, s->W, step, min_acc, max_acc, cond, cs),
                           "mix_end");
            } catch (...) {
                cudaGraph_t tmp = nullptr;
                cudaStreamEndCapture(cs, &tmp);
                throw;
            }
            cuda_check(cudaStreamEndCapture(cs, &body), "cudaStreamEndCapture");
            cuda_check(cudaGraphInstantiate(&ex, g, 0), "cudaGraphInstantiate(adapt)");
            cuda_check(cudaGraphLaunch(ex, c->stream), "cudaGraphLaunch(adapt)");
            bay_mix_state h{};
            cuda_check(cudaMemcpyAsync(&h, s->mix, sizeof(h), cudaMemcpyDeviceToHost, c->stream),
                       "cudaMemcpy(mix state)");
            cuda_check(cudaStreamSynchronize(c->stream), "sync");
            s->check_status();
            // the host mirror of what the probes did: init-move! per probe, one accu step
            s->seed_accu += 2u * h.probes;
            s->step_accu = 1;
            s->a = (float)h.a;
            s->iteration_counter += h.probes;
            bay::count_launches((uint64_t)h.probes * (2u + (s->streaming ? 6u : 2u)));
            if (h.bad)
                fail(BAY_ERR_ARG, "the stretch parameter a must be > 1 (the adaptation took a "
                                  "to " + std::to_string(h.a) + ")");
            out->a = h.a;
            out->acc_rate = h.rate;
            out->probes = h.probes;
        } catch (...) {
            cleanup();
            throw;
        }
        cleanup();
    });
}

int bay_run_sampler(bay_sampler* s, uint64_t n, float a, bay_run_result* res, double* tau,
                    double* mean, double* sigma, float* means_out) {
    NvtxRange trace_("bay_run_sampler");
    return guarded([&] {
        if (!s || !res) fail(BAY_ERR_ARG, "NULL argument");
        if (!(a > 1.0f)) fail(BAY_ERR_ARG, "the stretch parameter a must be > 1");
        if (n == 0 || n > 0xffffffffull) fail(BAY_ERR_ARG, "steps must be in [1, 2^32)");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        s->require_positions();
        s->ensure_means(n);
        init_move(s, a);
        s->steps(true, n);
        s->iteration_counter += n;
        const uint64_t acc = read_accepted(s);
        res->acceptance_rate = (double)acc / ((double)s->W * (double)n);
        res->a = a;
        res->steps = n;
        if (means_out)
            cuda_check(cudaMemcpyAsync(means_out, s->means, sizeof(float) * (size_t)s->D * n,
                                       cudaMemcpyDefault, s->ctx->stream),
                       "cudaMemcpy(means)");
        uint32_t lag = 0;
        const std::string keep = g_err;
        res->acor_status = acor_device(s->ctx, s->means, s->D, n, tau, mean, sigma, &lag);
        if (res->acor_status == BAY_OK) g_err = keep;
        res->lag = lag;
        cuda_check(cudaStreamSynchronize(s->ctx->stream), "sync");
    });
}

int bay_sample(bay_sampler* s, uint64_t n_cols, float* out) {
    NvtxRange trace_("bay_sample");
    return guarded([&] {
        if (!s || (n_cols && !out)) fail(BAY_ERR_ARG, "NULL argument");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        s->require_positions();
        s->set_a_beta(s->a, 1.0f);
        uint64_t ofs = 0;
        while (ofs < n_cols) {
            s->steps(false, 1);
            s->iteration_counter += 1;
            const uint64_t take = std::min<uint64_t>(s->W, n_cols - ofs);
            // the walker state is the reference's dim x walkers column-major layout
            cuda_check(cudaMemcpyAsync(out + ofs * s->D, s->xs, sizeof(float) * take * s->D,
                                       cudaMemcpyDefault, s->ctx->stream),
                       "cudaMemcpy(sample)");
            ofs += take;
        }
        cuda_check(cudaStreamSynchronize(s->ctx->stream), "sync");
    });
}

static int moments_out(bay_sampler* s, double* out, int which) {
    NvtxRange trace_(which ? "bay_variance" : "bay_mean");
    return guarded([&] {
        if (!s || !out) fail(BAY_ERR_ARG, "NULL argument");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        s->require_positions();
        cuda_check(bay::launch_moments(s->dim_major(), s->D, s->W, s->stats, s->stats + s->D,
                                       s->ctx->stream),
                   "moments");
        cuda_check(cudaMemcpyAsync(out, s->stats + (which ? s->D : 0), sizeof(double) * s->D,
                                   cudaMemcpyDefault, s->ctx->stream),
                   "cudaMemcpy(moments)");
        cuda_check(cudaStreamSynchronize(s->ctx->stream), "sync");
        s->check_status();
        if (which == 2 && !is_device_ptr(out, s->ctx->device))
            for (uint32_t d = 0; d < s->D; ++d) out[d] = std::sqrt(out[d]);
    });
}

int bay_mean(bay_sampler* s, double* out) { return moments_out(s, out, 0); }
int bay_variance(bay_sampler* s, double* out) { return moments_out(s, out, 1); }
int bay_sd(bay_sampler* s, double* out) {
    bool dev = false;
    const int g = guarded([&] {
        if (s && out) dev = is_device_ptr(out, s->ctx->device);
    });
    if (g != BAY_OK) return g;
    if (dev) {
        g_err = "bay_sd writes host memory only";
        return BAY_ERR_ARG;
    }
    return moments_out(s, out, 2);
}

int bay_histogram(bay_sampler* s, uint32_t cycles, uint32_t bins, uint32_t flags, float* limits,
                  float* pdf, float* ranks) {
    NvtxRange trace_("bay_histogram");
    return guarded([&] {
        if (!s || !limits || !pdf || !ranks) fail(BAY_ERR_ARG, "NULL argument");
        if (cycles == 0) fail(BAY_ERR_ARG, "cycles must be >= 1");
        if (bins == 0) bins = s->ctx->wgs;
        if (bins < 2 || bins > 1024 || (bins & (bins - 1)))
            fail(BAY_ERR_ARG, "bins must be a power of two in [2, 1024]");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        bay_ctx* c = s->ctx;
        c->use();
        s->require_positions();
        if (s->hist_bins < bins) {
            c->release(s->hist);
            c->release(s->counts);
            s->hist = nullptr;
            s->counts = nullptr;
            s->hist = (float*)c->alloc(sizeof(float) * (2 * (size_t)s->D + 2 * (size_t)bins * s->D));
            s->counts = (uint32_t*)c->alloc(sizeof(uint32_t) * (size_t)bins * s->D);
            s->hist_bins = bins;
        }
        float* d_lim = s->hist;
        float* d_pdf = d_lim + 2 * s->D;
        float* d_rank = d_pdf + (size_t)bins * s->D;
        // Q7: the reference's min/max reduction folds 0.0 in when a level has a partial
        // block; wgsn = WGS / min(dim, sqrt(WGS)) (nvidia_gtx.clj:486-488).
        int zero = 0;
        if (flags & BAY_HIST_COMPAT_ZERO_LIMITS) {
            uint64_t sq = (uint64_t)std::sqrt((double)c->wgs);
            uint64_t wgsm = std::min<uint64_t>(s->D, sq);
            if (!wgsm) wgsm = 1;
            const uint64_t wgsn = c->wgs / wgsm;
            uint64_t cnt = s->W;
            do {
                const uint64_t B = std::min(cnt, wgsn);
                if (cnt % B) zero = 1;
                cnt = (cnt + B - 1) / B;
            } while (cnt > 1);
        }
        const float* dm = s->dim_major();
        cuda_check(bay::launch_minmax(dm, s->D, s->W, zero, d_lim, c->stream), "minmax");
        cuda_check(bay::launch_fill_u32(s->counts, (flags & BAY_HIST_COMPAT_START1) ? 1u : 0u,
                                        (uint64_t)bins * s->D, c->stream),
                   "fill");
        hist_count(c, flags, dm, s->D, s->W, bins, d_lim, s->counts);
        if (cycles > 1) {
            s->set_a_beta(s->a, 1.0f);
            for (uint32_t i = 1; i < cycles; ++i) {
                s->steps(false, 1);
                hist_count(c, flags, s->dim_major(), s->D, s->W, bins, d_lim, s->counts);
            }
            s->iteration_counter += cycles - 1;
        }
        cuda_check(bay::launch_hist_finish(s->counts, d_lim, s->D, bins, (uint64_t)cycles * s->W,
                                           d_pdf, d_rank, c->stream),
                   "hist_finish");
        cuda_check(cudaMemcpyAsync(limits, d_lim, sizeof(float) * 2 * s->D, cudaMemcpyDefault, c->stream), "copy");
        cuda_check(cudaMemcpyAsync(pdf, d_pdf, sizeof(float) * bins * s->D, cudaMemcpyDefault, c->stream), "copy");
        cuda_check(cudaMemcpyAsync(ranks, d_rank, sizeof(float) * bins * s->D, cudaMemcpyDefault, c->stream), "copy");
        cuda_check(cudaStreamSynchronize(c->stream), "sync");
    });
}

int bay_acor(bay_ctx* c, const float* series, uint32_t D, uint64_t n, double* tau, double* mean,
             double* sigma, uint32_t* lag) {
    NvtxRange trace_("bay_acor");
    int rc = BAY_OK;
    const int g = guarded([&] {
        if (!c || !series) fail(BAY_ERR_ARG, "NULL argument");
        if (D == 0) fail(BAY_ERR_ARG, "dim must be >= 1");
        std::lock_guard<std::recursive_mutex> lk(c->mu);
        c->use();
        if (is_device_ptr(series, c->device)) {
            rc = acor_device(c, series, D, n, tau, mean, sigma, lag);
            return;
        }
        float* d = (float*)c->alloc(sizeof(float) * (size_t)D * std::max<uint64_t>(n, 1));
        try {
            cuda_check(cudaMemcpyAsync(d, series, sizeof(float) * (size_t)D * n,
                                       cudaMemcpyHostToDevice, c->stream),
                       "cudaMemcpy(series)");
            rc = acor_device(c, d, D, n, tau, mean, sigma, lag);
        } catch (...) {
            c->release(d);
            throw;
        }
        c->release(d);
    });
    return g != BAY_OK ? g : rc;
}

// Allocation-free acor for callers that cannot allocate device memory at call time:
// the work space is the library's fixed device scratch (BAY_ACOR_NOALLOC_MAX_DOUBLES).
int bay_acor_noalloc(bay_ctx* c, const float* d_series, uint32_t D, uint64_t n, double* tau,
                     double* mean, double* sigma, uint32_t* lag_out) {
    NvtxRange trace_("bay_acor_noalloc");
    return guarded([&] {
        if (!c || !d_series) fail(BAY_ERR_ARG, "NULL argument");
        if (D == 0) fail(BAY_ERR_ARG, "dim must be >= 1");
        if (!is_device_ptr(d_series, c->device))
            fail(BAY_ERR_ARG, "bay_acor_noalloc needs the series in device memory");
        const uint64_t need = (uint64_t)D * n + 3ull * D;
        if (n > 0xffffffffull || need > BAY_ACOR_NOALLOC_MAX_DOUBLES)
            fail(BAY_ERR_ARG, "series too large for the fixed acor scratch: dim * n + 3 * dim = " +
                                  std::to_string(need) + " doubles > " +
                                  std::to_string(BAY_ACOR_NOALLOC_MAX_DOUBLES));
        const uint32_t lag = acor_lag(n, c->wgs);
        if (lag_out) *lag_out = lag;
        if ((uint64_t)lag * 5 > n)
            fail(BAY_ERR_ARG, "The autocorrelation time is too long relative to the variance. "
                              "Number of steps (" + std::to_string(n) +
                                  ") must not be less than " + std::to_string(lag * 5) + ".");
        std::lock_guard<std::recursive_mutex> lk(c->mu);
        c->use();
        double* work = c->acor_scratch;
        double* res = work + (size_t)D * n;
        cuda_check(bay::launch_acor(d_series, D, (uint32_t)n, c->wgs, lag, work, res, res + D,
                                    res + 2 * D, c->stream),
                   "acor");
        if (tau) cuda_check(cudaMemcpyAsync(tau, res, sizeof(double) * D, cudaMemcpyDefault, c->stream), "copy");
        if (mean) cuda_check(cudaMemcpyAsync(mean, res + D, sizeof(double) * D, cudaMemcpyDefault, c->stream), "copy");
        if (sigma) cuda_check(cudaMemcpyAsync(sigma, res + 2 * D, sizeof(double) * D, cudaMemcpyDefault, c->stream), "copy");
        cuda_check(cudaStreamSynchronize(c->stream), "sync");
    });
}

int bay_state_export(bay_sampler* s, float* positions, float* logfn, uint32_t* rng) {
    NvtxRange trace_("bay_state_export");
    return guarded([&] {
        if (!s) fail(BAY_ERR_ARG, "NULL sampler");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        s->require_positions();
        if (positions)
            cuda_check(cudaMemcpyAsync(positions, s->xs, sizeof(float) * (size_t)s->D * s->W,
                                       cudaMemcpyDefault, s->ctx->stream),
                       "copy");
        if (logfn)
            cuda_check(cudaMemcpyAsync(logfn, s->logfn, sizeof(float) * s->W, cudaMemcpyDefault,
                                       s->ctx->stream),
                       "copy");
        if (rng) {
            rng[0] = s->seed_bare;
            rng[1] = s->seed_accu;
            rng[2] = s->step_bare;
            rng[3] = s->step_accu;
            rng[4] = (uint32_t)s->iteration_counter;
            rng[5] = (uint32_t)(s->iteration_counter >> 32);
            std::memcpy(&rng[6], &s->a, 4);
            std::memcpy(&rng[7], &s->beta, 4);
        }
        cuda_check(cudaStreamSynchronize(s->ctx->stream), "sync");
    });
}

int bay_state_import(bay_sampler* s, const float* positions, const float* logfn,
                     const uint32_t* rng) {
    NvtxRange trace_("bay_state_import");
    return guarded([&] {
        if (!s || !positions || !logfn || !rng) fail(BAY_ERR_ARG, "NULL argument");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        cuda_check(cudaMemcpyAsync(s->xs, positions, sizeof(float) * (size_t)s->D * s->W,
                                   cudaMemcpyDefault, s->ctx->stream),
                   "copy");
        cuda_check(cudaMemcpyAsync(s->logfn, logfn, sizeof(float) * s->W, cudaMemcpyDefault,
                                   s->ctx->stream),
                   "copy");
        s->seed_bare = rng[0];
        s->seed_accu = rng[1];
        s->step_bare = rng[2];
        s->step_accu = rng[3];
        s->iteration_counter = (uint64_t)rng[4] | ((uint64_t)rng[5] << 32);
        std::memcpy(&s->a, &rng[6], 4);
        std::memcpy(&s->beta, &rng[7], 4);
        bay_ctl_op op{};
        op.mask = BAY_CTL_SET_SEED0 | BAY_CTL_SET_SEED1 | BAY_CTL_SET_STEP0 | BAY_CTL_SET_STEP1 |
                  BAY_CTL_SET_A | BAY_CTL_SET_BETA | BAY_CTL_RESET_TICKETS;
        op.seed[0] = s->seed_bare;
        op.seed[1] = s->seed_accu;
        op.step[0] = s->step_bare;
        op.step[1] = s->step_accu;
        op.a = s->a;
        op.beta = s->beta;
        s->ctl_op(op);
        cuda_check(cudaStreamSynchronize(s->ctx->stream), "sync");
        s->positioned = true;
    });
}

int bay_logfn_values(bay_sampler* s, float* out) {
    return guarded([&] {
        if (!s || !out) fail(BAY_ERR_ARG, "NULL argument");
        std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
        s->ctx->use();
        cuda_check(cudaMemcpyAsync(out, s->logfn, sizeof(float) * s->W, cudaMemcpyDefault,
                                   s->ctx->stream),
                   "copy");
        cuda_check(cudaStreamSynchronize(s->ctx->stream), "sync");
    });
}

}  // extern "C"

#include "bay_batch_api.inc"
#include "bay_engines_api.inc"
#include "bay_tune_api.inc"
