// Allocation-free solve entry point (gbdpcg_solve_plain_noalloc_f32).
//
// Who needs it: callers that must not allocate device memory once they are
// running — a model-predictive controller solving at a fixed rate, where a
// cudaMalloc in the control loop adds latency with no upper bound; a process
// whose device memory is already handed out by another allocator, so that a
// cudaMalloc from this library would fail or fragment that pool; deployments
// whose rules forbid dynamic allocation after start-up.  The other entry
// points allocate a small per-handle workspace, and the plain algorithm grows
// a scratch buffer for its r / p vectors and dot partials.
//
// This entry point runs the same plain kernel (one CTA per knot, the
// reference's arithmetic order) with its scratch — r and p (n*N floats each),
// the two dot-partial arrays (N floats each) and the result record — placed
// in one file-scope __device__ array of kNoAllocScratchBytes.  The array lives
// in the library's device code, which CUDA loads into a device's context when
// the library's kernels are first needed there (lazily, by default), so the
// first call on each device is what loads the module and reserves the array.
// That first call can therefore still fail for want of device memory: make it
// at start-up, as a warm-up, before other allocators take the memory and
// before any stream capture.  From then on the device holds the array until
// the process exits.  Every call looks up the array's device address with
// cudaGetSymbolAddress, with the calling device current (a host-side lookup
// that allocates nothing), so a context reset that reloads the module is
// picked up.  All calls share the array and it keeps the last call's
// contents; nothing in it needs to start at zero (the kernel writes every
// scratch element before reading it).  Calls whose kernels overlap on the GPU
// (two streams, two threads) race on the array.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <string>

#include "../../include/gbdpcg.h"
#include "pcg_types.h"
#include "pcg_variants.h"

namespace gbdpcg {
void set_last_error(const std::string &msg);
int check_config(const gbdpcg_config *cfg, uint32_t layout);
}

namespace {

constexpr size_t kNoAllocMaxVec = GBDPCG_NOALLOC_MAX_ELEMS;    // n*N
constexpr size_t kNoAllocMaxKnots = GBDPCG_NOALLOC_MAX_KNOTS;  // N
constexpr size_t kNoAllocScratchBytes =
    2 * kNoAllocMaxVec * sizeof(float) + 2 * kNoAllocMaxKnots * sizeof(float) + 256;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

int noalloc_fail(int code, const std::string &msg) {
    gbdpcg::set_last_error(msg);  // read back with gbdpcg_last_error()
    return code;
}

// Device address of the scratch array on the current device, and that
// device's limits.  Looked up on every call: nothing is cached across calls.
int scratch_for_current_device(void **ptr, int *sm_count, int *smem_optin) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(GBDPCG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
        return noalloc_fail(GBDPCG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    int sms = 0, optin = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess)
        return noalloc_fail(GBDPCG_ERR_CUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
    *ptr = p;
    *sm_count = sms;
    *smem_optin = optin;
    return GBDPCG_SUCCESS;
}

}  // namespace

extern "C" {

int gbdpcg_solve_plain_noalloc_f32(const float *d_S, const float *d_Pinv, const float *d_gamma,
                                   float *d_lambda, uint32_t n, uint32_t N,
                                   const gbdpcg_config *cfg, gbdpcg_result *result,
                                   gbdpcg_stream_t stream_) {
    if (!d_S || !d_Pinv || !d_gamma || !d_lambda || !cfg)
        return noalloc_fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (n == 0 || N == 0) return noalloc_fail(GBDPCG_ERR_INVALID_ARGUMENT, "n and N must be positive");
    if ((size_t)n * N > kNoAllocMaxVec || N > kNoAllocMaxKnots)
        return noalloc_fail(GBDPCG_ERR_UNSUPPORTED,
                            "n*N = " + std::to_string((size_t)n * N) + ", N = " + std::to_string(N) +
                                " exceed the allocation-free limits n*N <= " +
                                std::to_string(kNoAllocMaxVec) + ", N <= " +
                                std::to_string(kNoAllocMaxKnots));
    // the checks of the handle entry points (cbtd Phi^-1, as the plain algorithm reads it)
    int rc = gbdpcg::check_config(cfg, GBDPCG_PINV_CBTD);
    if (rc) return rc;
    void *scratch = nullptr;
    int sm_count = 0, smem_optin = 0;
    rc = scratch_for_current_device(&scratch, &sm_count, &smem_optin);
    if (rc) return rc;
    cudaStream_t stream = (cudaStream_t)stream_;
    char *base = static_cast<char *>(scratch);
    float *d_r = reinterpret_cast<float *>(base);
    float *d_p = d_r + kNoAllocMaxVec;
    float *d_part1 = d_p + kNoAllocMaxVec;
    float *d_part2 = d_part1 + kNoAllocMaxKnots;
    gbdpcg::SysResult *d_res =
        reinterpret_cast<gbdpcg::SysResult *>(base + kNoAllocScratchBytes - 256);
    const void *func = gbdpcg::plain_kernel_ptr(false);
    const size_t smem = gbdpcg::plain_smem_bytes(false, n, N);
    if (smem > (size_t)smem_optin)
        return noalloc_fail(GBDPCG_ERR_UNSUPPORTED, "block row exceeds shared memory");
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024) e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, 64, smem);
    if (e != cudaSuccess) return noalloc_fail(GBDPCG_ERR_CUDA, std::string("launch set-up: ") + cudaGetErrorString(e));
    if ((int64_t)per_sm * sm_count < (int64_t)N)
        return noalloc_fail(GBDPCG_ERR_UNSUPPORTED, "knots exceed co-resident CTAs");
    uint32_t mi = cfg->max_iter;
    uint32_t fl = (cfg->exit_mode == GBDPCG_EXIT_RELRES ? gbdpcg::SYS_EXIT_RELRES : 0u) |
                  (cfg->zero_guess ? gbdpcg::SYS_LAMBDA0_ZERO : 0u);
    double tol = cfg->exit_tol;
    const void *S = d_S, *P = d_Pinv, *g = d_gamma, *l0 = d_lambda;
    void *l = d_lambda;
    void *args[] = {&S, &P, &g, &l0, &l, &d_r, &d_p, &d_part1, &d_part2, &n, &N, &mi, &tol, &fl, &d_res};
    e = cudaLaunchCooperativeKernel(func, dim3(N), dim3(64), args, smem, stream);
    if (e != cudaSuccess) return noalloc_fail(GBDPCG_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    if (result) {
        gbdpcg::SysResult r;
        e = cudaMemcpyAsync(&r, d_res, sizeof(r), cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) return noalloc_fail(GBDPCG_ERR_CUDA, std::string("result: ") + cudaGetErrorString(e));
        result->iters = r.iters;
        result->status = r.status;
        result->eta = r.eta;
        result->relres = (r.rr >= 0 && r.gg > 0) ? sqrt(r.rr / r.gg) : (r.rr >= 0 ? 0.0 : -1.0);
        result->outer = 0;
        result->reserved = 0;
    }
    return GBDPCG_SUCCESS;
}

}  // extern "C"
