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
// in one file-scope __device__ array of kNoAllocScratchBytes.  Every GPU that
// loads the library reserves that array until the process exits.  The device
// address of the array is looked up with cudaGetSymbolAddress once per
// device, on the first call on that device, with that device current; make
// that first call before any stream capture.  All calls share the array and
// it keeps the last call's contents; nothing in it needs to start at zero
// (the kernel writes every scratch element before reading it).  Calls whose
// kernels overlap on the GPU (two streams, two threads) race on the array.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <mutex>
#include <string>

#include "../../include/gbdpcg.h"
#include "pcg_types.h"
#include "pcg_variants.h"

namespace gbdpcg {
void set_last_error(const std::string &msg);
}

namespace {

constexpr size_t kNoAllocMaxVec = GBDPCG_NOALLOC_MAX_ELEMS;    // n*N
constexpr size_t kNoAllocMaxKnots = GBDPCG_NOALLOC_MAX_KNOTS;  // N
constexpr size_t kNoAllocScratchBytes =
    2 * kNoAllocMaxVec * sizeof(float) + 2 * kNoAllocMaxKnots * sizeof(float) + 256;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_ptr[kMaxDevices] = {};
int g_sm_count[kMaxDevices] = {};
int g_smem_optin[kMaxDevices] = {};

int noalloc_fail(int code, const std::string &msg) {
    gbdpcg::set_last_error(msg);  // read back with gbdpcg_last_error()
    return code;
}

// Device address of the scratch array and device limits, looked up once per
// device with that device current.
int scratch_for_current_device(void **ptr, int *sm_count, int *smem_optin) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(GBDPCG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(GBDPCG_ERR_UNSUPPORTED, "device index too large");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return noalloc_fail(GBDPCG_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        int sms = 0, optin = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess)
            return noalloc_fail(GBDPCG_ERR_CUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
        g_sm_count[dev] = sms;
        g_smem_optin[dev] = optin;
        g_scratch_ptr[dev] = p;
    }
    *ptr = g_scratch_ptr[dev];
    *sm_count = g_sm_count[dev];
    *smem_optin = g_smem_optin[dev];
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
    if (cfg->exit_mode > GBDPCG_EXIT_RELRES || !(cfg->exit_tol >= 0))
        return noalloc_fail(GBDPCG_ERR_INVALID_ARGUMENT, "bad config field");
    void *scratch = nullptr;
    int sm_count = 0, smem_optin = 0;
    int rc = scratch_for_current_device(&scratch, &sm_count, &smem_optin);
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
