// Test infrastructure only.  Host-side launcher for the reference kernel
// pcg<T, n, N> rebuilt into oracle/_ref/ref_pcg_{f32,f64}.cubin by
// oracle/build_oracle.py.  It does what the reference's device-pointer
// solvePCG (include/interface.cuh:94-146) does — cooperative launch of N
// blocks of 64 threads (interface.cuh:134), 12 kernel arguments
// (include/pcg.cuh:56-68) — with two differences, both needed to run the
// reference safely and to time it:
//   * dynamic shared memory is the larger of the reference's own size
//     (pcgSharedMemSize, include/pcg.cuh:13-20) and the size its carve-up
//     actually uses (include/pcg.cuh:83-95: 6n^2 + 12n + 2 max(n, N)
//     elements), because the former is 2n elements short for some sizes;
//   * the kernel is launched `reps` times from the same inputs (lambda is
//     reset before each) and the device time of each launch is measured with
//     CUDA events; outputs of the last launch are returned.
// The kernel is looked up by its Itanium-mangled name, which the caller
// passes (oracle/oracle.py computes it).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <map>
#include <mutex>
#include <string>

namespace {
std::mutex g_mu;
std::map<std::string, cudaLibrary_t> g_libs;

cudaLibrary_t load_lib(const char *path) {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_libs.find(path);
    if (it != g_libs.end()) return it->second;
    cudaLibrary_t lib = nullptr;
    if (cudaLibraryLoadFromFile(&lib, path, nullptr, nullptr, 0, nullptr, nullptr, 0) !=
        cudaSuccess)
        return nullptr;
    g_libs[path] = lib;
    return lib;
}
}  // namespace

#define REF_CHECK(x)                                                                 \
    do {                                                                             \
        cudaError_t e_ = (x);                                                        \
        if (e_ != cudaSuccess) {                                                     \
            snprintf(err, errlen, "%s: %s", #x, cudaGetErrorString(e_));             \
            rc = -1;                                                                 \
            goto done;                                                               \
        }                                                                            \
    } while (0)

extern "C" int refpcg_solve(const char *cubin_path, const char *kernel_name, int is_f64,
                            uint32_t n, uint32_t N, const void *h_S, const void *h_Pinv,
                            const void *h_gamma, void *h_lambda, uint32_t max_iter,
                            double tol, int reps, uint32_t *iters_out, int *max_iter_exit_out,
                            float *ms_out, char *err, int errlen) {
    int rc = 0;
    const size_t s = is_f64 ? sizeof(double) : sizeof(float);
    const size_t mat = (size_t)3 * n * n * N * s, vec = (size_t)n * N * s;
    const size_t mx = n > N ? n : N;
    size_t smem_ref = (size_t)6 * n * n + 10 * n + 2 * mx;
    if ((size_t)9 * n * n > smem_ref) smem_ref = (size_t)9 * n * n;
    size_t smem_use = (size_t)6 * n * n + 12 * n + 2 * mx;
    const size_t smem = (smem_ref > smem_use ? smem_ref : smem_use) * s;
    char *d_S = nullptr, *d_P = nullptr, *d_g = nullptr, *d_l = nullptr, *d_r = nullptr,
         *d_p = nullptr, *d_v = nullptr, *d_e = nullptr;
    uint32_t *d_iters = nullptr;
    bool *d_exit = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaKernel_t kern = nullptr;
    float tol_f = (float)tol;
    double tol_d = tol;
    bool h_exit = true;
    cudaLibrary_t lib = load_lib(cubin_path);
    if (!lib) {
        snprintf(err, errlen, "cannot load %s", cubin_path);
        return -2;
    }
    REF_CHECK(cudaLibraryGetKernel(&kern, lib, kernel_name));
    if (smem > 48 * 1024)
        REF_CHECK(cudaKernelSetAttributeForDevice(
            kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem, 0));
    REF_CHECK(cudaMalloc(&d_S, mat));
    REF_CHECK(cudaMalloc(&d_P, mat));
    REF_CHECK(cudaMalloc(&d_g, vec));
    REF_CHECK(cudaMalloc(&d_l, vec));
    REF_CHECK(cudaMalloc(&d_r, vec));
    REF_CHECK(cudaMalloc(&d_p, vec));
    REF_CHECK(cudaMalloc(&d_v, N * s));
    REF_CHECK(cudaMalloc(&d_e, N * s));
    REF_CHECK(cudaMalloc(&d_iters, sizeof(uint32_t)));
    REF_CHECK(cudaMalloc(&d_exit, sizeof(bool)));
    REF_CHECK(cudaMemcpy(d_S, h_S, mat, cudaMemcpyHostToDevice));
    REF_CHECK(cudaMemcpy(d_P, h_Pinv, mat, cudaMemcpyHostToDevice));
    REF_CHECK(cudaMemcpy(d_g, h_gamma, vec, cudaMemcpyHostToDevice));
    REF_CHECK(cudaEventCreate(&e0));
    REF_CHECK(cudaEventCreate(&e1));
    if (reps < 1) reps = 1;
    for (int rep = 0; rep < reps; ++rep) {
        REF_CHECK(cudaMemcpy(d_l, h_lambda, vec, cudaMemcpyHostToDevice));
        void *args[12] = {&d_S, &d_P, &d_g, &d_l, &d_r, &d_p, &d_v, &d_e, &d_iters, &d_exit,
                          &max_iter, is_f64 ? (void *)&tol_d : (void *)&tol_f};
        cudaLaunchConfig_t cfg;
        memset(&cfg, 0, sizeof(cfg));
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.gridDim = dim3(N);
        cfg.blockDim = dim3(64);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = 0;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        REF_CHECK(cudaEventRecord(e0, 0));
        REF_CHECK(cudaLaunchKernelExC(&cfg, (const void *)kern, args));
        REF_CHECK(cudaEventRecord(e1, 0));
        REF_CHECK(cudaEventSynchronize(e1));
        if (ms_out) REF_CHECK(cudaEventElapsedTime(&ms_out[rep], e0, e1));
    }
    REF_CHECK(cudaMemcpy(h_lambda, d_l, vec, cudaMemcpyDeviceToHost));
    REF_CHECK(cudaMemcpy(iters_out, d_iters, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    REF_CHECK(cudaMemcpy(&h_exit, d_exit, sizeof(bool), cudaMemcpyDeviceToHost));
    *max_iter_exit_out = h_exit ? 1 : 0;
done:
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d_S); cudaFree(d_P); cudaFree(d_g); cudaFree(d_l); cudaFree(d_r);
    cudaFree(d_p); cudaFree(d_v); cudaFree(d_e); cudaFree(d_iters); cudaFree(d_exit);
    return rc;
}
