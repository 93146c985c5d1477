// C++ drop-in for the reference's PCG interface (Sdevaud/GBD-PCG
// include/gpu_pcg.cuh -> interface.cuh, types.cuh, constants.cuh,
// gpuassert.cuh), implemented over the C ABI of gbdpcg.h.
//
// Same names, argument meaning and defaults:
//   pcg_config<T>      include/types.cuh:18-34 (tol 1e-6, 25 iterations,
//                      grid 128, block 64, empty_pinv 1)
//   pcg_constants::*   include/constants.cuh:14-20
//   solvePCG<T>(h_S, h_Pinv, h_gamma, h_lambda, stateSize, knotPoints, config)
//                      include/interface.cuh:24-91
//   solvePCG<T>(state_size, knot_points, d_S, d_Pinv, d_gamma, d_lambda,
//               d_r, d_p, d_v_temp, d_eta_new_temp, config)
//                      include/interface.cuh:94-146
//   pcg_solve<T>(h_S, h_gamma, h_lambda, stateSize, knotPoints, config)
//                      README.md:42 (documented there, not implemented in the
//                      reference; here Phi^-1 = blockdiag(S_kk^-1) is built on
//                      the GPU)
//   csr_t<T>           include/types.cuh:7-15 (and the CSR overload of solvePCG,
//                      include/interface.cuh:8-20, implemented here)
//   gpuErrchk / gpuAssert  include/gpuassert.cuh:5-14
// Differences a caller can observe, all deliberate:
//   * sizes are runtime arguments only; the STATE_SIZE / KNOT_POINTS macros
//     the reference needs at compile time (README.md:58-64) are not used;
//   * the host solvePCG returns the iteration count (the reference returns 1,
//     include/interface.cuh:90) and does not write h_S or h_gamma back
//     (interface.cuh:77,79);
//   * pcg_grid and pcg_block are accepted and ignored, as in the reference
//     (interface.cuh:134 launches N blocks of DEFAULT_BLOCK);
//   * d_r, d_p, d_v_temp, d_eta_new_temp of the device overload are not
//     needed (the cluster solver keeps them on chip) and may be null;
//   * a zero right-hand side returns lambda unchanged after one pass (the
//     reference divides 0 by 0).
// Define GBDPCG_DROPIN_ALGORITHM=GBDPCG_ALGO_PLAIN for the reference's exact
// arithmetic order (one CTA per knot) instead of the cluster solver.
// Errors print "GPUassert: <message>" and exit with the status code, as
// gpuErrchk does (include/gpuassert.cuh:10); define GBDPCG_THROW_ON_ERROR to
// throw std::runtime_error instead.
// A solve that stops without meeting its exit test (pcg_max_iter passes, or a
// non-finite p.Sp / r.z) returns its iteration count, as the reference does
// (include/pcg.cuh:212 records d_max_iter_exit and nothing reads it); define
// GBDPCG_ERROR_ON_MAX_ITER to treat it as the error GBDPCG_ERR_NOT_CONVERGED
// instead (printed and exited, or thrown, like any other error).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <type_traits>
#ifdef GBDPCG_THROW_ON_ERROR
#include <stdexcept>
#include <string>
#endif

#include "gbdpcg.h"

namespace pcg_constants {
inline uint32_t DEFAULT_MAX_PCG_ITER = 25;
template <typename T>
inline T DEFAULT_EPSILON = T(1e-6);
inline dim3 DEFAULT_GRID(128);
inline dim3 DEFAULT_BLOCK(64);
}  // namespace pcg_constants

template <typename T>
struct csr_t {
    uint32_t *row_ptr;
    uint32_t *col_ind;
    T *val;
    uint32_t rows;
    uint32_t cols;
    uint32_t nnz;
};

template <typename T>
struct pcg_config {
    T pcg_exit_tol;
    uint32_t pcg_max_iter;
    dim3 pcg_grid;
    dim3 pcg_block;
    int empty_pinv;

    pcg_config(T exit_tol = pcg_constants::DEFAULT_EPSILON<T>,
               uint32_t max_iter = pcg_constants::DEFAULT_MAX_PCG_ITER,
               dim3 grid = pcg_constants::DEFAULT_GRID, dim3 block = pcg_constants::DEFAULT_BLOCK,
               int empty_pinv = 1)
        : pcg_exit_tol(exit_tol), pcg_max_iter(max_iter), pcg_grid(grid), pcg_block(block),
          empty_pinv(empty_pinv) {}
};

inline void gpuAssert(int code, const char *file, int line, bool abort = true) {
    if (code != GBDPCG_SUCCESS) {
        // the library records a message for its own failures; a solve that did
        // not converge is reported by this header, not by a failed call
        const char *detail = code == GBDPCG_ERR_NOT_CONVERGED
                                 ? "the solve stopped without meeting its exit test"
                                 : gbdpcg_last_error();
#ifdef GBDPCG_THROW_ON_ERROR
        (void)abort;
        throw std::runtime_error(std::string("GPUassert: ") + gbdpcg_status_string(code) + ": " +
                                 detail + " " + file + " " + std::to_string(line));
#else
        fprintf(stderr, "GPUassert: %s: %s %s %d\n", gbdpcg_status_string(code), detail, file, line);
        if (abort) exit(code);
#endif
    }
}
#define gpuErrchk(ans) \
    { gpuAssert((ans), __FILE__, __LINE__); }

// Algorithm behind the drop-in calls.  AUTO runs the cluster solver (n <= 32);
// GBDPCG_ALGO_PLAIN reproduces the reference kernel's arithmetic bit for bit.
#ifndef GBDPCG_DROPIN_ALGORITHM
#define GBDPCG_DROPIN_ALGORITHM GBDPCG_ALGO_AUTO
#endif

namespace gbdpcg_detail {
template <typename T>
inline gbdpcg_config to_config(const pcg_config<T> *c) {
    gbdpcg_config g;
    gbdpcg_config_init(&g);
    g.algorithm = GBDPCG_DROPIN_ALGORITHM;
    if (c) {
        g.exit_tol = (double)c->pcg_exit_tol;
        g.max_iter = c->pcg_max_iter;
    }
    return g;
}

// GBDPCG_ERR_NOT_CONVERGED for a solve that ended without meeting its exit
// test, when the caller asked for that (GBDPCG_ERROR_ON_MAX_ITER).
inline int convergence_status(const gbdpcg_result &res) {
#ifdef GBDPCG_ERROR_ON_MAX_ITER
    return res.status == GBDPCG_CONVERGED ? GBDPCG_SUCCESS : GBDPCG_ERR_NOT_CONVERGED;
#else
    (void)res;
    return GBDPCG_SUCCESS;
#endif
}

inline gbdpcg_handle_t thread_handle() {
    static thread_local gbdpcg_handle_t h = nullptr;
    static thread_local int dev = -1;
    int cur = 0;
    cudaGetDevice(&cur);
    if (!h || dev != cur) {
        gpuErrchk(gbdpcg_create(&h, cur));
        dev = cur;
    }
    return h;
}
}  // namespace gbdpcg_detail

// Host pointers.  h_Pinv is a cbtd Phi^-1, or nullptr for the block-Jacobi
// preconditioner built on the GPU.  Returns the PCG iteration count.
template <typename T>
uint32_t solvePCG(T *h_S, T *h_Pinv, T *h_gamma, T *h_lambda, unsigned stateSize,
                  unsigned knotPoints, struct pcg_config<T> *config) {
    static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value,
                  "float or double");
    const gbdpcg_config cfg = gbdpcg_detail::to_config(config);
    gbdpcg_result res;
    int rc;
    if constexpr (std::is_same<T, float>::value)
        rc = gbdpcg_solve_f32(h_S, h_Pinv, h_gamma, h_lambda, stateSize, knotPoints, &cfg, &res);
    else
        rc = gbdpcg_solve_f64(h_S, h_Pinv, h_gamma, h_lambda, stateSize, knotPoints, &cfg, &res);
    gpuErrchk(rc);
    gpuErrchk(gbdpcg_detail::convergence_status(res));
    return res.iters;
}

// Device pointers (cbtd S and Phi^-1).  The scratch arguments of the
// reference are accepted and unused.  Synchronous, like the reference's
// read-back of the iteration count (interface.cuh:138).
template <typename T>
uint32_t solvePCG(const uint32_t state_size, const uint32_t knot_points, T *d_S, T *d_Pinv,
                  T *d_gamma, T *d_lambda, T *d_r, T *d_p, T *d_v_temp, T *d_eta_new_temp,
                  struct pcg_config<T> *config) {
    (void)d_r; (void)d_p; (void)d_v_temp; (void)d_eta_new_temp;
    const gbdpcg_config cfg = gbdpcg_detail::to_config(config);
    gbdpcg_result res;
    gbdpcg_handle_t h = gbdpcg_detail::thread_handle();
    int rc;
    if constexpr (std::is_same<T, float>::value)
        rc = gbdpcg_solve_dev_f32(h, d_S, d_Pinv, GBDPCG_PINV_CBTD, d_gamma, d_lambda, state_size,
                                  knot_points, &cfg, &res, nullptr);
    else
        rc = gbdpcg_solve_dev_f64(h, d_S, d_Pinv, GBDPCG_PINV_CBTD, d_gamma, d_lambda, state_size,
                                  knot_points, &cfg, &res, nullptr);
    gpuErrchk(rc);
    gpuErrchk(gbdpcg_detail::convergence_status(res));
    return res.iters;
}

// CSR overload (include/interface.cuh:8-20, which exits "NOT IMPLEMENTED" in
// the reference).  h_S and, if non-null, h_Pinv are csr_t with host arrays
// describing n N x n N block-tridiagonal matrices (row r in knot r / n); they
// are copied to the device and scattered into the cbtd layout there
// (gbdpcg_csr_to_cbtd_*).  A null h_Pinv builds the block-Jacobi Phi^-1 on the
// GPU.  Returns the iteration count; h_lambda is the initial guess on entry.
template <typename T>
uint32_t solvePCG(csr_t<T> *h_S, csr_t<T> *h_Pinv, T *h_gamma, T *h_lambda, unsigned stateSize,
                  unsigned knotPoints, struct pcg_config<T> *config) {
    static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value, "float or double");
    const uint32_t n = stateSize, N = knotPoints, rows = n * N;
    if (!h_S || h_S->rows != rows || h_S->cols != rows || (h_Pinv && (h_Pinv->rows != rows || h_Pinv->cols != rows)))
        gpuErrchk(GBDPCG_ERR_INVALID_ARGUMENT);
    const size_t mat = (size_t)3 * n * n * N;
    gbdpcg_handle_t h = gbdpcg_detail::thread_handle();
    T *d_S = nullptr, *d_P = nullptr, *d_g = nullptr, *d_l = nullptr;
    uint32_t *d_err = nullptr;
    gpuErrchk(cudaMalloc(&d_S, sizeof(T) * mat) == cudaSuccess ? GBDPCG_SUCCESS : GBDPCG_ERR_NO_MEMORY);
    gpuErrchk(cudaMalloc(&d_P, sizeof(T) * mat) == cudaSuccess ? GBDPCG_SUCCESS : GBDPCG_ERR_NO_MEMORY);
    gpuErrchk(cudaMalloc(&d_g, sizeof(T) * rows) == cudaSuccess ? GBDPCG_SUCCESS : GBDPCG_ERR_NO_MEMORY);
    gpuErrchk(cudaMalloc(&d_l, sizeof(T) * rows) == cudaSuccess ? GBDPCG_SUCCESS : GBDPCG_ERR_NO_MEMORY);
    gpuErrchk(cudaMalloc(&d_err, sizeof(uint32_t)) == cudaSuccess ? GBDPCG_SUCCESS : GBDPCG_ERR_NO_MEMORY);
    auto upload_csr = [&](const csr_t<T> *m, T *d_out) {
        uint32_t *d_rp = nullptr, *d_ci = nullptr;
        T *d_v = nullptr;
        const size_t nnz = m->nnz;
        gpuErrchk(cudaMalloc(&d_rp, sizeof(uint32_t) * (rows + 1)) == cudaSuccess ? GBDPCG_SUCCESS : GBDPCG_ERR_NO_MEMORY);
        gpuErrchk(cudaMalloc(&d_ci, sizeof(uint32_t) * (nnz ? nnz : 1)) == cudaSuccess ? GBDPCG_SUCCESS : GBDPCG_ERR_NO_MEMORY);
        gpuErrchk(cudaMalloc(&d_v, sizeof(T) * (nnz ? nnz : 1)) == cudaSuccess ? GBDPCG_SUCCESS : GBDPCG_ERR_NO_MEMORY);
        cudaMemcpy(d_rp, m->row_ptr, sizeof(uint32_t) * (rows + 1), cudaMemcpyHostToDevice);
        if (nnz) {
            cudaMemcpy(d_ci, m->col_ind, sizeof(uint32_t) * nnz, cudaMemcpyHostToDevice);
            cudaMemcpy(d_v, m->val, sizeof(T) * nnz, cudaMemcpyHostToDevice);
        }
        int rc;
        if constexpr (std::is_same<T, float>::value) rc = gbdpcg_csr_to_cbtd_f32(d_rp, d_ci, d_v, n, N, d_out, d_err, nullptr);
        else rc = gbdpcg_csr_to_cbtd_f64(d_rp, d_ci, d_v, n, N, d_out, d_err, nullptr);
        cudaFree(d_rp);
        cudaFree(d_ci);
        cudaFree(d_v);
        gpuErrchk(rc);
    };
    upload_csr(h_S, d_S);
    if (h_Pinv) {
        upload_csr(h_Pinv, d_P);
    } else {
        int rc;
        if constexpr (std::is_same<T, float>::value) rc = gbdpcg_block_jacobi_f32(h, d_S, d_P, GBDPCG_PINV_CBTD, n, N, nullptr);
        else rc = gbdpcg_block_jacobi_f64(h, d_S, d_P, GBDPCG_PINV_CBTD, n, N, nullptr);
        gpuErrchk(rc);
    }
    cudaMemcpy(d_g, h_gamma, sizeof(T) * rows, cudaMemcpyHostToDevice);
    cudaMemcpy(d_l, h_lambda, sizeof(T) * rows, cudaMemcpyHostToDevice);
    const uint32_t iters = solvePCG<T>(n, N, d_S, d_P, d_g, d_l, nullptr, nullptr, nullptr, nullptr, config);
    cudaMemcpy(h_lambda, d_l, sizeof(T) * rows, cudaMemcpyDeviceToHost);
    cudaFree(d_S);
    cudaFree(d_P);
    cudaFree(d_g);
    cudaFree(d_l);
    cudaFree(d_err);
    return iters;
}

// The documented API (README.md:42): Phi^-1 is built on the GPU.
template <typename T>
int pcg_solve(T *h_S, T *h_gamma, T *h_lambda, unsigned stateSize, unsigned knotPoints,
              struct pcg_config<T> *config = nullptr) {
    return (int)solvePCG<T>(h_S, nullptr, h_gamma, h_lambda, stateSize, knotPoints, config);
}
