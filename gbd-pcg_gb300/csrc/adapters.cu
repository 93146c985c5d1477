// Input adapters around the solver.
//
// CSR -> cbtd.  The reference declares a solvePCG overload taking S and Phi^-1
// as csr_t (include/interface.cuh:8-20, type at include/types.cuh:7-15) but
// its body prints "NOT IMPLEMENTED" and exits.  Here a CSR matrix of a
// block-tridiagonal system (rows = cols = n N; row r belongs to knot r / n)
// is scattered into the compressed block-tridiagonal layout the solver reads:
// entry (r, c) goes to block b = c / n - r / n + 1 of knot k = r / n, at
// k*3n^2 + (b*n + c % n)*n + r % n.  One thread per row, so no two threads
// write the same element; duplicate entries of a row add up.  An entry
// outside the three diagonal blocks of its row (or past the last column) is
// not written and raises the error word.
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/gbdpcg.h"

namespace gbdpcg {
void set_last_error(const std::string &msg);
}

namespace {

template <typename T>
__global__ void csr_to_cbtd_kernel(const uint32_t *__restrict__ row_ptr, const uint32_t *__restrict__ col_ind,
                                   const T *__restrict__ val, uint32_t n, uint32_t N, T *__restrict__ out,
                                   uint32_t *err) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t rows = n * N;
    if (r >= rows) return;
    const uint32_t k = r / n, i = r - k * n;
    T *row = out + (size_t)k * 3 * n * n + i;
    const uint32_t e0 = row_ptr[r], e1 = row_ptr[r + 1];
    for (uint32_t e = e0; e < e1; ++e) {
        const uint32_t c = col_ind[e];
        const uint32_t kc = c / n;
        if (c >= rows || kc + 1 < k || kc > k + 1) {
            atomicOr(err, 1u);
            continue;
        }
        const uint32_t b = kc + 1 - k, j = c - kc * n;
        row[(size_t)(b * n + j) * n] += val[e];
    }
}

template <typename T>
int csr_to_cbtd(const uint32_t *d_row_ptr, const uint32_t *d_col_ind, const T *d_val, uint32_t n, uint32_t N,
                T *d_out, uint32_t *d_err, cudaStream_t st) {
    if (!d_row_ptr || !d_col_ind || !d_val || !d_out || !d_err) {
        gbdpcg::set_last_error("NULL pointer");
        return GBDPCG_ERR_INVALID_ARGUMENT;
    }
    if (n == 0 || N == 0) {
        gbdpcg::set_last_error("n and N must be positive");
        return GBDPCG_ERR_INVALID_ARGUMENT;
    }
    cudaError_t e = cudaMemsetAsync(d_out, 0, sizeof(T) * 3 * (size_t)n * n * N, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_err, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) {
        const uint32_t rows = n * N, tpb = 128;
        csr_to_cbtd_kernel<T><<<(rows + tpb - 1) / tpb, tpb, 0, st>>>(d_row_ptr, d_col_ind, d_val, n, N, d_out, d_err);
        e = cudaGetLastError();
    }
    uint32_t h_err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_err, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        gbdpcg::set_last_error(std::string("csr_to_cbtd: ") + cudaGetErrorString(e));
        return GBDPCG_ERR_CUDA;
    }
    if (h_err) {
        gbdpcg::set_last_error("csr_to_cbtd: an entry lies outside the block-tridiagonal band of its row");
        return GBDPCG_ERR_INVALID_ARGUMENT;
    }
    return GBDPCG_SUCCESS;
}

}  // namespace

extern "C" {

int gbdpcg_csr_to_cbtd_f32(const uint32_t *d_row_ptr, const uint32_t *d_col_ind, const float *d_val, uint32_t n,
                           uint32_t N, float *d_out, uint32_t *d_err, gbdpcg_stream_t stream) {
    return csr_to_cbtd<float>(d_row_ptr, d_col_ind, d_val, n, N, d_out, d_err, (cudaStream_t)stream);
}

int gbdpcg_csr_to_cbtd_f64(const uint32_t *d_row_ptr, const uint32_t *d_col_ind, const double *d_val, uint32_t n,
                           uint32_t N, double *d_out, uint32_t *d_err, gbdpcg_stream_t stream) {
    return csr_to_cbtd<double>(d_row_ptr, d_col_ind, d_val, n, N, d_out, d_err, (cudaStream_t)stream);
}

}  // extern "C"
