// Input adapters around the solver.
//
// CSR -> cbtd.  The reference declares a solvePCG overload taking S and Phi^-1
// as csr_t (include/interface.cuh:8-20, type at include/types.cuh:7-15) but
// its body prints "NOT IMPLEMENTED" and exits.  Here a CSR matrix of a
// block-tridiagonal system (rows = cols = n N; row r belongs to knot r / n)
// is scattered into the compressed block-tridiagonal layout the solver reads:
// entry (r, c) goes to block b = c / n - r / n + 1 of knot k = r / n, at
// k*3n^2 + (b*n + c % n)*n + r % n.
//
// One warp per knot.  The knot's n rows are one contiguous run of entries, so
// the lanes read column indices and values coalesced; each entry is added
// into a shared-memory tile of the knot's n x 3n block row (its row from a
// per-lane cursor over the knot's n + 1 row pointers, its block and column
// from one subtraction), and the finished tile is written once, coalesced, padding
// blocks included (no separate zeroing pass).  Duplicate entries of a row add
// (in an unspecified order when there are more than two).  An entry outside
// the three diagonal blocks of its row (or past the last column) is not
// written and raises the error word.  For n > 32 (tiles too large for shared
// memory) one thread per row scatters into the zeroed output instead.
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/gbdpcg.h"

namespace gbdpcg {
void set_last_error(const std::string &msg);
}

namespace {

constexpr int kCsrWarps = 4;  // knots per CTA

// elements of one warp's tile, rounded to keep every tile 16-byte aligned
__host__ __device__ inline uint32_t csr_tile_elems(uint32_t n) { return (3 * n * n + 3) & ~3u; }

template <typename T>
__host__ __device__ inline size_t csr_smem_bytes(uint32_t n) {
    return (size_t)kCsrWarps * (csr_tile_elems(n) * sizeof(T) + 33 * sizeof(uint32_t));
}

template <typename T>
__global__ void __launch_bounds__(kCsrWarps * 32)
    csr_to_cbtd_kernel(const uint32_t *__restrict__ row_ptr, const uint32_t *__restrict__ col_ind,
                       const T *__restrict__ val, uint32_t n, uint32_t N, T *__restrict__ out, uint32_t *err) {
    extern __shared__ __align__(16) unsigned char csr_smem[];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t k = blockIdx.x * kCsrWarps + warp;
    if (k >= N) return;  // warp-uniform; no CTA-wide barrier below
    const uint32_t te = csr_tile_elems(n), nn3 = 3 * n * n;
    T *tile = reinterpret_cast<T *>(csr_smem) + (size_t)warp * te;
    uint32_t *rpl = reinterpret_cast<uint32_t *>(csr_smem + (size_t)kCsrWarps * te * sizeof(T)) + warp * 33;
    for (uint32_t e = lane; e < nn3; e += 32) tile[e] = T(0);
    if (lane <= n) rpl[lane] = row_ptr[(size_t)k * n + lane];
    __syncwarp();
    const uint32_t e0 = rpl[0], e1 = rpl[n], rows = n * N;
    const uint32_t cbase = k * n - n;  // first column of knot k-1 (wraps for k = 0)
    bool bad = false;
    constexpr int U = 8;  // entries per lane in flight
    uint32_t row = 0;     // this lane's entries only move forward: rpl[row] <= e < rpl[row + 1]
    for (uint32_t base = e0; base < e1; base += 32 * U) {
        uint32_t cc[U];
        T vv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t e = base + u * 32 + lane;
            cc[u] = e < e1 ? col_ind[e] : 0u;
            vv[u] = e < e1 ? val[e] : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t e = base + u * 32 + lane;
            if (e >= e1) break;
            while (rpl[row + 1] <= e) ++row;  // stops below n: e < rpl[n]
            const uint32_t d = cc[u] - cbase;  // column offset from knot k-1's first column
            if (cc[u] >= rows || d >= 3 * n) bad = true;
            else atomicAdd(&tile[d * n + row], vv[u]);  // (b n + j) n + i with d = b n + j
        }
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(err, 1u);
    __syncwarp();
    T *dst = out + (size_t)k * nn3;
    for (uint32_t e = lane; e < nn3; e += 32) dst[e] = tile[e];
}

// n > 32: one thread per row, adding into the zeroed output (no two threads
// write one element).
template <typename T>
__global__ void csr_rows_to_cbtd_kernel(const uint32_t *__restrict__ row_ptr, const uint32_t *__restrict__ col_ind,
                                        const T *__restrict__ val, uint32_t n, uint32_t N, T *__restrict__ out,
                                        uint32_t *err) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t rows = n * N;
    if (r >= rows) return;
    const uint32_t k = r / n, i = r - k * n;
    T *row = out + (size_t)k * 3 * n * n + i;
    const uint32_t cbase = k * n - n;
    for (uint32_t e = row_ptr[r], e1 = row_ptr[r + 1]; e < e1; ++e) {
        const uint32_t c = col_ind[e], d = c - cbase;
        if (c >= rows || d >= 3 * n) {
            atomicOr(err, 1u);
            continue;
        }
        row[(size_t)d * n] += val[e];
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
    if ((uint64_t)n * N >= (1ull << 32) / 3) {
        gbdpcg::set_last_error("csr_to_cbtd: n N too large for 32-bit column indices");
        return GBDPCG_ERR_INVALID_ARGUMENT;
    }
    cudaError_t e = cudaMemsetAsync(d_err, 0, sizeof(uint32_t), st);
    if (n <= 32) {
        const size_t smem = csr_smem_bytes<T>(n);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(csr_to_cbtd_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) {
            csr_to_cbtd_kernel<T><<<(N + kCsrWarps - 1) / kCsrWarps, kCsrWarps * 32, smem, st>>>(
                d_row_ptr, d_col_ind, d_val, n, N, d_out, d_err);
            e = cudaGetLastError();
        }
    } else {
        if (e == cudaSuccess) e = cudaMemsetAsync(d_out, 0, sizeof(T) * 3 * (size_t)n * n * N, st);
        if (e == cudaSuccess) {
            const uint32_t rows = n * N, tpb = 128;
            csr_rows_to_cbtd_kernel<T><<<(rows + tpb - 1) / tpb, tpb, 0, st>>>(d_row_ptr, d_col_ind, d_val, n, N,
                                                                               d_out, d_err);
            e = cudaGetLastError();
        }
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

// Dense -> cbtd.  A dense n N x n N matrix (leading dimension ld, column- or
// row-major) gives its three diagonal blocks per block row: block b of knot k
// is D[k n .. k n + n, (k + b - 1) n .. (k + b - 1) n + n].  One CTA per (knot,
// block); column-major sources are copied straight (contiguous on both sides),
// row-major ones through a shared-memory transpose.  The padding blocks of
// knots 0 and N-1 are written as zeros.
template <typename T, bool ROW_MAJOR>
__global__ void __launch_bounds__(128) dense_to_cbtd_kernel(const T *__restrict__ D, uint64_t ld, uint32_t n,
                                                            uint32_t N, T *__restrict__ out) {
    __shared__ T tile[32 * 33];
    const uint32_t k = blockIdx.x / 3, b = blockIdx.x - 3 * (blockIdx.x / 3);
    const uint32_t nn = n * n;
    T *dst = out + (size_t)k * 3 * nn + (size_t)b * nn;
    const bool present = (b != 0 || k > 0) && (b != 2 || k + 1 < N);
    if (!present) {
        for (uint32_t e = threadIdx.x; e < nn; e += blockDim.x) dst[e] = T(0);
        return;
    }
    const uint64_t r0 = (uint64_t)k * n, c0 = (uint64_t)(k + b - 1) * n;
    if constexpr (!ROW_MAJOR) {
        for (uint32_t e = threadIdx.x; e < nn; e += blockDim.x) {
            const uint32_t j = e / n, i = e - j * n;  // e = j n + i: (i, j) of the block
            dst[e] = D[(c0 + j) * ld + r0 + i];
        }
    } else {
        // n <= 32: the block goes through one padded tile
        for (uint32_t e = threadIdx.x; e < nn; e += blockDim.x) {
            const uint32_t i = e / n, j = e - i * n;  // e = i n + j: row-major read
            tile[i * 33 + j] = D[(r0 + i) * ld + c0 + j];
        }
        __syncthreads();
        for (uint32_t e = threadIdx.x; e < nn; e += blockDim.x) {
            const uint32_t j = e / n, i = e - j * n;
            dst[e] = tile[i * 33 + j];
        }
    }
}

// Flags any nonzero entry of D outside the block-tridiagonal band.
template <typename T, bool ROW_MAJOR>
__global__ void dense_band_check_kernel(const T *__restrict__ D, uint64_t ld, uint32_t n, uint32_t N,
                                        uint32_t *err) {
    const uint64_t rows = (uint64_t)n * N, total = rows * rows;
    bool bad = false;
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t outer = e / rows, inner = e - outer * rows;  // contiguous index inner
        const uint64_t r = ROW_MAJOR ? outer : inner, cc = ROW_MAJOR ? inner : outer;
        const uint64_t kr = r / n, kc = cc / n;
        if (kr > kc + 1 || kc > kr + 1) bad |= D[outer * ld + inner] != T(0);
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(err, 1u);
}

template <typename T>
int dense_to_cbtd(const T *d_D, uint64_t ld, int row_major, uint32_t n, uint32_t N, T *d_out, uint32_t *d_err,
                  cudaStream_t st) {
    if (!d_D || !d_out) {
        gbdpcg::set_last_error("NULL pointer");
        return GBDPCG_ERR_INVALID_ARGUMENT;
    }
    if (n == 0 || N == 0 || n > 32) {
        gbdpcg::set_last_error("dense_to_cbtd: need 1 <= n <= 32 and N >= 1");
        return GBDPCG_ERR_INVALID_ARGUMENT;
    }
    if (ld < (uint64_t)n * N || (uint64_t)N * 3 > 0x7fffffffull) {
        gbdpcg::set_last_error("dense_to_cbtd: leading dimension below n N, or N too large");
        return GBDPCG_ERR_INVALID_ARGUMENT;
    }
    cudaError_t e = cudaSuccess;
    if (row_major) dense_to_cbtd_kernel<T, true><<<3 * N, 128, 0, st>>>(d_D, ld, n, N, d_out);
    else dense_to_cbtd_kernel<T, false><<<3 * N, 128, 0, st>>>(d_D, ld, n, N, d_out);
    e = cudaGetLastError();
    if (e == cudaSuccess && d_err) {
        e = cudaMemsetAsync(d_err, 0, sizeof(uint32_t), st);
        if (e == cudaSuccess) {
            if (row_major) dense_band_check_kernel<T, true><<<1216, 256, 0, st>>>(d_D, ld, n, N, d_err);
            else dense_band_check_kernel<T, false><<<1216, 256, 0, st>>>(d_D, ld, n, N, d_err);
            e = cudaGetLastError();
        }
        uint32_t h_err = 0;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&h_err, d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e == cudaSuccess && h_err) {
            gbdpcg::set_last_error("dense_to_cbtd: a nonzero entry lies outside the block-tridiagonal band");
            return GBDPCG_ERR_INVALID_ARGUMENT;
        }
    }
    if (e != cudaSuccess) {
        gbdpcg::set_last_error(std::string("dense_to_cbtd: ") + cudaGetErrorString(e));
        return GBDPCG_ERR_CUDA;
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

int gbdpcg_dense_to_cbtd_f32(const float *d_D, uint64_t ld, int row_major, uint32_t n, uint32_t N, float *d_out,
                             uint32_t *d_err, gbdpcg_stream_t stream) {
    return dense_to_cbtd<float>(d_D, ld, row_major, n, N, d_out, d_err, (cudaStream_t)stream);
}

int gbdpcg_dense_to_cbtd_f64(const double *d_D, uint64_t ld, int row_major, uint32_t n, uint32_t N, double *d_out,
                             uint32_t *d_err, gbdpcg_stream_t stream) {
    return dense_to_cbtd<double>(d_D, ld, row_major, n, N, d_out, d_err, (cudaStream_t)stream);
}

}  // extern "C"
