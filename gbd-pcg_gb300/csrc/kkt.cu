// The steps on either side of the PCG in a trajectory-optimisation solver
// (the callers of solvePCG in MPCGPU / GATO, outside the reference repo):
// forming the Schur complement S and its right-hand side gamma from the
// problem data, and recovering the primal step from the multipliers lambda.
//
// Problem (one system): states x_0..x_N (n each), controls u_0..u_{N-1}
// (m each), z = (x, u); cost 1/2 z^T Theta z + g^T z with Theta =
// blockdiag(Q_0..Q_N, R_0..R_{N-1}), Q_k = diag(Qd_k), R_k = diag(Rd_k),
// g = (q_0..q_N, r_0..r_{N-1}); constraints C z = c with one block row
// [A_k  B_k  -I] per knot acting on (x_k, u_k, x_{k+1}), k = 0..N-1.  The KKT
// system [Theta C^T; C 0] [z; lambda] = [-g; c] reduces to
//     S lambda = gamma,  S = C Theta^-1 C^T,  gamma = -(c + C Theta^-1 g),
//     z = -Theta^-1 (g + C^T lambda):
//   S_kk      = A_k Q_k^-1 A_k^T + B_k R_k^-1 B_k^T + Q_{k+1}^-1
//   S_{k,k+1} = -Q_{k+1}^-1 A_{k+1}^T,  S_{k+1,k} = S_{k,k+1}^T
//   gamma_k   = -(c_k + A_k Q_k^-1 q_k + B_k R_k^-1 r_k - Q_{k+1}^-1 q_{k+1})
//   x_k = -Q_k^-1 (q_k + A_k^T lambda_k - lambda_{k-1})   (terms present for k < N, k > 0)
//   u_k = -R_k^-1 (r_k + B_k^T lambda_k)
// Inputs A_k (n x n) and B_k (n x m) are column-major blocks, knot-major:
// element (r, c) of A_k at k n^2 + c n + r, of B_k at k n m + c n + r.  S is
// written in the cbtd layout (padding blocks of knots 0 and N-1 zero), gamma
// and lambda are n N, x is n (N+1), u is m N.
//
// Both kernels run one warp per knot (lane i owns row i of the knot's
// blocks); they read each input once and write each output once, so HBM
// bandwidth bounds them.  S_kk is symmetrised through shared memory
// (0.5 (S + S^T), exactly symmetric).
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/gbdpcg.h"

namespace gbdpcg {
void set_last_error(const std::string &msg);
}

namespace {

constexpr int kKktMaxN = 32;  // n, m <= 32
// knots per CTA (4 float, 2 double: 36 KB of static shared memory either way)
template <typename T>
constexpr int kkt_warps() { return sizeof(T) == 8 ? 2 : 4; }

// Shared-memory rows of a knot's blocks: kKktMaxN columns padded to a 16-byte
// multiple, so that 16-byte vectors of consecutive columns can be loaded.
template <typename T>
__host__ __device__ constexpr int kkt_vw() { return 16 / (int)sizeof(T); }
template <typename T>
__host__ __device__ constexpr uint32_t kkt_ld() { return kKktMaxN + kkt_vw<T>(); }

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using type = float4;
    __device__ static void get(const float *p, float (&v)[4]) {
        const float4 t = *reinterpret_cast<const float4 *>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
};
template <>
struct Vec16<double> {
    __device__ static void get(const double *p, double (&v)[2]) {
        const double2 t = *reinterpret_cast<const double2 *>(p);
        v[0] = t.x; v[1] = t.y;
    }
};

// Lane r (< rows) loads row r of a column-major rows x cols block into sM[r][*]
// (one coalesced column per load, all loads in flight together); columns from
// cols up to the next vector boundary are zero.
template <typename T>
__device__ __forceinline__ void load_block(T *sM, uint32_t ld, const T *g, uint32_t rows, uint32_t cols,
                                           uint32_t lane) {
    constexpr int VW = kkt_vw<T>();
    T t[kKktMaxN];
#pragma unroll
    for (int cc = 0; cc < kKktMaxN; ++cc) t[cc] = ((uint32_t)cc < cols && lane < rows) ? g[(size_t)cc * rows + lane] : T(0);
    const uint32_t cpad = (cols + VW - 1) / VW * VW;
#pragma unroll
    for (int cc = 0; cc < kKktMaxN; ++cc)
        if ((uint32_t)cc < cpad && lane < rows) sM[lane * ld + cc] = t[cc];
}

// acc[j] += sum_l a[l] * M[j][l] over l < cols (VW columns per load), and
// g += sum_l a[l] * w[l], with a[l] = M[i][l] * d[l]: lane i's row of
// M diag(d) M^T and of M diag(d) w.
template <typename T>
__device__ __forceinline__ void row_gram(const T *M, uint32_t ld, const T *d, const T *w, uint32_t i, uint32_t rows,
                                         uint32_t cols, T (&acc)[kKktMaxN], T &g) {
    constexpr int VW = kkt_vw<T>();
    for (uint32_t l = 0; l < cols; l += VW) {
        T mi[VW], dv[VW], wv[VW], a[VW];
        Vec16<T>::get(M + i * ld + l, mi);
#pragma unroll
        for (int u = 0; u < VW; ++u) {
            const bool in = l + u < cols;
            dv[u] = in ? d[l + u] : T(0);
            wv[u] = in ? w[l + u] : T(0);
            a[u] = mi[u] * dv[u];
            g += mi[u] * (dv[u] * wv[u]);
        }
#pragma unroll
        for (int j = 0; j < kKktMaxN; ++j) {
            if ((uint32_t)j < rows) {
                T mj[VW];
                Vec16<T>::get(M + j * ld + l, mj);
#pragma unroll
                for (int u = 0; u < VW; ++u) acc[j] += a[u] * mj[u];
            }
        }
    }
}

template <typename T, int kKktWarps = kkt_warps<T>()>
__global__ void __launch_bounds__(kKktWarps * 32)
    form_schur_kernel(const T *__restrict__ A, const T *__restrict__ B, const T *__restrict__ Qd,
                      const T *__restrict__ Rd, const T *__restrict__ q, const T *__restrict__ r,
                      const T *__restrict__ c, uint32_t n, uint32_t m, uint32_t N, T *__restrict__ S,
                      T *__restrict__ gamma) {
    constexpr uint32_t ld = kkt_ld<T>();
    __shared__ __align__(16) T sA[kKktWarps][kKktMaxN * ld];  // A_k, then S_kk
    __shared__ __align__(16) T sB[kKktWarps][kKktMaxN * ld];
    __shared__ T sv[kKktWarps][5][kKktMaxN];  // Qi_k, Ri_k, Qi_{k+1}, q_k, r_k
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t k = blockIdx.x * kKktWarps + warp;
    if (k >= N) return;  // warp-uniform; no CTA barrier below
    T *Ak = sA[warp], *Bk = sB[warp];
    T *qi = sv[warp][0], *ri = sv[warp][1], *qn = sv[warp][2], *qk = sv[warp][3], *rk = sv[warp][4];
    load_block(Ak, ld, A + (size_t)k * n * n, n, n, lane);  // Ak[row][col]
    load_block(Bk, ld, B + (size_t)k * n * m, n, m, lane);
    if (lane < n) {
        qi[lane] = T(1) / Qd[(size_t)k * n + lane];
        qn[lane] = T(1) / Qd[(size_t)(k + 1) * n + lane];
        qk[lane] = q[(size_t)k * n + lane];
    }
    if (lane < m) {
        ri[lane] = T(1) / Rd[(size_t)k * m + lane];
        rk[lane] = r[(size_t)k * m + lane];
    }
    __syncwarp();
    T *Sk = S + (size_t)k * 3 * n * n;
    // block 0 of row k: S_{k,k-1}, element (i, j) = -Qi_k[j] A_k[i][j]; block 2
    // of row k-1: S_{k-1,k}, element (i, j) = -Qi_k[i] A_k[j][i] (this warp holds
    // A_k, so each A_k is read once); the last row's block 2 is padding
    T *Sup = (k > 0) ? S + (size_t)(k - 1) * 3 * n * n + 2 * (size_t)n * n : nullptr;
    if (lane < n) {  // column by column, lane = row: coalesced, no index division
        const uint32_t row = lane;
        for (uint32_t col = 0; col < n; ++col) {
            const uint32_t e = col * n + row;
            Sk[e] = (k > 0) ? -qi[col] * Ak[row * ld + col] : T(0);
            if (k > 0) Sup[e] = -qi[row] * Ak[col * ld + row];
            if (k + 1 == N) Sk[2 * (size_t)n * n + e] = T(0);
        }
    }
    // row i of S_kk (unsymmetrised) and gamma_k
    T srow[kKktMaxN];
    T g = T(0);
    if (lane < n) {
        const uint32_t i = lane;
#pragma unroll
        for (int j = 0; j < kKktMaxN; ++j) srow[j] = T(0);
        row_gram(Ak, ld, qi, qk, i, n, n, srow, g);  // A Q^-1 A^T, A Q^-1 q
        row_gram(Bk, ld, ri, rk, i, n, m, srow, g);  // B R^-1 B^T, B R^-1 r
#pragma unroll
        for (int j = 0; j < kKktMaxN; ++j)
            if ((uint32_t)j == i) srow[j] += qn[i];
        gamma[(size_t)k * n + i] = -(c[(size_t)k * n + i] + g - qn[i] * q[(size_t)(k + 1) * n + i]);
    }
    __syncwarp();  // every lane is done with Ak
    if (lane < n) {
#pragma unroll
        for (int j = 0; j < kKktMaxN; ++j)
            if ((uint32_t)j < n) Ak[lane * ld + j] = srow[j];
    }
    __syncwarp();
    // block 1: S_kk symmetrised
    if (lane < n) {
        const uint32_t row = lane;
        for (uint32_t col = 0; col < n; ++col)
            Sk[n * n + col * n + row] = T(0.5) * (Ak[row * ld + col] + Ak[col * ld + row]);
    }
}

// s + sum_j col[j] w[j], j ascending.  A lane reads its own contiguous column:
// 16-byte loads when both pointers are 16-byte aligned and n is a multiple of
// the vector width (a quarter of the L1 requests of scalar loads; the
// products are added in the same order either way).
template <typename T>
__device__ __forceinline__ T col_dot(const T *col, const T *w, uint32_t n, T s) {
    constexpr int VW = kkt_vw<T>();
    if ((n % VW) == 0 && ((reinterpret_cast<uintptr_t>(col) | reinterpret_cast<uintptr_t>(w)) & 15u) == 0) {
        for (uint32_t j = 0; j < n; j += VW) {
            T a[VW], b[VW];
            Vec16<T>::get(col + j, a);
            Vec16<T>::get(w + j, b);
#pragma unroll
            for (int u = 0; u < VW; ++u) s += a[u] * b[u];
        }
        return s;
    }
    for (uint32_t j = 0; j < n; ++j) s += col[j] * w[j];
    return s;
}

template <typename T, int kKktWarps = kkt_warps<T>()>
__global__ void __launch_bounds__(kKktWarps * 32)
    kkt_backsub_kernel(const T *__restrict__ A, const T *__restrict__ B, const T *__restrict__ Qd,
                       const T *__restrict__ Rd, const T *__restrict__ q, const T *__restrict__ r,
                       const T *__restrict__ lambda, uint32_t n, uint32_t m, uint32_t N, T *__restrict__ x,
                       T *__restrict__ u) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t k = blockIdx.x * kKktWarps + warp;  // knots 0..N (x) and 0..N-1 (u)
    if (k > N) return;
    if (lane < n) {
        const uint32_t i = lane;
        T s = q[(size_t)k * n + i];
        if (k < N) {  // + (A_k^T lambda_k)_i = sum_j A_k[j][i] lambda_k[j]; column i of A_k is contiguous
            const T *Acol = A + (size_t)k * n * n + (size_t)i * n;
            const T *lk = lambda + (size_t)k * n;
            s = col_dot(Acol, lk, n, s);
        }
        if (k > 0) s -= lambda[(size_t)(k - 1) * n + i];
        x[(size_t)k * n + i] = -s / Qd[(size_t)k * n + i];
    }
    if (k < N && lane < m) {
        const uint32_t i = lane;
        T s = r[(size_t)k * m + i];
        const T *Bcol = B + (size_t)k * n * m + (size_t)i * n;
        const T *lk = lambda + (size_t)k * n;
        s = col_dot(Bcol, lk, n, s);
        u[(size_t)k * m + i] = -s / Rd[(size_t)k * m + i];
    }
}

int check(const void *const *ptrs, int np, uint32_t n, uint32_t m, uint32_t N) {
    for (int i = 0; i < np; ++i)
        if (!ptrs[i]) {
            gbdpcg::set_last_error("NULL pointer");
            return GBDPCG_ERR_INVALID_ARGUMENT;
        }
    if (n == 0 || m == 0 || N == 0) {
        gbdpcg::set_last_error("n, m and N must be positive");
        return GBDPCG_ERR_INVALID_ARGUMENT;
    }
    if (n > (uint32_t)kKktMaxN || m > (uint32_t)kKktMaxN) {
        gbdpcg::set_last_error("n and m must be <= 32");
        return GBDPCG_ERR_UNSUPPORTED;
    }
    return GBDPCG_SUCCESS;
}

int launched(const char *what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        gbdpcg::set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
        return GBDPCG_ERR_CUDA;
    }
    return GBDPCG_SUCCESS;
}

template <typename T>
int form_schur(const T *A, const T *B, const T *Qd, const T *Rd, const T *q, const T *r, const T *c, uint32_t n,
               uint32_t m, uint32_t N, T *S, T *gamma, cudaStream_t st) {
    const void *p[] = {A, B, Qd, Rd, q, r, c, S, gamma};
    int rc = check(p, 9, n, m, N);
    if (rc) return rc;
    constexpr int W = kkt_warps<T>();
    form_schur_kernel<T><<<(N + W - 1) / W, W * 32, 0, st>>>(A, B, Qd, Rd, q, r, c, n, m,
                                                                                       N, S, gamma);
    return launched("form_schur");
}

template <typename T>
int kkt_backsub(const T *A, const T *B, const T *Qd, const T *Rd, const T *q, const T *r, const T *lambda,
                uint32_t n, uint32_t m, uint32_t N, T *x, T *u, cudaStream_t st) {
    const void *p[] = {A, B, Qd, Rd, q, r, lambda, x, u};
    int rc = check(p, 9, n, m, N);
    if (rc) return rc;
    constexpr int W = kkt_warps<T>();
    kkt_backsub_kernel<T><<<(N + 1 + W - 1) / W, W * 32, 0, st>>>(A, B, Qd, Rd, q, r,
                                                                                           lambda, n, m, N, x, u);
    return launched("kkt_backsub");
}

}  // namespace

extern "C" {

int gbdpcg_form_schur_f32(const float *d_A, const float *d_B, const float *d_Qd, const float *d_Rd,
                          const float *d_q, const float *d_r, const float *d_c, uint32_t n, uint32_t m, uint32_t N,
                          float *d_S, float *d_gamma, gbdpcg_stream_t stream) {
    return form_schur<float>(d_A, d_B, d_Qd, d_Rd, d_q, d_r, d_c, n, m, N, d_S, d_gamma, (cudaStream_t)stream);
}
int gbdpcg_form_schur_f64(const double *d_A, const double *d_B, const double *d_Qd, const double *d_Rd,
                          const double *d_q, const double *d_r, const double *d_c, uint32_t n, uint32_t m,
                          uint32_t N, double *d_S, double *d_gamma, gbdpcg_stream_t stream) {
    return form_schur<double>(d_A, d_B, d_Qd, d_Rd, d_q, d_r, d_c, n, m, N, d_S, d_gamma, (cudaStream_t)stream);
}
int gbdpcg_kkt_backsub_f32(const float *d_A, const float *d_B, const float *d_Qd, const float *d_Rd,
                           const float *d_q, const float *d_r, const float *d_lambda, uint32_t n, uint32_t m,
                           uint32_t N, float *d_x, float *d_u, gbdpcg_stream_t stream) {
    return kkt_backsub<float>(d_A, d_B, d_Qd, d_Rd, d_q, d_r, d_lambda, n, m, N, d_x, d_u, (cudaStream_t)stream);
}
int gbdpcg_kkt_backsub_f64(const double *d_A, const double *d_B, const double *d_Qd, const double *d_Rd,
                           const double *d_q, const double *d_r, const double *d_lambda, uint32_t n, uint32_t m,
                           uint32_t N, double *d_x, double *d_u, gbdpcg_stream_t stream) {
    return kkt_backsub<double>(d_A, d_B, d_Qd, d_Rd, d_q, d_r, d_lambda, n, m, N, d_x, d_u, (cudaStream_t)stream);
}

}  // extern "C"
