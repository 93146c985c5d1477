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
// Both kernels run one warp per knot and read each input once and write each
// output once, so HBM bandwidth bounds them.  The formation stages [A_k | B_k]
// in shared memory and forms its Gram product as a register tile per lane;
// S_kk is symmetrised through shared memory (0.5 (S + S^T), exactly
// symmetric), and the formation can invert S_kk in the same warp (the
// block-Jacobi Phi^-1).  The back-substitution's lane i reads column i of
// A_k and B_k.
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <type_traits>

#include "../../include/gbdpcg.h"
#include "gauss_jordan.cuh"

namespace gbdpcg {
void set_last_error(const std::string &msg);
}

namespace {

constexpr int kKktMaxN = 32;  // n, m <= 32
// knots per CTA (4 float, 2 double: at most about 40 KB of dynamic shared
// memory either way in the formation)
template <typename T>
constexpr int kkt_warps() { return sizeof(T) == 8 ? 2 : 4; }

// elements of one 16-byte vector
template <typename T>
__host__ __device__ constexpr int kkt_vw() { return 16 / (int)sizeof(T); }

// 16-byte global loads of consecutive elements (the back-substitution's columns)
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
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

// Shared-memory layout of one knot for the formation: Mt[l][r] = M[r][l] with
// M = [A_k | B_k] (n x (n + m)), i.e. row l of Mt is column l of A_k (l < n)
// or of B_k, contiguous in global memory, so it loads coalesced with no
// transpose; rows are NP + 4 elements (a 16-byte multiple), rows n..NP-1 zero.
template <int NP>
__host__ __device__ constexpr uint32_t schur_ldt() { return NP + 4; }

// per-warp elements: Mt (L rows) + d (L) + w (L) + Qi_{k+1} (32) + two pivot
// rows of the fused block-Jacobi inverse (32 each), L = n + m
__host__ __device__ inline uint32_t schur_warp_elems(uint32_t L, uint32_t ldt) {
    return (L * ldt + 2 * ((L + 3) & ~3u) + 96);
}

// Asynchronous copy of one element global -> shared (cp.async, no registers,
// nothing waits until cp_async_wait_all); valid = false writes a zero instead.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T *smem, const T *gmem, bool valid) {
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    const uint32_t bytes = valid ? (uint32_t)sizeof(T) : 0u;
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(s), "l"(gmem), "r"(bytes) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(s), "l"(gmem), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// loads TR consecutive elements starting at an 8-byte-aligned float address
// (pairs) or any double address
template <typename T, int TR>
__device__ __forceinline__ void load_run(const T *p, T (&v)[TR]) {
    if constexpr (sizeof(T) == 4 && TR % 2 == 0) {
#pragma unroll
        for (int t = 0; t < TR; t += 2) {
            const float2 x = *reinterpret_cast<const float2 *>(p + t);
            v[t] = x.x;
            v[t + 1] = x.y;
        }
    } else {
#pragma unroll
        for (int t = 0; t < TR; ++t) v[t] = p[t];
    }
}

// One warp per knot.  The Gram product S_kk = M diag(d) M^T is a 2D register
// tile per lane: lanes form a 4 x 8 grid, lane (rg, cg) owns rows
// rg TR .. rg TR + TR - 1 and columns cg TC .. cg TC + TC - 1 of the NP x NP
// product (TR = NP / 4, TC = NP / 8), and each column l of M adds a rank-1
// term: TR + TC shared-memory loads for TR TC FMAs.  Every element is rounded
// as sum_l fma(M[i][l] d_l, M[j][l], .) in ascending l, then + Qi_{k+1} on the
// diagonal, and symmetrised as 0.5 (S + S^T) through shared memory.  With
// PINV the warp then inverts the symmetrised S_kk (rotating Gauss-Jordan, the
// block-Jacobi builder's own routine and rounding) and writes the compact
// block-Jacobi Phi^-1, so the preconditioner is built with S and never
// re-read.
template <typename T, int NP, int W, bool PINV>
__global__ void __launch_bounds__(W * 32)
    form_schur_kernel(const T *__restrict__ A, const T *__restrict__ B, const T *__restrict__ Qd,
                      const T *__restrict__ Rd, const T *__restrict__ q, const T *__restrict__ r,
                      const T *__restrict__ c, uint32_t n, uint32_t m, uint32_t N, T *__restrict__ S,
                      T *__restrict__ gamma, T *__restrict__ Pinv) {
    constexpr int TR = NP / 4, TC = NP / 8;
    constexpr uint32_t ldt = schur_ldt<NP>();
    extern __shared__ __align__(16) unsigned char schur_smem[];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t k = blockIdx.x * W + warp;
    if (k >= N) return;  // warp-uniform; no CTA barrier below
    const uint32_t L = n + m, L4 = (L + 3) & ~3u;
    T *Mt = reinterpret_cast<T *>(schur_smem) + (size_t)warp * schur_warp_elems(L, ldt);
    T *dv = Mt + L * ldt, *wv = dv + L4, *qn = wv + L4, *s_raw = qn + 32, *s_t = s_raw + 32;
    const T *Ak = A + (size_t)k * n * n, *Bk = B + (size_t)k * n * m;
    // every column in flight at once (cp.async); rows n..NP-1 zero-filled
    for (uint32_t l = 0; l < L; ++l) {
        const T *src = l < n ? Ak + (size_t)l * n : Bk + (size_t)(l - n) * n;
        if (lane < (uint32_t)NP) cp_async_elem(Mt + l * ldt + lane, src + (lane < n ? lane : 0u), lane < n);
    }
    if (lane < n) {
        dv[lane] = T(1) / Qd[(size_t)k * n + lane];
        wv[lane] = q[(size_t)k * n + lane];
        qn[lane] = T(1) / Qd[(size_t)(k + 1) * n + lane];
    }
    if (lane < m) {
        dv[n + lane] = T(1) / Rd[(size_t)k * m + lane];
        wv[n + lane] = r[(size_t)k * m + lane];
    }
    cp_async_wait_all();
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
            Sk[e] = (k > 0) ? -dv[col] * Mt[col * ldt + row] : T(0);
            if (k > 0) Sup[e] = -dv[row] * Mt[row * ldt + col];
            if (k + 1 == N) Sk[2 * (size_t)n * n + e] = T(0);
        }
        // gamma_k = -(c_k + M diag(d) w - Qi_{k+1} q_{k+1})
        T g = T(0);
        for (uint32_t l = 0; l < L; ++l) g += Mt[l * ldt + row] * (dv[l] * wv[l]);
        gamma[(size_t)k * n + row] = -(c[(size_t)k * n + row] + g - qn[row] * q[(size_t)(k + 1) * n + row]);
    }
    // the Gram tile
    const uint32_t rg = lane >> 3, cg = lane & 7, r0 = rg * TR, c0 = cg * TC;
    T acc[TR][TC];
#pragma unroll
    for (int t = 0; t < TR; ++t)
#pragma unroll
        for (int u = 0; u < TC; ++u) acc[t][u] = T(0);
#pragma unroll 2
    for (uint32_t l = 0; l < L; ++l) {
        T a[TR], b[TC];
        load_run<T, TR>(Mt + l * ldt + r0, a);
#pragma unroll
        for (int u = 0; u < TC; ++u) b[u] = Mt[l * ldt + c0 + u];
        const T d = dv[l];
#pragma unroll
        for (int t = 0; t < TR; ++t) {
            const T ad = a[t] * d;
#pragma unroll
            for (int u = 0; u < TC; ++u) acc[t][u] += ad * b[u];
        }
    }
    __syncwarp();  // every lane is done with Mt: it now holds S_kk, row stride NP + 1
    constexpr uint32_t xs = NP + 1;
    T *X = Mt;
#pragma unroll
    for (int t = 0; t < TR; ++t)
#pragma unroll
        for (int u = 0; u < TC; ++u) {
            const uint32_t i = r0 + t, j = c0 + u;
            if (i < n && j < n) X[i * xs + j] = (i == j) ? acc[t][u] + qn[i] : acc[t][u];
        }
    __syncwarp();
    // block 1: S_kk symmetrised
    if (lane < n) {
        const uint32_t row = lane;
        for (uint32_t col = 0; col < n; ++col)
            Sk[n * n + col * n + row] = T(0.5) * (X[row * xs + col] + X[col * xs + row]);
    }
    if constexpr (PINV) {
        // lane r: row r of the symmetrised S_kk (the values just written),
        // identity beyond n
        T a[NP];
#pragma unroll
        for (int cc = 0; cc < NP; ++cc)
            a[cc] = (lane < n && (uint32_t)cc < n) ? T(0.5) * (X[lane * xs + cc] + X[cc * xs + lane])
                                                   : ((uint32_t)cc == lane ? T(1) : T(0));
        gbdpcg::gj_rotate<T, NP>(a, s_raw, s_t, lane);  // ends with a warp sync: X is free
        if (lane < n) {
#pragma unroll
            for (int cc = 0; cc < NP; ++cc)
                if ((uint32_t)cc < n) X[lane * xs + cc] = a[cc];
        }
        __syncwarp();
        if (lane < n) {  // symmetrised, compact n^2 per knot, column-major
            T *Pk = Pinv + (size_t)k * n * n;
            for (uint32_t col = 0; col < n; ++col)
                Pk[col * n + lane] = T(0.5) * (X[lane * xs + col] + X[col * xs + lane]);
        }
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
               uint32_t m, uint32_t N, T *S, T *gamma, T *Pinv, cudaStream_t st) {
    const void *p[] = {A, B, Qd, Rd, q, r, c, S, gamma};
    int rc = check(p, 9, n, m, N);
    if (rc) return rc;
    constexpr int W = kkt_warps<T>();
    auto go = [&](auto np) -> int {
        constexpr int NP = decltype(np)::value;
        const size_t smem = (size_t)W * schur_warp_elems(n + m, schur_ldt<NP>()) * sizeof(T);
        auto launch = [&](auto kern) -> int {
            cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) {
                gbdpcg::set_last_error(std::string("form_schur: ") + cudaGetErrorString(e));
                return GBDPCG_ERR_CUDA;
            }
            kern<<<(N + W - 1) / W, W * 32, smem, st>>>(A, B, Qd, Rd, q, r, c, n, m, N, S, gamma, Pinv);
            return launched("form_schur");
        };
        return Pinv ? launch(form_schur_kernel<T, NP, W, true>) : launch(form_schur_kernel<T, NP, W, false>);
    };
    if (n <= 8) return go(std::integral_constant<int, 8>());
    if (n <= 16) return go(std::integral_constant<int, 16>());
    if (n <= 24) return go(std::integral_constant<int, 24>());
    return go(std::integral_constant<int, 32>());
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
    return form_schur<float>(d_A, d_B, d_Qd, d_Rd, d_q, d_r, d_c, n, m, N, d_S, d_gamma, nullptr,
                             (cudaStream_t)stream);
}
int gbdpcg_form_schur_f64(const double *d_A, const double *d_B, const double *d_Qd, const double *d_Rd,
                          const double *d_q, const double *d_r, const double *d_c, uint32_t n, uint32_t m, uint32_t N,
                          double *d_S, double *d_gamma, gbdpcg_stream_t stream) {
    return form_schur<double>(d_A, d_B, d_Qd, d_Rd, d_q, d_r, d_c, n, m, N, d_S, d_gamma, nullptr,
                              (cudaStream_t)stream);
}
int gbdpcg_form_schur_pinv_f32(const float *d_A, const float *d_B, const float *d_Qd, const float *d_Rd,
                               const float *d_q, const float *d_r, const float *d_c, uint32_t n, uint32_t m,
                               uint32_t N, float *d_S, float *d_gamma, float *d_Pinv, gbdpcg_stream_t stream) {
    if (!d_Pinv) {
        gbdpcg::set_last_error("NULL pointer");
        return GBDPCG_ERR_INVALID_ARGUMENT;
    }
    return form_schur<float>(d_A, d_B, d_Qd, d_Rd, d_q, d_r, d_c, n, m, N, d_S, d_gamma, d_Pinv,
                             (cudaStream_t)stream);
}
int gbdpcg_form_schur_pinv_f64(const double *d_A, const double *d_B, const double *d_Qd, const double *d_Rd,
                               const double *d_q, const double *d_r, const double *d_c, uint32_t n, uint32_t m,
                               uint32_t N, double *d_S, double *d_gamma, double *d_Pinv, gbdpcg_stream_t stream) {
    if (!d_Pinv) {
        gbdpcg::set_last_error("NULL pointer");
        return GBDPCG_ERR_INVALID_ARGUMENT;
    }
    return form_schur<double>(d_A, d_B, d_Qd, d_Rd, d_q, d_r, d_c, n, m, N, d_S, d_gamma, d_Pinv,
                              (cudaStream_t)stream);
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
