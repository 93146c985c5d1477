// Plain one-system-per-launch PCG with runtime sizes.
//
// The same structure as the reference kernel pcg<T, n, N>
// (include/pcg.cuh:54-218), without its compile-time sizes: a cooperative
// launch of one CTA per knot (include/interface.cuh:134), the knot's S and
// Phi^-1 block rows in shared memory, halo vectors r and p published through
// global memory between grid-wide barriers, and per-knot dot partials reduced
// redundantly by every CTA.  Arithmetic order: per row a sequential fused
// multiply-add over the present block columns (include/utils.cuh:46-85); dots
// as rounded products summed by the halving fold (len -> ceil(len/2),
// x[i] += x[i + ceil(len/2)]).  On the same inputs it reproduces the CPU
// restatement of the reference bit for bit.
//
// It is the library's "plain" algorithm: the baseline the batched cluster
// solver is measured against, and the path for blocks larger than 32.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "pcg_types.h"

namespace gbdpcg {
namespace cgp = cooperative_groups;

template <typename T>
__device__ __forceinline__ T plain_fma(T a, T b, T c);
template <>
__device__ __forceinline__ float plain_fma<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <>
__device__ __forceinline__ double plain_fma<double>(double a, double b, double c) { return __fma_rn(a, b, c); }

template <typename T>
__device__ void plain_fold(T *x, uint32_t len) {
    while (len > 1) {
        const uint32_t h = len / 2, up = len - h;
        for (uint32_t i = threadIdx.x; i < h; i += blockDim.x) x[i] = x[i] + x[i + up];
        __syncthreads();
        len = up;
    }
}

// w = [v_{k-1} | v_k | v_{k+1}] from global memory (include/utils.cuh:9-40)
template <typename T>
__device__ void plain_window(T *w, const T *v, uint32_t n, uint32_t N, uint32_t k) {
    for (uint32_t t = threadIdx.x; t < 3 * n; t += blockDim.x) {
        const uint32_t b = t / n;
        const bool present = (b != 0 || k > 0) && (b != 2 || k + 1 < N);
        if (present) w[t] = v[(size_t)(k + b - 1) * n + (t - b * n)];
    }
}

// y = M_k w over the present block columns (include/utils.cuh:46-85)
template <typename T>
__device__ void plain_bdmv(T *y, const T *M, const T *w, uint32_t n, uint32_t N, uint32_t k) {
    const uint32_t c0 = (k == 0) ? n : 0, c1 = (k + 1 == N) ? 2 * n : 3 * n;
    for (uint32_t r = threadIdx.x; r < n; r += blockDim.x) {
        T val = T(0);
        for (uint32_t c = c0; c < c1; ++c) val = plain_fma(M[(size_t)n * c + r], w[c], val);
        y[r] = val;
    }
}

template <typename T>
__device__ T plain_dot(T *scratch, const T *a, const T *b, uint32_t n) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const T prod = a[i] * b[i];
        scratch[i] = prod;
    }
    __syncthreads();
    plain_fold(scratch, n);
    return scratch[0];
}

template <typename T>
__device__ T plain_reduce(T *scratch, const T *d_part, uint32_t N) {
    for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) scratch[i] = d_part[i];
    __syncthreads();
    plain_fold(scratch, N);
    return scratch[0];
}

// Shared memory: 6n^2 + 9n + max(n, N) elements (S, Phi^-1, gamma, 3n window,
// upsilon, lambda, r, p, z, fold scratch).
template <typename T>
__global__ void pcg_plain_kernel(const T *__restrict__ S, const T *__restrict__ P,
                                 const T *__restrict__ gamma, const T *__restrict__ lambda0,
                                 T *__restrict__ lambda, T *d_r, T *d_p, T *d_part1, T *d_part2,
                                 uint32_t n, uint32_t N, uint32_t max_iter, double tol_d,
                                 uint32_t flags, SysResult *result) {
    cgp::grid_group grid = cgp::this_grid();
    const uint32_t k = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    const size_t n2 = (size_t)n * n, off = (size_t)k * n;
    extern __shared__ __align__(16) unsigned char plain_smem[];
    T *sS = reinterpret_cast<T *>(plain_smem);
    T *sP = sS + 3 * n2;
    T *sg = sP + 3 * n2;
    T *sw = sg + n;       // 3n window
    T *sy = sw + 3 * n;   // n
    T *sl = sy + n;       // own lambda
    T *sr = sl + n;       // own r
    T *sp = sr + n;       // own p
    T *sz = sp + n;       // own z
    T *scr = sz + n;      // max(n, N) fold scratch
    const bool relres = (flags & SYS_EXIT_RELRES) != 0;
    const T tol = T(tol_d);

    for (uint32_t e = tid; e < 3 * n2; e += nt) {
        const uint32_t b = e / n2;
        const bool present = (b != 0 || k > 0) && (b != 2 || k + 1 < N);
        sS[e] = present ? S[(size_t)k * 3 * n2 + e] : T(0);
        sP[e] = present ? P[(size_t)k * 3 * n2 + e] : T(0);
    }
    for (uint32_t e = tid; e < n; e += nt) {
        sg[e] = gamma[off + e];
        sl[e] = (flags & SYS_LAMBDA0_ZERO) ? T(0) : lambda0[off + e];
    }
    // r = gamma - S lambda
    const T *lam_src = (flags & SYS_LAMBDA0_ZERO) ? nullptr : lambda0;
    if (lam_src) plain_window(sw, lam_src, n, N, k);
    else
        for (uint32_t t = tid; t < 3 * n; t += nt) sw[t] = T(0);
    __syncthreads();
    plain_bdmv(sy, sS, sw, n, N, k);
    __syncthreads();
    for (uint32_t e = tid; e < n; e += nt) {
        sr[e] = sg[e] - sy[e];
        d_r[off + e] = sr[e];
    }
    grid.sync();
    // z = Phi^-1 r, p = z, eta = r.z
    plain_window(sw, d_r, n, N, k);
    __syncthreads();
    plain_bdmv(sz, sP, sw, n, N, k);
    __syncthreads();
    for (uint32_t e = tid; e < n; e += nt) {
        sp[e] = sz[e];
        d_p[off + e] = sp[e];
    }
    T part = plain_dot(scr, sr, sz, n);
    if (tid == 0) d_part2[k] = part;
    T gpart = T(0);
    if (relres) {
        __syncthreads();
        gpart = plain_dot(scr, sg, sg, n);
        if (tid == 0) d_part1[k] = gpart;
    }
    grid.sync();
    T eta = plain_reduce(scr, d_part2, N);
    T gg = T(0);
    if (relres) {
        __syncthreads();
        gg = plain_reduce(scr, d_part1, N);
    }
    __syncthreads();
    const T thr = T(tol_d * tol_d * (double)gg);

    uint32_t iter = 0;
    int32_t status = ST_MAX_ITER;
    T eta_new = T(0), rr = T(0);
    grid.sync();
    for (iter = 0; iter < max_iter;) {
        // upsilon = S p; alpha = eta / p.upsilon
        plain_window(sw, d_p, n, N, k);
        __syncthreads();
        plain_bdmv(sy, sS, sw, n, N, k);
        __syncthreads();
        part = plain_dot(scr, sp, sy, n);
        if (tid == 0) d_part1[k] = part;
        grid.sync();
        const T pap = plain_reduce(scr, d_part1, N);
        __syncthreads();
        const T alpha = (pap == T(0)) ? T(0) : eta / pap;
        for (uint32_t e = tid; e < n; e += nt) {
            sl[e] = plain_fma(alpha, sp[e], sl[e]);
            sr[e] = plain_fma(-alpha, sy[e], sr[e]);
            d_r[off + e] = sr[e];
        }
        grid.sync();
        // z = Phi^-1 r; eta_new = r.z
        plain_window(sw, d_r, n, N, k);
        __syncthreads();
        plain_bdmv(sz, sP, sw, n, N, k);
        __syncthreads();
        part = plain_dot(scr, sr, sz, n);
        if (tid == 0) d_part2[k] = part;
        if (relres) {
            __syncthreads();
            const T rpart = plain_dot(scr, sr, sr, n);
            if (tid == 0) d_part1[k] = rpart;
        }
        grid.sync();
        eta_new = plain_reduce(scr, d_part2, N);
        if (relres) {
            __syncthreads();
            rr = plain_reduce(scr, d_part1, N);
        }
        __syncthreads();
        ++iter;
        if (!isfinite(eta_new) || !isfinite(pap)) { status = ST_BREAKDOWN; break; }
        if (relres ? (rr <= thr) : (fabs(eta_new) < tol)) { status = ST_CONVERGED; break; }
        const T beta = eta_new / eta;
        eta = eta_new;
        for (uint32_t e = tid; e < n; e += nt) {
            sp[e] = plain_fma(beta, sp[e], sz[e]);
            d_p[off + e] = sp[e];
        }
        grid.sync();
    }
    for (uint32_t e = tid; e < n; e += nt) lambda[off + e] = sl[e];
    if (k == 0 && tid == 0) {
        SysResult res;
        res.iters = iter;
        res.status = status;
        res.eta = (double)eta_new;
        res.rr = relres ? (double)rr : -1.0;
        res.gg = (double)gg;
        res.outer = 0;
        res.pad = 0;
        *result = res;
    }
}

template __global__ void pcg_plain_kernel<float>(const float *, const float *, const float *,
                                                 const float *, float *, float *, float *, float *,
                                                 float *, uint32_t, uint32_t, uint32_t, double,
                                                 uint32_t, SysResult *);
template __global__ void pcg_plain_kernel<double>(const double *, const double *, const double *,
                                                  const double *, double *, double *, double *,
                                                  double *, double *, uint32_t, uint32_t, uint32_t,
                                                  double, uint32_t, SysResult *);

const void *plain_kernel_ptr(bool f64) {
    return f64 ? (const void *)pcg_plain_kernel<double> : (const void *)pcg_plain_kernel<float>;
}

size_t plain_smem_bytes(bool f64, uint32_t n, uint32_t N) {
    const size_t mx = n > N ? n : N;
    return ((size_t)6 * n * n + 9 * n + mx) * (f64 ? 8 : 4);
}

}  // namespace gbdpcg
