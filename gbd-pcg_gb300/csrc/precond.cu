// Block-Jacobi preconditioner Phi^-1 = blockdiag(S_kk^-1), built on the GPU.
//
// The reference takes Phi^-1 from its caller (include/interface.cuh:24-32) and
// its documented pcg_solve(S, gamma, lambda, ...) (README.md:42) has no Phi^-1
// argument; this kernel supplies it.  One warp per knot: lane r holds row r of
// the diagonal block S_kk (the middle block of the cbtd block row) in
// registers, padded with the identity to NP x NP (NP in {8, 12, 16, 24, 32},
// the smallest that holds n), and the warp inverts it by Gauss-Jordan
// elimination without pivoting (S_kk is symmetric positive definite) in the
// rotating form: step j pivots on row j and on the row's first register; every
// row then shifts one column to the left and the column of the inverse being
// formed enters at the right, so all register indices are compile-time
// constants while the step loop stays rolled, and after NP steps the columns
// are back in order.  The pivot row goes through shared memory: lane j stores
// it, lane c scales its element c, and every lane reads the scaled row back
// with 16-byte broadcast loads.  A shared-memory transpose symmetrises the
// inverse, written either as a cbtd block row [0 | S_kk^-1 | 0] or compactly
// (n^2 per knot, column-major), column by column.  Work item = (system, knot)
// over a batch; the knot-prefix array maps a warp to its system.  TI: element
// type of S, TO: of Phi^-1, CT: arithmetic (double S with float Phi^-1 serves
// the FP32-inner refinement).
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "gauss_jordan.cuh"
#include "pcg_types.h"

namespace gbdpcg {

constexpr int kPrecWarps = 4;  // knots per CTA
constexpr int kPrecMaxN = 32;

template <typename TI, typename TO, typename CT, int NP>
__device__ __forceinline__ void invert_knot(const TI *Sk, TO *row, uint32_t n, int tri_layout, CT *s_raw, CT *s_t,
                                            CT *X, uint32_t lane) {
    // lane r: row r of S_kk (column-major: (r, c) at c*n + r; coalesced over
    // lanes), identity beyond n
    CT a[NP];
#pragma unroll
    for (int c = 0; c < NP; ++c)
        a[c] = (lane < n && (uint32_t)c < n) ? CT(Sk[(size_t)c * n + lane]) : ((uint32_t)c == lane ? CT(1) : CT(0));
    gj_rotate<CT, NP>(a, s_raw, s_t, lane);
    // symmetrise through a shared-memory transpose: X[r][c] = inverse (r, c)
    const uint32_t ld = kPrecMaxN + 1;
    if (lane < n) {
#pragma unroll
        for (int c = 0; c < NP; ++c)
            if ((uint32_t)c < n) X[lane * ld + c] = a[c];
    }
    __syncwarp();
    // column by column, lane = row: coalesced stores, no index division
    const uint32_t nn = n * n, mid = tri_layout ? nn : 0;
    if (lane < n) {
        const uint32_t r = lane;
        for (uint32_t c = 0; c < n; ++c) {
            row[mid + c * n + r] = TO(CT(0.5) * (X[r * ld + c] + X[c * ld + r]));
            if (tri_layout) {
                row[c * n + r] = TO(0);
                row[2 * nn + c * n + r] = TO(0);
            }
        }
    }
}

template <typename TI, typename TO, typename CT>
__global__ void __launch_bounds__(kPrecWarps * 32)
    block_jacobi_kernel(const SysDesc *__restrict__ descs, const uint64_t *__restrict__ knot_prefix,
                        uint32_t nsys, uint64_t total_knots, int tri_layout, const SysDesc one) {
    __shared__ CT sX[kPrecWarps][kPrecMaxN * (kPrecMaxN + 1)];
    __shared__ __align__(16) CT sR[kPrecWarps][2][kPrecMaxN];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t gk = (uint64_t)blockIdx.x * kPrecWarps + warp;
    if (gk >= total_knots) return;  // warp-uniform; no CTA-wide barrier below
    // system owning global knot gk: last s with knot_prefix[s] <= gk (or the
    // one system passed by value)
    uint32_t lo = 0, hi = nsys;
    if (descs) {
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) / 2;
            if (knot_prefix[mid] <= gk) lo = mid; else hi = mid;
        }
    }
    const SysDesc d = descs ? descs[lo] : one;
    const uint32_t n = d.n, k = (uint32_t)(descs ? gk - knot_prefix[lo] : gk);
    if (n == 0 || n > (uint32_t)kPrecMaxN) return;
    const TI *Sk = static_cast<const TI *>(d.S) + (size_t)k * 3 * n * n + (size_t)n * n;
    TO *row = static_cast<TO *>(const_cast<void *>(d.P)) + (size_t)k * (tri_layout ? 3 : 1) * n * n;
    CT *s_raw = sR[warp][0], *s_t = sR[warp][1], *X = sX[warp];
    if (n <= 8) invert_knot<TI, TO, CT, 8>(Sk, row, n, tri_layout, s_raw, s_t, X, lane);
    else if (n <= 12) invert_knot<TI, TO, CT, 12>(Sk, row, n, tri_layout, s_raw, s_t, X, lane);
    else if (n <= 16) invert_knot<TI, TO, CT, 16>(Sk, row, n, tri_layout, s_raw, s_t, X, lane);
    else if (n <= 24) invert_knot<TI, TO, CT, 24>(Sk, row, n, tri_layout, s_raw, s_t, X, lane);
    else invert_knot<TI, TO, CT, 32>(Sk, row, n, tri_layout, s_raw, s_t, X, lane);
}

// kind: 0 float S -> float Phi^-1 (float arithmetic); 1 double -> double;
// 2 double S -> float Phi^-1 (double arithmetic, for the refinement's inner solve)
// d_descs == nullptr: the single system *one (total_knots = its N), passed to
// the kernel by value (no descriptor upload).
cudaError_t launch_block_jacobi(int kind, const SysDesc *d_descs, const uint64_t *d_prefix,
                                uint32_t nsys, uint64_t total_knots, int tri_layout,
                                cudaStream_t stream, const SysDesc *one) {
    if (total_knots == 0) return cudaSuccess;
    SysDesc o;
    if (one) o = *one;
    else memset(&o, 0, sizeof(o));
    const dim3 grid((unsigned)((total_knots + kPrecWarps - 1) / kPrecWarps)), block(kPrecWarps * 32);
    if (kind == 1)
        block_jacobi_kernel<double, double, double><<<grid, block, 0, stream>>>(
            d_descs, d_prefix, nsys, total_knots, tri_layout, o);
    else if (kind == 2)
        block_jacobi_kernel<double, float, double><<<grid, block, 0, stream>>>(
            d_descs, d_prefix, nsys, total_knots, tri_layout, o);
    else
        block_jacobi_kernel<float, float, float><<<grid, block, 0, stream>>>(
            d_descs, d_prefix, nsys, total_knots, tri_layout, o);
    return cudaGetLastError();
}

}  // namespace gbdpcg
