// Block-Jacobi preconditioner Phi^-1 = blockdiag(S_kk^-1), built on the GPU.
//
// The reference takes Phi^-1 from its caller (include/interface.cuh:24-32) and
// its documented pcg_solve(S, gamma, lambda, ...) (README.md:42) has no Phi^-1
// argument; this kernel supplies it.  One warp per knot: lane r holds row r of
// the diagonal block S_kk (the middle block of the cbtd block row) in
// registers, and the warp inverts the block in place by Gauss-Jordan
// elimination without pivoting (S_kk is symmetric positive definite): at step
// j lane j's row is the pivot row, broadcast element by element with warp
// shuffles, and every lane updates its own row.  No shared-memory round trip
// is on the critical path; a final shared-memory transpose symmetrises the
// inverse, which is written either as a cbtd block row [0 | S_kk^-1 | 0] or
// compactly (n^2 per knot, column-major).  Work item = (system, knot) over a
// batch; the knot-prefix array maps a warp to its system.  TI: element type
// of S, TO: of Phi^-1, CT: arithmetic (double S with float Phi^-1 serves the
// FP32-inner refinement).
#include <cuda_runtime.h>
#include <stdint.h>

#include "pcg_types.h"

namespace gbdpcg {

constexpr int kPrecWarps = 4;  // knots per CTA
constexpr int kPrecMaxN = 32;

template <typename TI, typename TO, typename CT>
__global__ void __launch_bounds__(kPrecWarps * 32)
    block_jacobi_kernel(const SysDesc *__restrict__ descs, const uint64_t *__restrict__ knot_prefix,
                        uint32_t nsys, uint64_t total_knots, int tri_layout) {
    __shared__ CT sX[kPrecWarps][kPrecMaxN * (kPrecMaxN + 1)];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t gk = (uint64_t)blockIdx.x * kPrecWarps + warp;
    if (gk >= total_knots) return;  // warp-uniform; no CTA-wide barrier below
    // system owning global knot gk: last s with knot_prefix[s] <= gk
    uint32_t lo = 0, hi = nsys;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (knot_prefix[mid] <= gk) lo = mid; else hi = mid;
    }
    const SysDesc d = descs[lo];
    const uint32_t n = d.n, k = (uint32_t)(gk - knot_prefix[lo]);
    if (n == 0 || n > (uint32_t)kPrecMaxN) return;
    const TI *Sk = static_cast<const TI *>(d.S) + (size_t)k * 3 * n * n + (size_t)n * n;
    // lane r: row r of S_kk (column-major: (r, c) at c*n + r; coalesced over lanes)
    CT a[kPrecMaxN];
#pragma unroll
    for (int c = 0; c < kPrecMaxN; ++c) a[c] = (lane < n && (uint32_t)c < n) ? CT(Sk[(size_t)c * n + lane]) : CT(0);
    // in-place Gauss-Jordan: after step j, column j holds the inverse's column
#pragma unroll
    for (int j = 0; j < kPrecMaxN; ++j) {
        if ((uint32_t)j < n) {  // warp-uniform
            CT piv = __shfl_sync(0xffffffffu, a[j], j);
            if (piv == CT(0)) piv = CT(1);  // singular block: leave that column unscaled
            const CT inv = CT(1) / piv;
            const CT g = a[j] * inv;  // lane j: 1
#pragma unroll
            for (int c = 0; c < kPrecMaxN; ++c) {
                if ((uint32_t)c < n) {
                    const CT rj = __shfl_sync(0xffffffffu, a[c], j);  // pivot row, before this step
                    if (c == j) a[c] = ((int)lane == j) ? inv : -g;
                    else a[c] = ((int)lane == j) ? rj * inv : a[c] - g * rj;
                }
            }
        }
    }
    // symmetrise through a shared-memory transpose: X[r][c] = inverse (r, c)
    CT *X = sX[warp];
    const uint32_t ld = kPrecMaxN + 1;
    if (lane < n) {
#pragma unroll
        for (int c = 0; c < kPrecMaxN; ++c)
            if ((uint32_t)c < n) X[lane * ld + c] = a[c];
    }
    __syncwarp();
    TO *out = static_cast<TO *>(const_cast<void *>(d.P));
    if (tri_layout) {
        TO *row = out + (size_t)k * 3 * n * n;
        for (uint32_t e = lane; e < 3 * n * n; e += 32) {
            const uint32_t b = e / (n * n), w = e - b * n * n;
            const uint32_t c = w / n, r = w - c * n;
            row[e] = (b == 1) ? TO(CT(0.5) * (X[r * ld + c] + X[c * ld + r])) : TO(0);
        }
    } else {
        TO *blk = out + (size_t)k * n * n;
        for (uint32_t e = lane; e < n * n; e += 32) {
            const uint32_t c = e / n, r = e - c * n;
            blk[e] = TO(CT(0.5) * (X[r * ld + c] + X[c * ld + r]));
        }
    }
}

// kind: 0 float S -> float Phi^-1 (float arithmetic); 1 double -> double;
// 2 double S -> float Phi^-1 (double arithmetic, for the refinement's inner solve)
cudaError_t launch_block_jacobi(int kind, const SysDesc *d_descs, const uint64_t *d_prefix,
                                uint32_t nsys, uint64_t total_knots, int tri_layout,
                                cudaStream_t stream) {
    if (total_knots == 0) return cudaSuccess;
    const dim3 grid((unsigned)((total_knots + kPrecWarps - 1) / kPrecWarps)), block(kPrecWarps * 32);
    if (kind == 1)
        block_jacobi_kernel<double, double, double><<<grid, block, 0, stream>>>(
            d_descs, d_prefix, nsys, total_knots, tri_layout);
    else if (kind == 2)
        block_jacobi_kernel<double, float, double><<<grid, block, 0, stream>>>(
            d_descs, d_prefix, nsys, total_knots, tri_layout);
    else
        block_jacobi_kernel<float, float, float><<<grid, block, 0, stream>>>(
            d_descs, d_prefix, nsys, total_knots, tri_layout);
    return cudaGetLastError();
}

}  // namespace gbdpcg
