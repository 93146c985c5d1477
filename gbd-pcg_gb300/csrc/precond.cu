// Block-Jacobi preconditioner Phi^-1 = blockdiag(S_kk^-1), built on the GPU.
//
// The reference takes Phi^-1 from its caller (include/interface.cuh:24-32) and
// its documented pcg_solve(S, gamma, lambda, ...) (README.md:42) has no Phi^-1
// argument; this kernel supplies it.  One warp per knot: the diagonal block
// S_kk (the middle block of the cbtd block row) is factored S_kk = L L^T by a
// warp-parallel Cholesky in shared memory, then lane j solves L L^T x = e_j for
// column j of the inverse, and the result is symmetrised and written either as
// a cbtd block row [0 | S_kk^-1 | 0] or compactly (n^2 per knot, column-major).
// Work item = (system, knot) over a batch; the knot-prefix array maps a warp to
// its system.  TI: element type of S, TO: of Phi^-1, CT: arithmetic (double
// S with float Phi^-1 serves the FP32-inner refinement).
#include <cuda_runtime.h>
#include <stdint.h>

#include "pcg_types.h"

namespace gbdpcg {

constexpr int kPrecWarps = 2;  // knots per CTA
constexpr int kPrecMaxN = 32;

template <typename TI, typename TO, typename CT>
__global__ void __launch_bounds__(kPrecWarps * 32)
    block_jacobi_kernel(const SysDesc *__restrict__ descs, const uint64_t *__restrict__ knot_prefix,
                        uint32_t nsys, uint64_t total_knots, int tri_layout) {
    __shared__ CT sL[kPrecWarps][kPrecMaxN * (kPrecMaxN + 1)];
    __shared__ CT sX[kPrecWarps][kPrecMaxN * (kPrecMaxN + 1)];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t gk = (uint64_t)blockIdx.x * kPrecWarps + warp;
    if (gk >= total_knots) return;
    // system owning global knot gk: last s with knot_prefix[s] <= gk
    uint32_t lo = 0, hi = nsys;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (knot_prefix[mid] <= gk) lo = mid; else hi = mid;
    }
    const SysDesc d = descs[lo];
    const uint32_t n = d.n, k = (uint32_t)(gk - knot_prefix[lo]);
    if (n == 0 || n > (uint32_t)kPrecMaxN) return;
    const uint32_t ld = kPrecMaxN + 1;  // padded row stride, conflict-free columns
    CT *L = sL[warp];
    CT *X = sX[warp];
    const TI *Sk = static_cast<const TI *>(d.S) + (size_t)k * 3 * n * n + (size_t)n * n;
    // L <- S_kk (row-major, lower triangle used); S_kk column-major: (r, c) at c*n + r
    for (uint32_t e = lane; e < n * n; e += 32) {
        const uint32_t c = e / n, r = e - c * n;
        L[r * ld + c] = CT(Sk[e]);
    }
    __syncwarp();
    // right-looking Cholesky, lane r updates row r
    for (uint32_t j = 0; j < n; ++j) {
        const CT djj = L[j * ld + j];
        const CT ljj = djj > CT(0) ? sqrt(djj) : CT(1);  // non-SPD block: leave it unscaled
        __syncwarp();
        if (lane == j) L[j * ld + j] = ljj;
        if (lane > j && lane < n) L[lane * ld + j] = L[lane * ld + j] / ljj;
        __syncwarp();
        if (lane > j && lane < n) {
            const CT lrj = L[lane * ld + j];
            for (uint32_t c = j + 1; c <= lane; ++c) L[lane * ld + c] -= lrj * L[c * ld + j];
        }
        __syncwarp();
    }
    // lane j: x = L^-T L^-1 e_j  -> column j of X (stored X[j][r])
    if (lane < n) {
        const uint32_t j = lane;
        CT *x = X + j * ld;
        for (uint32_t r = 0; r < n; ++r) {
            CT s = (r == j) ? CT(1) : CT(0);
            for (uint32_t c = 0; c < r; ++c) s -= L[r * ld + c] * x[c];
            x[r] = s / L[r * ld + r];
        }
        for (int r = (int)n - 1; r >= 0; --r) {
            CT s = x[r];
            for (uint32_t c = r + 1; c < n; ++c) s -= L[c * ld + r] * x[c];
            x[r] = s / L[r * ld + r];
        }
    }
    __syncwarp();
    TO *out = static_cast<TO *>(const_cast<void *>(d.P));
    if (tri_layout) {
        TO *row = out + (size_t)k * 3 * n * n;
        for (uint32_t e = lane; e < 3 * n * n; e += 32) {
            const uint32_t b = e / (n * n), w = e - b * n * n;
            const uint32_t c = w / n, r = w - c * n;
            row[e] = (b == 1) ? TO(CT(0.5) * (X[c * ld + r] + X[r * ld + c])) : TO(0);
        }
    } else {
        TO *blk = out + (size_t)k * n * n;
        for (uint32_t e = lane; e < n * n; e += 32) {
            const uint32_t c = e / n, r = e - c * n;
            blk[e] = TO(CT(0.5) * (X[c * ld + r] + X[r * ld + c]));
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
