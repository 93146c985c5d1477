// Persistent thread-block-cluster PCG kernel for block-tridiagonal
// Schur-complement systems (the hot path of Sdevaud/GBD-PCG,
// include/pcg.cuh:54-218), written for sm_103a.
//
// Mapping
//   * One cluster of C CTAs solves one system at a time and then pulls the next
//     system from a device work queue (an atomic counter over a host-sorted,
//     longest-first list).  C comes from the launch's cluster dimension.
//   * CTA `rank` owns the contiguous knots [kb, ke), kb = rank*K, K = ceil(N/C).
//   * Thread t of a CTA owns RPT consecutive matrix rows (RPT = 2 only for even
//     n, so both rows lie in one knot and share every vector load).  The rows
//     of S (3 blocks) and of Phi^-1 (1 or 3 blocks) are held for the whole
//     solve on chip; ST selects where: 0 both in registers, 1 S in registers
//     and Phi^-1 in shared memory, 2 both in shared memory, 3 hybrid (two S
//     blocks in registers, the third and Phi^-1 in shared memory), 4 tensor
//     memory (the diagonal S block in registers, the others and Phi^-1 in the
//     SM's TMEM).  Streamed rows (ST 5) are pcg_stream.cuh's kernel.
//   * Vectors p and r live in shared memory with one halo knot on each side.
//     Neighbour CTAs exchange boundary vectors through distributed shared
//     memory (DSMEM): instead of re-publishing p and r after every update (as
//     the reference does through global memory, include/pcg.cuh:175,205, with
//     4 grid.sync per iteration), each CTA pushes its boundary upsilon = S p and
//     z = Phi^-1 r with its next reduction (st.async counted on the
//     receiver's mbarrier), and the receiver applies the same fused
//     multiply-add to its halo copy that the owner applies to the original
//     (r_h -= alpha upsilon_h; p_h = z_h + beta p_h), so the halos stay
//     bit-identical without a cluster barrier.
//   * Dot products: see cluster_allreduce and cluster_allreduce_tx.  All
//     threads of the cluster hold identical alpha, beta and exit decisions.
// Arithmetic follows the reference: alpha = eta / p.Sp, lambda += alpha p,
// r -= alpha Sp, beta = eta'/eta, p = z + beta p as fused multiply-adds; exit
// on |r.z| < tol (include/pcg.cuh:195) or, optionally, on the relative
// recursive residual ||r|| <= tol ||gamma||.  The iteration count includes the
// converging pass, as the reference's does.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "accum.cuh"
#include "tmem.cuh"
#include "pcg_types.h"

namespace gbdpcg {
namespace cg = cooperative_groups;

__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

__host__ __device__ constexpr size_t round_up(size_t x, size_t m) { return (x + m - 1) / m * m; }

// Storage of the matrix rows: ST_REG S and Phi^-1 in registers; ST_REG_S S in
// registers, Phi^-1 in shared memory; ST_SMEM both in shared memory; ST_HYB
// the sub-diagonal and diagonal blocks of S in registers, the super-diagonal
// block of S and Phi^-1 (block-diagonal) in shared memory; ST_TMEM the
// diagonal block of S in registers, its two off-diagonal blocks and Phi^-1
// (block-diagonal) in tensor memory.
// ST_STREAM (pcg_stream.cuh): no storage; the rows are read from global memory
// in every product.
enum : int { ST_REG = 0, ST_REG_S = 1, ST_SMEM = 2, ST_HYB = 3, ST_TMEM = 4, ST_STREAM = 5 };

// A CTA of the tensor-memory storage allocates all of its SM's tensor memory;
// it asks for more than half an SM's shared memory so that no second such CTA
// can share the SM (an allocation would otherwise wait on the first one).
constexpr size_t kTmemExclusiveSmem = 120 * 1024;

// Per-CTA bookkeeping area of the kernels' shared memory (32-byte aligned):
// word 0 the popped work item, word 1 the tensor-memory base address, bytes
// 32..47 the two mbarriers of the transaction-counted reductions, word 12 the
// CTA's reduction-timeout flag.
constexpr size_t kItemBytes = 64;
// Word 13 of the item area: 1 while the next pass of the persistent loop is
// the adjoint pass of a forward + adjoint pair (SYS_FWD_ADJ), which takes the
// same item again instead of popping a new one.
constexpr int kAdjPassWord = 13;

// Reduction slots: [2 buffers][3 values][C ranks x 32 warps]
constexpr int kMaxValues = 3;
__host__ __device__ constexpr size_t slot_stride(uint32_t C) { return (size_t)32 * C; }

// Shared-memory plan of one CTA (every buffer 32-byte aligned).
template <typename T, typename A, int NP, bool PTRI, int ST>
struct SmemPlan {
    static constexpr int NB_P = PTRI ? 3 : 1;
    __host__ __device__ static size_t vec(uint32_t kmax) {
        return round_up((size_t)(kmax + 2) * NP * sizeof(T), 32);
    }
    __host__ __device__ static size_t halo() { return round_up((size_t)2 * NP * sizeof(T), 32); }
    __host__ __device__ static size_t mat_s(uint32_t kmax) {
        return ST == ST_SMEM  ? round_up((size_t)kmax * 3 * NP * NP * sizeof(T), 32)
               : ST == ST_HYB ? round_up((size_t)kmax * NP * NP * sizeof(T), 32)
                              : 0;
    }
    __host__ __device__ static size_t mat_p(uint32_t kmax) {
        return (ST >= ST_REG_S && ST != ST_TMEM) ? round_up((size_t)kmax * NB_P * NP * NP * sizeof(T), 32) : 0;
    }
    __host__ __device__ static size_t slots(uint32_t C) {
        return round_up(2 * kMaxValues * slot_stride(C) * sizeof(A), 32);
    }
    // per-warp scratch of the first reduction stage: [warp][value][lane]
    __host__ __device__ static size_t wscr(uint32_t nwarps) {
        return round_up((size_t)nwarps * kMaxValues * 32 * sizeof(A), 32);
    }
    __host__ __device__ static size_t bytes(uint32_t kmax, uint32_t C, uint32_t nwarps) {
        const size_t b = 2 * vec(kmax) + 2 * halo() + slots(C) + wscr(nwarps) + kItemBytes + mat_s(kmax) + mat_p(kmax);
        return (ST == ST_TMEM && b < kTmemExclusiveSmem) ? kTmemExclusiveSmem : b;
    }
};

// Register budget of one thread: the matrix rows it holds plus a fixed base.
// The launch bound caps the compiler at that budget, so a CTA of up to
// max_threads rows always fits one SM's 64K registers (warps are spread over 4
// sub-partitions of 16K registers: whole groups of 4 warps).
template <typename T, typename A, int NP, bool PTRI, int ST, int RPT>
struct RegBudget {
    static constexpr int words = (int)(sizeof(T) / 4);
    static constexpr int matrix =
        RPT *
        ((ST <= ST_REG_S ? 3 * NP : (ST == ST_HYB ? 2 * NP : (ST == ST_TMEM ? NP : 0))) +
         (ST == ST_REG ? (PTRI ? 3 : 1) * NP : 0)) *
        words;
    // the tensor-memory storage also holds TMEM addresses and the 16 values of a load pair
    static constexpr int base =
        ((sizeof(T) == 8 || sizeof(A) == 8) ? 72 : 56) + 8 * (RPT - 1) * words + (ST == ST_TMEM ? 24 : 0);
    static constexpr int regs = matrix + base > 255 ? 255 : matrix + base;
    static constexpr int max_threads_raw = 65536 / regs / 128 * 128;
    static constexpr int max_threads = max_threads_raw > 1024 ? 1024 : max_threads_raw;
};

// Load NP consecutive shared-memory elements (NP-element aligned) into
// registers with the widest aligned vector loads.
template <typename T, int NP>
__device__ __forceinline__ void lds_row(T (&x)[NP], const T *p) {
    if constexpr (sizeof(T) == 4 && NP % 4 == 0) {
#pragma unroll
        for (int j = 0; j < NP; j += 4) {
            const float4 v = *reinterpret_cast<const float4 *>(p + j);
            x[j] = v.x; x[j + 1] = v.y; x[j + 2] = v.z; x[j + 3] = v.w;
        }
    } else if constexpr (NP % 2 == 0 && sizeof(T) == 4) {
#pragma unroll
        for (int j = 0; j < NP; j += 2) {
            const float2 v = *reinterpret_cast<const float2 *>(p + j);
            x[j] = v.x; x[j + 1] = v.y;
        }
    } else if constexpr (NP % 2 == 0 && sizeof(T) == 8) {
#pragma unroll
        for (int j = 0; j < NP; j += 2) {
            const double2 v = *reinterpret_cast<const double2 *>(p + j);
            x[j] = v.x; x[j + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int j = 0; j < NP; ++j) x[j] = p[j];
    }
}

// Register-tile block-row matvec of RPT rows sharing one window:
// y[q] = sum_b sum_j M[q][b*NP + j] * x[b*NP + j]; one accumulator chain per
// block, summed in block order.
template <typename T, int NP, int NB, int RPT>
__device__ __forceinline__ void reg_matvec(const T (&M)[RPT][NB * NP], const T *x, T (&y)[RPT]) {
    T acc[RPT][NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
        T xv[NP];
        lds_row<T, NP>(xv, x + b * NP);
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
            acc[q][b] = T(0);
#pragma unroll
            for (int j = 0; j < NP; ++j) acc[q][b] = fma_rn(M[q][b * NP + j], xv[j], acc[q][b]);
        }
    }
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
        T s = acc[q][0];
#pragma unroll
        for (int b = 1; b < NB; ++b) s += acc[q][b];
        y[q] = s;
    }
}

// One block of a shared-memory block-row matvec: acc[q][b] = sum_{j<n}
// col[j*R + q] * x[j] for the RPT adjacent rows at col, one FMA chain per row
// in ascending j.  The window x (NP-aligned) is read VW elements at a time
// with vector loads (4 floats when NP is a multiple of 4, else 2); a column
// costs one matrix load (two rows at once when RPT = 2).  Columns j >= n of
// the staged matrix hold no data and are never read.
template <typename T, int NP, int RPT>
__device__ __forceinline__ void smem_col(const T *col, uint32_t R, uint32_t j, T xj, T (&a)[RPT]) {
    if constexpr (RPT == 2 && sizeof(T) == 4) {
        const float2 m = *reinterpret_cast<const float2 *>(col + (size_t)j * R);
        a[0] = fma_rn(m.x, xj, a[0]);
        a[1] = fma_rn(m.y, xj, a[1]);
    } else if constexpr (RPT == 2) {
        const double2 m = *reinterpret_cast<const double2 *>(col + (size_t)j * R);
        a[0] = fma_rn(m.x, xj, a[0]);
        a[1] = fma_rn(m.y, xj, a[1]);
    } else {
        a[0] = fma_rn(col[(size_t)j * R], xj, a[0]);
    }
}

template <typename T, int NP, int RPT, int NBA>
__device__ __forceinline__ void smem_block(const T *col, uint32_t R, const T *x, uint32_t n, T (&acc)[RPT][NBA],
                                           int b) {
    constexpr int VW = (sizeof(T) == 4 && NP % 4 == 0) ? 4 : (NP % 2 == 0 ? 2 : 1);
    T a[RPT];
#pragma unroll
    for (int q = 0; q < RPT; ++q) a[q] = acc[q][b];
    uint32_t j = 0;
#pragma unroll 2
    for (; j + VW <= n; j += VW) {
        T xv[VW];
        if constexpr (VW == 4) {
            const float4 t = *reinterpret_cast<const float4 *>(x + j);
            xv[0] = t.x; xv[1] = t.y; xv[2] = t.z; xv[3] = t.w;
        } else if constexpr (VW == 2 && sizeof(T) == 4) {
            const float2 t = *reinterpret_cast<const float2 *>(x + j);
            xv[0] = t.x; xv[1] = t.y;
        } else if constexpr (VW == 2) {
            const double2 t = *reinterpret_cast<const double2 *>(x + j);
            xv[0] = t.x; xv[1] = t.y;
        } else {
            xv[0] = x[j];
        }
#pragma unroll
        for (int u = 0; u < VW; ++u) smem_col<T, NP, RPT>(col, R, j + u, xv[u], a);
    }
    for (; j < n; ++j) smem_col<T, NP, RPT>(col, R, j, x[j], a);
#pragma unroll
    for (int q = 0; q < RPT; ++q) acc[q][b] = a[q];
}

// Shared-memory matrices are staged column-interleaved across the CTA's rows:
// element (row r of the CTA, column c of the block row) at M[c*R + r], R the
// row stride (even).  A warp then reads consecutive addresses for every column
// (conflict-free 8-byte loads of two adjacent rows), where the cbtd layout
// would put the warp's 4-5 knots on overlapping banks.
//
// Block-row matvec of RPT adjacent rows r..r+RPT-1 over the present blocks
// [b0, b1) of an NB-block row; x points at the window of block 0 (windows are
// NP apart).  Same summation order as reg_matvec (whose padding contributes
// exact zeros).
template <typename T, int NP, int NB, int RPT>
__device__ __forceinline__ void smem_matvec(const T *M, uint32_t R, uint32_t r, int b0, int b1,
                                            const T *x, uint32_t n, T (&y)[RPT]) {
    T acc[RPT][NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
#pragma unroll
        for (int q = 0; q < RPT; ++q) acc[q][b] = T(0);
        if (b >= b0 && b < b1) smem_block<T, NP, RPT>(M + (size_t)b * n * R + r, R, x + b * NP, n, acc, b);
    }
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
        T s = acc[q][0];
#pragma unroll
        for (int b = 1; b < NB; ++b) s += acc[q][b];
        y[q] = s;
    }
}

// Block-row matvec of the hybrid storage: blocks 0 and 1 (sub-diagonal,
// diagonal) from registers, block 2 (super-diagonal, present when b2) from the
// staged matrix M (one n x n block per knot, column-interleaved like
// smem_matvec's).  Same chains and summation order as reg_matvec.
template <typename T, int NP, int RPT>
__device__ __forceinline__ void hyb_matvec(const T (&Mr)[RPT][2 * NP], const T *M, uint32_t R, uint32_t r,
                                           bool b2, const T *x, uint32_t n, T (&y)[RPT]) {
    T acc[RPT][3];
#pragma unroll
    for (int b = 0; b < 2; ++b) {
        T xv[NP];
        lds_row<T, NP>(xv, x + b * NP);
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
            acc[q][b] = T(0);
#pragma unroll
            for (int j = 0; j < NP; ++j) acc[q][b] = fma_rn(Mr[q][b * NP + j], xv[j], acc[q][b]);
        }
    }
#pragma unroll
    for (int q = 0; q < RPT; ++q) acc[q][2] = T(0);
    if (b2) smem_block<T, NP, RPT>(M + r, R, x + 2 * NP, n, acc, 2);
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
        T s = acc[q][0];
        s += acc[q][1];
        s += acc[q][2];
        y[q] = s;
    }
}

// Rounds of loads the tensor-memory staging keeps in flight ahead of its stores.
constexpr int kTmemDepth = 3;

// Columns of one row's block in tensor memory (a multiple of 8: x8 moves).
template <int NP>
__host__ __device__ constexpr int tmem_cols() { return (NP + 7) / 8 * 8; }

// Block-row matvec of the tensor-memory storage, two rows per thread: blocks
// 0 and 2 (sub- and super-diagonal) from this thread's TMEM lane at trow
// (row q: S block 0 at columns 3q NPT, S block 2 at (3q + 1) NPT, Phi^-1 at
// (3q + 2) NPT), block 1 (diagonal) from registers.  Same chains and summation order as reg_matvec.  Warp-wide: every
// thread of the warp calls it (inactive rows read a valid window and discard
// the result).
// Elements [8c, 8c+8) of an NP-element window (those below NP), loaded with
// the widest aligned vectors.
template <int NP>
__device__ __forceinline__ void lds_chunk8(float (&xv)[8], const float *x, int c) {
    constexpr int VW = NP % 4 == 0 ? 4 : (NP % 2 == 0 ? 2 : 1);
#pragma unroll
    for (int u = 0; u < 8; u += VW) {
        if (8 * c + u < NP) {
            if constexpr (VW == 4) {
                const float4 t = *reinterpret_cast<const float4 *>(x + 8 * c + u);
                xv[u] = t.x; xv[u + 1] = t.y; xv[u + 2] = t.z; xv[u + 3] = t.w;
            } else if constexpr (VW == 2) {
                const float2 t = *reinterpret_cast<const float2 *>(x + 8 * c + u);
                xv[u] = t.x; xv[u + 1] = t.y;
            } else {
                xv[u] = x[8 * c + u];
            }
        }
    }
}

template <int NP>
__device__ __forceinline__ void tmem_matvec(const float (&Md)[2][NP], uint32_t trow, const float *x, float (&y)[2]) {
    constexpr int NPT = tmem_cols<NP>();
    __syncwarp();  // tcgen05 loads are warp-wide: the warp is converged here
    float acc[2][3];
#pragma unroll
    for (int bi = 0; bi < 2; ++bi) {
        const int b = 2 * bi;
        acc[0][b] = 0.f;
        acc[1][b] = 0.f;
#pragma unroll
        for (int c = 0; c < NPT / 8; ++c) {
            float m0[8], m1[8], xv[8];
            tmem_ld8x2(trow + (0 * 3 + bi) * NPT + 8 * c, trow + (1 * 3 + bi) * NPT + 8 * c, m0, m1);
            lds_chunk8<NP>(xv, x + b * NP, c);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (8 * c + u < NP) {
                    acc[0][b] = fma_rn(m0[u], xv[u], acc[0][b]);
                    acc[1][b] = fma_rn(m1[u], xv[u], acc[1][b]);
                }
            }
        }
    }
    acc[0][1] = 0.f;
    acc[1][1] = 0.f;
#pragma unroll
    for (int c = 0; c < NPT / 8; ++c) {
        float xv[8];
        lds_chunk8<NP>(xv, x + NP, c);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (8 * c + u < NP) {
                acc[0][1] = fma_rn(Md[0][8 * c + u], xv[u], acc[0][1]);
                acc[1][1] = fma_rn(Md[1][8 * c + u], xv[u], acc[1][1]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        float s = acc[q][0];
        s += acc[q][1];
        s += acc[q][2];
        y[q] = s;
    }
}

// Phi^-1 (block-diagonal) times the centre block of the window, two rows per
// thread, from TMEM columns (3q + 2) NPT.  Same chain as smem_matvec's.
// Warp-wide, like tmem_matvec.
template <int NP>
__device__ __forceinline__ void tmem_pmatvec(uint32_t trow, const float *x, float (&y)[2]) {
    constexpr int NPT = tmem_cols<NP>();
    __syncwarp();
    float a0 = 0.f, a1 = 0.f;
#pragma unroll
    for (int c = 0; c < NPT / 8; ++c) {
        float m0[8], m1[8], xv[8];
        tmem_ld8x2(trow + 2 * NPT + 8 * c, trow + 5 * NPT + 8 * c, m0, m1);
        lds_chunk8<NP>(xv, x + NP, c);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (8 * c + u < NP) {
                a0 = fma_rn(m0[u], xv[u], a0);
                a1 = fma_rn(m1[u], xv[u], a1);
            }
        }
    }
    y[0] = a0;
    y[1] = a1;
}

// Hint the L2 to fetch [p, p + bytes) from HBM now (cp.async.bulk.prefetch:
// one instruction for a whole contiguous range, no registers, no completion to
// wait for).  Only the 16-byte-aligned interior is named, so the hint never
// reaches outside the array.
__device__ __forceinline__ void prefetch_l2_range(const void *p, size_t bytes) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    const uintptr_t lo = (a + 15) & ~(uintptr_t)15, hi = (a + bytes) & ~(uintptr_t)15;
    if (hi <= lo) return;
    for (uintptr_t x = lo; x < hi; x += (uintptr_t)1 << 30) {
        const uint32_t sz = (uint32_t)((hi - x) < ((uintptr_t)1 << 30) ? (hi - x) : ((uintptr_t)1 << 30));
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(x), "r"(sz) : "memory");
    }
}

// One element global -> shared memory: an asynchronous copy (cp.async, which
// holds no register and does not wait) when the types agree, so that all of a
// thread's elements are in flight at once; a load and a converting store
// otherwise.  stage_wait() completes the thread's copies.
template <typename TO, typename TI>
__device__ __forceinline__ void stage_elem(TO *dst, const TI *src) {
    if constexpr (std::is_same<TO, TI>::value && (sizeof(TO) == 4 || sizeof(TO) == 8)) {
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                     "l"(src), "n"((int)sizeof(TO))
                     : "memory");
    } else {
        *dst = static_cast<TO>(__ldg(src));
    }
}

// Waits for this thread's staging copies (a barrier must follow before other
// threads read them).
__device__ __forceinline__ void stage_wait() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Stage the block rows of knots [kb, kb+nk) (blk = NB n^2 elements each,
// column-major n x NB n) into the column-interleaved layout M[c*R + k*n + i].
template <typename TO, typename TI>
__device__ __forceinline__ void stage_rows(TO *M, uint32_t R, const TI *__restrict__ g, uint32_t nk,
                                           uint32_t n, uint32_t blk, uint32_t tid, uint32_t nthr) {
    for (uint32_t e = tid; e < nk * blk; e += nthr) {
        const uint32_t kl = e / blk, w = e - kl * blk;
        const uint32_t c = w / n, i = w - c * n;
        stage_elem(M + (size_t)c * R + kl * n + i, g + e);
    }
}

// Stage block `blk_off` (n^2 elements) of each of the block rows of knots
// [kb, kb+nk) (stride elements apart) into M[c*R + k*n + i].
template <typename TO, typename TI>
__device__ __forceinline__ void stage_block(TO *M, uint32_t R, const TI *__restrict__ g, uint32_t nk,
                                            uint32_t n, uint32_t stride, uint32_t tid, uint32_t nthr) {
    const uint32_t blk = n * n;
    for (uint32_t e = tid; e < nk * blk; e += nthr) {
        const uint32_t kl = e / blk, w = e - kl * blk;
        const uint32_t c = w / n, i = w - c * n;
        stage_elem(M + (size_t)c * R + kl * n + i, g + (size_t)kl * stride + w);
    }
}

template <typename A>
__device__ __forceinline__ A warp_sum(A v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += acc_shfl_xor(v, off);
    return v;
}

// Butterfly over the warp for NQ values at once (the shuffles of the values
// interleave): every lane ends with the warp's sums.
template <typename A, int NQ>
__device__ __forceinline__ void warp_sum_n(A (&v)[NQ]) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        A t[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) t[q] = acc_shfl_xor(v[q], off);
#pragma unroll
        for (int q = 0; q < NQ; ++q) v[q] += t[q];
    }
}

// Pairwise sums of M slots at p (A-typed, 16-byte aligned; M = 4, 8, 16, 32
// or 64): four or eight values from vector loads, added as a balanced tree,
// then the halves added.  Straight-line code: every load is issued at once.
template <typename A>
__device__ __forceinline__ void load4(const A *p, A (&x)[4]) {
    if constexpr (std::is_same<A, f2acc>::value) {
        const float4 t0 = reinterpret_cast<const float4 *>(p)[0];
        const float4 t1 = reinterpret_cast<const float4 *>(p)[1];
        x[0] = f2acc(t0.x, t0.y); x[1] = f2acc(t0.z, t0.w); x[2] = f2acc(t1.x, t1.y); x[3] = f2acc(t1.z, t1.w);
    } else if constexpr (sizeof(A) == 4) {
        const float4 t = reinterpret_cast<const float4 *>(p)[0];
        x[0] = t.x; x[1] = t.y; x[2] = t.z; x[3] = t.w;
    } else {
        const double2 t0 = reinterpret_cast<const double2 *>(p)[0];
        const double2 t1 = reinterpret_cast<const double2 *>(p)[1];
        x[0] = t0.x; x[1] = t0.y; x[2] = t1.x; x[3] = t1.y;
    }
}

template <typename A, int M>
__device__ __forceinline__ A tree_slots(const A *p) {
    static_assert(M == 4 || M == 8 || M == 16 || M == 32 || M == 64, "a power of two from 4 to 64");
    if constexpr (M == 4) {
        A x[4];
        load4<A>(p, x);
        return (x[0] + x[1]) + (x[2] + x[3]);
    } else {
        return tree_slots<A, M / 2>(p) + tree_slots<A, M / 2>(p + M / 2);
    }
}

// The slots of one reduction value, summed identically in every thread (the
// slots from `total` on are zero; a warp-uniform branch picks the smallest
// power of two from 4 that covers them): float, the pairwise tree of up to 64
// slots; double and float-float, whose additions are many times dearer than
// float ones on GB300, the tree up to 8 slots and otherwise lane l's slots l,
// l+32, ... finished by a warp butterfly (5 additions a thread); float beyond
// 64 slots the same way.
template <typename A, int NQ>
__device__ __forceinline__ void sum_all_slots(A (&v)[NQ], const A *sl, uint32_t stride, uint32_t total) {
    constexpr bool F = std::is_same<A, float>::value;
    if (total <= 4) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) v[q] = tree_slots<A, 4>(sl + q * stride);
    } else if (total <= 8) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) v[q] = tree_slots<A, 8>(sl + q * stride);
    } else if (F && total <= 16) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) v[q] = tree_slots<A, 16>(sl + q * stride);
    } else if (F && total <= 32) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) v[q] = tree_slots<A, 32>(sl + q * stride);
    } else if (F && total <= 64) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) v[q] = tree_slots<A, 64>(sl + q * stride);
    } else {
        const uint32_t lane = threadIdx.x & 31;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            A s = lane < total ? sl[q * stride + lane] : A(0);
            for (uint32_t j = lane + 32; j < total; j += 32) s += sl[q * stride + j];
            v[q] = s;
        }
        warp_sum_n<A, NQ>(v);
    }
}

// Cluster-wide sum of NQ values, identical in every thread of the cluster.
//   1. a warp butterfly (xor shuffles, the NQ values interleaved) gives every
//      lane of a warp the warp's sums, the same bits in every lane (each step
//      adds the same two values, in either order); for C == 1 lane 0 stores
//      them into slot [w] (for C >= 2, see below);
//   2. one barrier (barrier.cluster, or __syncthreads when C == 1), whose
//      release/acquire makes the stores — and any halo pushes the caller made
//      before this call — visible;
//   3. every thread sums the slots in use (sum_all_slots: pairwise trees, or
//      a strided sum and a warp butterfly).
// Every thread of every CTA reads the same slots in the same order, so all hold
// the same bits.  `buf` alternates between call sites so that a slot array is
// rewritten only after a barrier that every reader has passed.  Slots
// [buf][q][C*32] are zeroed at kernel start.  (The butterfly's five dependent
// shuffle rounds, with the values of a reduction interleaved, beat re-reading
// the warp's 32 values from shared memory by one lane: one value 162 against
// 192 ns, two 224 against 326, three 300 against 504, for a 256-thread CTA.)
// For C >= 2 the slot stage is in two levels, as in cluster_allreduce_tx:
// the warps' sums go into the CTA's local slots (`wscr`, [value][32], zeroed
// at kernel start), warp 0 sums them and stores the CTA's sums into slot
// [rank] of every CTA before the cluster barrier, and every thread adds C
// slots.
template <typename A, int NQ>
__device__ __forceinline__ void cluster_allreduce(A (&v)[NQ], A *slots, A *wscr, int buf,
                                                  const cg::cluster_group &cluster, uint32_t C,
                                                  uint32_t rank) {
    static_assert(NQ <= kMaxValues, "slot array holds kMaxValues values");
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nwarps = blockDim.x >> 5;
    const uint32_t stride = (uint32_t)slot_stride(C);
    A *sl = slots + (size_t)buf * stride * kMaxValues;
    A t[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) t[q] = v[q];
    warp_sum_n<A, NQ>(t);
    if (C == 1) {
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < NQ; ++q) sl[q * stride + warp] = t[q];
        }
        __syncthreads();
        sum_all_slots<A, NQ>(v, sl, stride, nwarps);
    } else {
        // two levels, as cluster_allreduce_tx: the CTA's warp sums in its
        // local slots (`wscr`), summed by warp 0, whose lanes store them into
        // slot [rank] of every CTA; then the cluster barrier
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < NQ; ++q) wscr[q * 32 + warp] = t[q];
        }
        __syncthreads();
        if (warp == 0) {
            sum_all_slots<A, NQ>(t, wscr, 32, nwarps);
            if (lane < C) {
                A *dst = cluster.map_shared_rank(sl, lane);
#pragma unroll
                for (int q = 0; q < NQ; ++q) dst[q * stride + rank] = t[q];
            }
        }
        cluster.sync();
        sum_all_slots<A, NQ>(v, sl, stride, C);
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) v[q] = acc_normalize(v[q]);
}

// Timeline of a launch (LaunchParams::stamps): the GPU's global nanosecond
// clock, read by the cluster's leading thread at four points of each system.
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t sm_id() {
    uint32_t s;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(s));
    return s;
}

struct Stamper {
    bool on;
    uint64_t t_pop = 0, t_staged = 0, t_solved = 0;
    __device__ Stamper(const LaunchParams &lp, uint32_t rank)
        : on(lp.stamps != nullptr && rank == 0 && threadIdx.x == 0) {
        if (lp.cta_sm && threadIdx.x == 0) lp.cta_sm[blockIdx.x] = sm_id();
    }
    __device__ __forceinline__ void pop() {
        if (on) t_pop = global_ns();
    }
    __device__ __forceinline__ void staged() {
        if (on) t_staged = global_ns();
    }
    __device__ __forceinline__ void solved() {
        if (on) t_solved = global_ns();
    }
    // a rejected system: every time equal, no iterations
    __device__ __forceinline__ void rejected() {
        t_staged = t_solved = t_pop;
    }
    __device__ __forceinline__ void done(const LaunchParams &lp, uint32_t item, uint32_t iters) {
        if (!on) return;
        StampRec rec;
        rec.t_pop = t_pop;
        rec.t_staged = t_staged;
        rec.t_solved = t_solved;
        rec.t_done = global_ns();
        rec.system = lp.order ? lp.order[item] : item;
        rec.launch = lp.launch_id;
        rec.cluster = blockIdx.x / cg::this_cluster().num_blocks();
        rec.iters = iters;
        lp.stamps[item] = rec;
    }
};

// ---------------------------------------------------------------- reductions by
// transaction-counted stores.  A cluster barrier (barrier.cluster with release
// and acquire) makes a CTA wait until its own distributed-shared-memory
// stores have reached the other CTAs and then until every CTA has arrived.
// Here each warp's partial sums go to every CTA with st.async, which counts
// the bytes on the receiving CTA's mbarrier (complete_tx); each CTA waits only
// until all of the bytes addressed to it have arrived.  Two mbarriers (and two
// slot buffers) alternate between calls: a CTA's partials for call k+2 can
// only be sent after every CTA has received all of call k+1, which every warp
// of the receiving CTA sent only after it had read its call-k slots.  Halo
// values a reduction's caller sends to its neighbours go the same way, counted
// on the same mbarrier, so their arrival is what the reduction waits for too.
// Every wait is bounded: after about a second without completion it sets the
// CTA's timeout flag and returns (the caller reports the system as timed out;
// every later wait of the CTA returns at once).

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint32_t map_rank_u32(uint32_t local, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes mbarrier initialisations visible to the other CTAs of the cluster
// (they must be followed by a cluster barrier before any remote use).
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void st_async(uint32_t raddr, float v, uint32_t rbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f32 [%0], %1, [%2];" ::"r"(raddr), "f"(v),
                 "r"(rbar)
                 : "memory");
}
__device__ __forceinline__ void st_async(uint32_t raddr, double v, uint32_t rbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f64 [%0], %1, [%2];" ::"r"(raddr), "d"(v),
                 "r"(rbar)
                 : "memory");
}
__device__ __forceinline__ void st_async(uint32_t raddr, f2acc v, uint32_t rbar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];" ::"r"(raddr),
                 "f"(v.hi), "f"(v.lo), "r"(rbar)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase of `bar` with the given parity; gives up after about a
// second (globaltimer), setting *timed_out.  Returns at once if *timed_out is set.
__device__ __forceinline__ void mbar_wait_bounded(uint64_t *bar, uint32_t parity, volatile uint32_t *timed_out) {
    if (mbar_try_wait(bar, parity)) return;
    const uint64_t t0 = global_ns();
    for (uint32_t spin = 1;; ++spin) {
        if (mbar_try_wait(bar, parity)) return;
        if (*timed_out) return;
        if ((spin & 255u) == 0 && global_ns() - t0 > 1000000000ull) {
            *timed_out = 1u;
            return;
        }
    }
}

// Shared state of the transaction-counted reductions of one CTA.
struct TxReduce {
    uint64_t *bar;        // [2] mbarriers, one per slot buffer
    uint32_t parity;      // bit b: parity of the phase buffer b waits for next
    uint32_t *timed_out;  // CTA-wide flag
};

// Cluster-wide sum of NQ values, identical in every thread of the cluster, for
// C >= 2 (C == 1 uses cluster_allreduce, whose barrier is __syncthreads), in
// two levels:
//   1. the warp butterfly gives every warp its sums; lane 0 stores them into
//      this CTA's local slots (`wscr`, [value][32], zero past the warps);
//   2. after a CTA barrier, warp 0 sums the local slots (sum_all_slots over
//      the W warps) and its lanes 0..C-1 send the CTA's sums into slot
//      [rank] of CTA `lane` (st.async counted on that CTA's mbarrier); thread
//      0 arms this CTA's mbarrier with the C values per reduced value it
//      expects plus `extra_bytes` of halo values the neighbours send on the
//      same buffer (push_halo_tx) before this call;
//   3. every thread waits for its CTA's bytes and sums the C slots.
// One CTA sends C values per reduced value instead of C W, and every thread
// adds C slots instead of C W: the adds of the slot stage move to one warp.
// The CTA barrier of step 2 also completes this CTA's stores into its own
// shared memory made before the call (the recurrence form relies on that).
// `wscr` is written by step 1 of the next call only after every warp has
// passed step 3 of this one, which needs warp 0's sends, made after its read.
// In two halves, so that work that needs neither the sums nor the halos can
// run while the partials travel: cluster_allreduce_tx_send (steps 1-2),
// cluster_allreduce_tx_finish (step 3).
template <typename A, int NQ>
__device__ __forceinline__ void cluster_allreduce_tx_send(A (&v)[NQ], A *slots, A *wscr, int buf, TxReduce &tx,
                                                          uint32_t C, uint32_t rank, uint32_t extra_bytes = 0) {
    static_assert(NQ <= kMaxValues, "slot array holds kMaxValues values");
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t nwarps = blockDim.x >> 5;
    const uint32_t stride = (uint32_t)slot_stride(C);
    A *sl = slots + (size_t)buf * stride * kMaxValues;
    A t[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) t[q] = v[q];
    warp_sum_n<A, NQ>(t);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NQ; ++q) wscr[q * 32 + warp] = t[q];
    }
    __syncthreads();
    if (warp == 0) {
        sum_all_slots<A, NQ>(t, wscr, 32, nwarps);
        if (lane == 0) mbar_arrive_expect_tx(tx.bar + buf, (uint32_t)(NQ * C * sizeof(A)) + extra_bytes);
        if (lane < C) {
            const uint32_t rbar = map_rank_u32(smem_u32(tx.bar + buf), lane);
            const uint32_t rsl = map_rank_u32(smem_u32(sl), lane);
#pragma unroll
            for (int q = 0; q < NQ; ++q) st_async(rsl + (uint32_t)((q * stride + rank) * sizeof(A)), t[q], rbar);
        }
    }
}

template <typename A, int NQ>
__device__ __forceinline__ void cluster_allreduce_tx_finish(A (&v)[NQ], A *slots, int buf, TxReduce &tx,
                                                            uint32_t C) {
    const uint32_t stride = (uint32_t)slot_stride(C);
    const A *sl = slots + (size_t)buf * stride * kMaxValues;
    mbar_wait_bounded(tx.bar + buf, (tx.parity >> buf) & 1u, tx.timed_out);
    tx.parity ^= 1u << buf;
    sum_all_slots<A, NQ>(v, sl, stride, C);
#pragma unroll
    for (int q = 0; q < NQ; ++q) v[q] = acc_normalize(v[q]);
}

template <typename A, int NQ>
__device__ __forceinline__ void cluster_allreduce_tx(A (&v)[NQ], A *slots, A *wscr, int buf, TxReduce &tx,
                                                     uint32_t C, uint32_t rank, uint32_t extra_bytes = 0) {
    cluster_allreduce_tx_send<A, NQ>(v, slots, wscr, buf, tx, C, rank, extra_bytes);
    cluster_allreduce_tx_finish<A, NQ>(v, slots, buf, tx, C);
}

// Halo values for a neighbouring CTA, sent like the reduction partials: RPT
// consecutive values into the neighbour's copy of `dst_local` (an address in
// this CTA's shared memory; the neighbour has the same layout), counted on the
// neighbour's mbarrier `buf`, i.e. part of the bytes its next reduction on
// that buffer waits for (cluster_allreduce_tx's extra_bytes).
template <typename T, int RPT>
__device__ __forceinline__ void push_halo_tx(const T *dst_local, uint32_t to, const T (&v)[RPT], const TxReduce &tx,
                                             int buf) {
    const uint32_t ra = map_rank_u32(smem_u32(dst_local), to);
    const uint32_t rb = map_rank_u32(smem_u32(tx.bar + buf), to);
#pragma unroll
    for (int q = 0; q < RPT; ++q) st_async(ra + (uint32_t)(q * sizeof(T)), v[q], rb);
}

// A cluster-wide reduction of the cluster solver: the transaction-counted
// form for C >= 2 (with `extra_bytes` of halo values expected on the same
// buffer), the CTA-barrier form for C == 1.
template <typename A, int NQ>
__device__ __forceinline__ void solver_allreduce(A (&v)[NQ], A *slots, A *wscr, int buf, TxReduce &tx,
                                                 const cg::cluster_group &cluster, uint32_t C, uint32_t rank,
                                                 uint32_t extra_bytes) {
    if (C == 1)
        cluster_allreduce<A, NQ>(v, slots, wscr, buf, cluster, C, rank);
    else
        cluster_allreduce_tx<A, NQ>(v, slots, wscr, buf, tx, C, rank, extra_bytes);
}

// The output fields of work item `item`'s descriptor, read again from memory
// after the iteration (volatile loads: the compiler cannot reuse the copy it
// read when the item was taken, so none of them has to stay in a register
// through the iteration).
struct OutFields {
    void *lambda, *mu, *dS;
    const void *lam_fwd;
    uint32_t flags, result, result_adj;
};
template <typename F>
__device__ __forceinline__ F ld_volatile(const F *p) {
    static_assert(sizeof(F) == 8 || sizeof(F) == 4, "one word");
    if constexpr (sizeof(F) == 8) {
        uint64_t v;
        asm volatile("ld.volatile.global.u64 %0, [%1];" : "=l"(v) : "l"(p));
        F f;
        memcpy(&f, &v, 8);
        return f;
    } else {
        uint32_t v;
        asm volatile("ld.volatile.global.u32 %0, [%1];" : "=r"(v) : "l"(p));
        F f;
        memcpy(&f, &v, 4);
        return f;
    }
}
__device__ __forceinline__ OutFields reload_outputs(const LaunchParams &lp, uint32_t item) {
    OutFields o;
    if (!lp.descs) {
        o.lambda = lp.one.lambda;
        o.mu = lp.one.mu;
        o.dS = lp.one.dS;
        o.lam_fwd = lp.one.lam_fwd;
        o.flags = lp.one.flags;
        o.result = lp.one.result;
        o.result_adj = lp.one.result_adj;
        return o;
    }
    const SysDesc *g = lp.descs + (lp.order ? lp.order[item] : item);
    o.lambda = ld_volatile(&g->lambda);
    o.mu = ld_volatile(&g->mu);
    o.dS = ld_volatile(&g->dS);
    o.lam_fwd = ld_volatile(&g->lam_fwd);
    o.flags = ld_volatile(&g->flags);
    o.result = ld_volatile(&g->result);
    o.result_adj = ld_volatile(&g->result_adj);
    return o;
}

__device__ __forceinline__ void group_sync(const cg::cluster_group &cluster, uint32_t C) {
    if (C > 1)
        cluster.sync();
    else
        __syncthreads();
}

// The solver.  T: storage and arithmetic type of matrices and vectors;
// A: accumulation type of the dot products (T, or double for mixed precision);
// NP: compile-time block-size bound (n <= NP); PTRI: Phi^-1 is block-
// tridiagonal; ST: storage of the matrix rows; RPT: rows per thread.
// REC: recurrence form — y = S p is carried by y = S z + beta y, with S z
// computed right after the reduction that yields beta (z and its halos are in
// the p window by then), so the barrier after the p update disappears: three
// barriers per iteration instead of four.  (Carrying z = Phi^-1 r by a
// recurrence too would remove a fourth, but in FP32 that recurrence drifts
// and the iteration stalls.)  Same passes on well-conditioned systems;
// iterates differ at roundoff level.
// FA: the variant also runs forward + adjoint pairs (SYS_FWD_ADJ) as two
// passes over the same item; without it every check of the adjoint pass is a
// compile-time false and the code is that of single solves.
template <typename T, typename A, int NP, bool PTRI, int ST, int RPT, bool REC, bool FA = false>
__global__ void __launch_bounds__((RegBudget<T, A, NP, PTRI, ST, RPT>::max_threads), 1)
    pcg_cluster_kernel(const LaunchParams lp) {
    using Plan = SmemPlan<T, A, NP, PTRI, ST>;
    constexpr int NBP = PTRI ? 3 : 1;
    constexpr bool S_REG = ST <= ST_REG_S, P_REG = ST == ST_REG, S_HYB = ST == ST_HYB, S_TM = ST == ST_TMEM;
    static_assert(!S_HYB || !PTRI, "the hybrid storage keeps a block-diagonal Phi^-1");
    static_assert(!S_TM || (!PTRI && RPT == 2 && sizeof(T) == 4), "tensor-memory storage: FP32, two rows per thread");
    constexpr int NPT = tmem_cols<NP>();
    static_assert(!S_TM || (RegBudget<T, A, NP, PTRI, ST, RPT>::max_threads + 127) / 128 * RPT * 3 * NPT <=
                               (int)kTmemColumns,
                  "the warps of a CTA fit the tensor memory's columns");
    const cg::cluster_group cluster = cg::this_cluster();
    const uint32_t C = cluster.num_blocks();
    const uint32_t rank = cluster.block_rank();
    const uint32_t tid = threadIdx.x, nthr = blockDim.x;

    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *sp = smem_raw;
    T *vp = reinterpret_cast<T *>(sp); sp += Plan::vec(lp.kmax);
    T *vr = reinterpret_cast<T *>(sp); sp += Plan::vec(lp.kmax);
    T *uh = reinterpret_cast<T *>(sp); sp += Plan::halo();
    T *zh = reinterpret_cast<T *>(sp); sp += Plan::halo();
    A *slots = reinterpret_cast<A *>(sp); sp += Plan::slots(C);
    A *wscr = reinterpret_cast<A *>(sp); sp += Plan::wscr(nthr >> 5);
    uint32_t *s_item = reinterpret_cast<uint32_t *>(sp); sp += kItemBytes;
    T *ms = reinterpret_cast<T *>(sp); sp += Plan::mat_s(lp.kmax);
    T *mp = reinterpret_cast<T *>(sp);
    const uint32_t zero_elems = (uint32_t)((2 * Plan::vec(lp.kmax) + 2 * Plan::halo()) / sizeof(T));

    for (uint32_t e = tid; e < (uint32_t)(Plan::slots(C) / sizeof(A)); e += nthr) slots[e] = A(0);
    for (uint32_t e = tid; e < (uint32_t)(kMaxValues * 32); e += nthr) wscr[e] = A(0);  // local slots
    // transaction-counted reductions (C >= 2): two mbarriers of one arrival each,
    // initialised and made visible to the cluster before any CTA sends to them
    TxReduce tx{reinterpret_cast<uint64_t *>(s_item + 8), 0u, s_item + 12};
    if constexpr (FA) {
        if (tid == 0) s_item[kAdjPassWord] = 0u;
    }
    if (C > 1) {
        if (tid == 0) {
            mbar_init(tx.bar, 1);
            mbar_init(tx.bar + 1, 1);
            *tx.timed_out = 0u;
            mbar_init_fence();
        }
        cluster.sync();
    }
    // this pass is the adjoint pass of a pair (read where needed, not held)
    auto adj_pass = [&]() {
        if constexpr (FA) return *reinterpret_cast<volatile uint32_t *>(s_item + kAdjPassWord) != 0u;
        else return false;
    };
    // tensor memory: warp 0 allocates every column (the CTA is alone on its SM);
    // warp w reaches lanes (w % 4) * 32 + lane, its rows at columns (w / 4) * 3 RPT NPT
    uint32_t tbase = 0, trow = 0;
    if constexpr (S_TM) {
        if ((tid >> 5) == 0) tmem_alloc(s_item + 1, kTmemColumns);
        tmem_fence_before_sync();
        __syncthreads();
        tmem_fence_after_sync();
        tbase = *reinterpret_cast<volatile uint32_t *>(s_item + 1);
        trow = tbase + ((((tid >> 5) & 3u) * 32u) << 16) + (tid >> 7) * (uint32_t)(RPT * 3 * NPT);
    }
    const uint32_t cluster_id = blockIdx.x / C, nclusters = gridDim.x / C;
    Stamper stamp(lp, rank);
    for (uint32_t pass = 0;; ++pass) {
        // ---- pull the next system (cluster leader pops, broadcasts by DSMEM);
        // the adjoint pass of a pair keeps the item it has
        uint32_t item;
        if (lp.queue) {
            if (rank == 0 && tid == 0 && !adj_pass()) {
                const uint32_t it = atomicAdd(lp.queue, 1u);
                for (uint32_t c = 0; c < C; ++c) *cluster.map_shared_rank(s_item, c) = it;
            }
            group_sync(cluster, C);
            item = *reinterpret_cast<volatile uint32_t *>(s_item);
        } else {
            item = cluster_id + pass * nclusters;
            __syncthreads();  // the previous system's epilogue has finished with shared memory
        }
        if (item >= lp.count) break;
        stamp.pop();
        const SysDesc d = lp.descs ? lp.descs[lp.order ? lp.order[item] : item] : lp.one;
        const uint32_t n = d.n, N = d.N;
        const uint32_t K = (N + C - 1) / C;
        if (n == 0 || N == 0 || n > (uint32_t)NP || K > lp.kmax || (size_t)K * n > (size_t)nthr * RPT ||
            (RPT > 1 && (n % RPT) != 0) || (!FA && (d.flags & SYS_FWD_ADJ))) {
            if (rank == 0 && tid == 0) {
                SysResult res = {};
                res.status = -1;
                lp.results[d.result] = res;
            }
            stamp.rejected();
            stamp.done(lp, item, 0);
            group_sync(cluster, C);  // s_item is read by every CTA before the next pop
            continue;                // uniform: every CTA of the cluster sees the same descriptor
        }
        const uint32_t kb = min(rank * K, N), ke = min(kb + K, N), nk = ke - kb;
        const uint32_t row0 = tid * RPT;
        const uint32_t lk = row0 / n, i = row0 - lk * n;  // rows i .. i+RPT-1 of local knot lk
        const bool act = lk < nk;
        const uint32_t k = kb + lk;
        const bool relres = (d.flags & SYS_EXIT_RELRES) != 0;
        const T *__restrict__ S = static_cast<const T *>(d.S);
        const T *__restrict__ P = static_cast<const T *>(d.P);
        const T *__restrict__ gamma = static_cast<const T *>(d.gamma);
        const T *__restrict__ lam0 =
            (d.flags & SYS_LAMBDA0_ZERO) ? nullptr : static_cast<const T *>(d.lambda0);
        const uint32_t blkS = 3 * n * n, blkP = NBP * n * n;
        const uint32_t R = (K * n + 1) & ~1u;  // row stride of staged matrices (even)
        const bool has_left = nk > 0 && kb > 0, has_right = nk > 0 && ke < N;
        const bool first_knot = act && lk == 0 && kb > 0, last_knot = act && lk + 1 == nk && ke < N;
        // halo bytes the neighbours send to this CTA before a reduction (n values each)
        const uint32_t halo_in = ((has_left ? n : 0u) + (has_right ? n : 0u)) * (uint32_t)sizeof(T);
        // this CTA's block rows of S and Phi^-1 into L2 at once: the staging
        // loads below then wait on L2, not on HBM, round after round
        if (tid == 0 && nk > 0 && !adj_pass()) {
            prefetch_l2_range(S + (size_t)kb * blkS, (size_t)nk * blkS * sizeof(T));
            prefetch_l2_range(P + (size_t)kb * blkP, (size_t)nk * blkP * sizeof(T));
        }

        for (uint32_t e = tid; e < zero_elems; e += nthr) vp[e] = T(0);

        // ---- matrices: registers or shared memory.  An adjoint pass finds the
        // rows of shared and tensor memory as the forward pass left them and
        // reloads only those held in registers (from L2).
        T Sr[S_REG || S_HYB || S_TM ? RPT : 1][S_REG ? 3 * NP : (S_HYB ? 2 * NP : (S_TM ? NP : 1))];
        T Pr[P_REG ? RPT : 1][P_REG ? NBP * NP : 1];
        if constexpr (S_REG || S_HYB) {
            const T *Sk = S + (size_t)k * blkS;
#pragma unroll
            for (int b = 0; b < (S_HYB ? 2 : 3); ++b) {
                const bool present = act && (b != 0 || k > 0) && (b != 2 || k + 1 < N);
#pragma unroll
                for (int j = 0; j < NP; ++j)
#pragma unroll
                    for (int q = 0; q < RPT; ++q)
                        Sr[q][b * NP + j] = (present && (uint32_t)j < n)
                                                ? __ldg(Sk + (b * n + j) * n + i + q)
                                                : T(0);
            }
            if constexpr (S_HYB)
                if (!adj_pass()) stage_block(ms, R, S + (size_t)kb * blkS + 2 * n * n, nk, n, blkS, tid, nthr);
        } else if constexpr (S_TM) {
            const T *Sk = S + (size_t)k * blkS;
#pragma unroll
            for (int j = 0; j < NP; ++j)
#pragma unroll
                for (int q = 0; q < RPT; ++q)
                    Sr[q][j] = (act && (uint32_t)j < n) ? __ldg(Sk + (n + j) * n + i + q) : T(0);
            __syncwarp();  // tcgen05 stores are warp-wide
            // The off-diagonal S blocks and Phi^-1 go to TMEM in 8-column pieces
            // ("rounds": 2 blocks x RPT rows x NPT/8 pieces of S, then RPT x NPT/8
            // of Phi^-1), each a tcgen05.st of 8 loaded values.  The loads run
            // kTmemDepth rounds ahead of the stores, so that several rounds' loads
            // are in flight while a store waits for its values.  (Not again in
            // an adjoint pass: the forward pass left them there.)
            if (!adj_pass()) {
                constexpr int NC = NPT / 8, RS = 2 * RPT * NC, RR = RS + RPT * NC;
                const T *Pk = P + (size_t)k * n * n;
                const bool pres0 = act && k > 0, pres2 = act && k + 1 < N;
                auto load_round = [&](int r, float (&v)[8]) {
                    const bool is_s = r < RS;
                    const int rr = is_s ? r % (RPT * NC) : r - RS;
                    const int bi = is_s ? r / (RPT * NC) : 0, q = rr / NC, cc = rr % NC;
                    const bool present = is_s ? (bi == 0 ? pres0 : pres2) : act;
                    const T *src = is_s ? Sk + (size_t)(2 * bi) * n * n + i + q : Pk + i + q;
#pragma unroll
                    for (int u = 0; u < 8; ++u) {
                        const uint32_t j = 8 * cc + u;
                        v[u] = (present && j < n) ? __ldg(src + (size_t)j * n) : 0.f;
                    }
                };
                auto col_of = [&](int r) -> uint32_t {
                    const bool is_s = r < RS;
                    const int rr = is_s ? r % (RPT * NC) : r - RS;
                    const int bi = is_s ? r / (RPT * NC) : 2, q = rr / NC, cc = rr % NC;
                    return (uint32_t)((q * 3 + bi) * NPT + 8 * cc);
                };
                float ring[kTmemDepth][8];
#pragma unroll
                for (int r = 0; r < kTmemDepth && r < RR; ++r) load_round(r, ring[r]);
#pragma unroll
                for (int r = 0; r < RR; ++r) {
                    tmem_st8(trow + col_of(r), ring[r % kTmemDepth]);
                    if (r + kTmemDepth < RR) load_round(r + kTmemDepth, ring[r % kTmemDepth]);
                }
            }
            tmem_wait_st();
        } else {
            const T *Sg = S + (size_t)kb * blkS;
            if (!adj_pass()) stage_rows(ms, R, Sg, nk, n, blkS, tid, nthr);
        }
        if constexpr (S_TM) {
            // Phi^-1 went to tensor memory with the off-diagonal S blocks
        } else if constexpr (P_REG) {
            const T *Pk = P + (size_t)k * blkP;
#pragma unroll
            for (int b = 0; b < NBP; ++b) {
                const bool present =
                    act && (!PTRI || ((b != 0 || k > 0) && (b != 2 || k + 1 < N)));
#pragma unroll
                for (int j = 0; j < NP; ++j)
#pragma unroll
                    for (int q = 0; q < RPT; ++q)
                        Pr[q][b * NP + j] = (present && (uint32_t)j < n)
                                                ? __ldg(Pk + (b * n + j) * n + i + q)
                                                : T(0);
            }
        } else {
            const T *Pg = P + (size_t)kb * blkP;
            if (!adj_pass()) stage_rows(mp, R, Pg, nk, n, blkP, tid, nthr);
        }
        const int sb0 = (k == 0) ? 1 : 0, sb1 = (k + 1 == N) ? 2 : 3;
        auto matS = [&](const T *x, T(&y)[RPT]) {
            if constexpr (S_REG) reg_matvec<T, NP, 3, RPT>(Sr, x, y);
            else if constexpr (S_TM) tmem_matvec<NP>(Sr, trow, x, y);
            else if constexpr (S_HYB) hyb_matvec<T, NP, RPT>(Sr, ms, R, lk * n + i, sb1 == 3, x, n, y);
            else smem_matvec<T, NP, 3, RPT>(ms, R, lk * n + i, sb0, sb1, x, n, y);
        };
        auto matP = [&](const T *x, T(&y)[RPT]) {
            if constexpr (S_TM) {
                tmem_pmatvec<NP>(trow, x, y);
            } else if constexpr (P_REG) {
                if constexpr (PTRI) reg_matvec<T, NP, 3, RPT>(Pr, x, y);
                else reg_matvec<T, NP, 1, RPT>(Pr, x + NP, y);
            } else {
                if constexpr (PTRI) smem_matvec<T, NP, 3, RPT>(mp, R, lk * n + i, sb0, sb1, x, n, y);
                else smem_matvec<T, NP, 1, RPT>(mp, R, lk * n + i, 0, 1, x + NP, n, y);
            }
        };
        // y = S p over this thread's rows (zero for a thread without rows); with
        // tensor memory every thread of a warp takes part in the loads
        auto matS_rows = [&](T(&y)[RPT]) {
            if constexpr (S_TM) {
                matS(vp + (act ? lk : 0u) * NP, y);
                if (!act) {
#pragma unroll
                    for (int q = 0; q < RPT; ++q) y[q] = T(0);
                }
            } else {
                if (act) matS(vp + lk * NP, y);
                else {
#pragma unroll
                    for (int q = 0; q < RPT; ++q) y[q] = T(0);
                }
            }
        };
        // z = Phi^-1 r over this thread's rows, the same way
        auto matP_rows = [&](T(&z)[RPT]) {
            if constexpr (S_TM) {
                matP(vr + (act ? lk : 0u) * NP, z);
                if (!act) {
#pragma unroll
                    for (int q = 0; q < RPT; ++q) z[q] = T(0);
                }
            } else {
                if (act) matP(vr + lk * NP, z);
                else {
#pragma unroll
                    for (int q = 0; q < RPT; ++q) z[q] = T(0);
                }
            }
        };
        T *my_p = vp + (lk + 1) * NP + i;  // this thread's rows in the windows
        T *my_r = vr + (lk + 1) * NP + i;
        stage_wait();
        __syncthreads();
        stamp.staged();

        // ---- r = gamma - S lambda0   (include/pcg.cuh:119-126); the adjoint pass
        // of a pair solves S mu = lambda - lambda* from mu = 0 (lambda: the
        // forward pass's output)
        T gam[RPT], lam[RPT], r[RPT], p[RPT], z[RPT], y[RPT];
        const bool adj0 = adj_pass();
        const T *lam_init = adj0 ? nullptr : lam0;
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
            const size_t row = (size_t)k * n + i + q;
            gam[q] = act ? (adj0 ? static_cast<const T *>(d.lambda)[row] - static_cast<const T *>(d.lstar)[row]
                                 : gamma[row])
                         : T(0);
            lam[q] = (act && lam_init) ? lam_init[row] : T(0);
            if (act) my_p[q] = lam[q];
        }
        if (lam_init) {
            for (uint32_t t = tid; t < 2 * n; t += nthr) {
                if (t < n && has_left) vp[t] = lam_init[(size_t)(kb - 1) * n + t];
                if (t >= n && has_right) vp[(nk + 1) * NP + (t - n)] = lam_init[(size_t)ke * n + (t - n)];
            }
        }
        __syncthreads();
        matS_rows(y);
#pragma unroll
        for (int q = 0; q < RPT; ++q) r[q] = act ? gam[q] - y[q] : T(0);
        group_sync(cluster, C);  // all windows read before any neighbour writes into them

        // ---- z = Phi^-1 r; p = z; eta = r.z   (include/pcg.cuh:131-149)
        if (act) {
#pragma unroll
            for (int q = 0; q < RPT; ++q) my_r[q] = r[q];
        }
        if constexpr (PTRI) {
            if (first_knot) {
                T *dst = cluster.map_shared_rank(vr, rank - 1) + (K + 1) * NP + i;
#pragma unroll
                for (int q = 0; q < RPT; ++q) dst[q] = r[q];
            }
            if (last_knot) {
                T *dst = cluster.map_shared_rank(vr, rank + 1) + i;
#pragma unroll
                for (int q = 0; q < RPT; ++q) dst[q] = r[q];
            }
            group_sync(cluster, C);
        } else {
            __syncthreads();
        }
        matP_rows(z);
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
            if (!act) z[q] = T(0);
            p[q] = z[q];
            if (act) my_p[q] = p[q];
        }
        if (first_knot) push_halo_tx<T, RPT>(vp + (K + 1) * NP + i, rank - 1, z, tx, 1);
        if (last_knot) push_halo_tx<T, RPT>(vp + i, rank + 1, z, tx, 1);
        A eta, gg;
        {
            A v2[2] = {A(0), A(0)};
#pragma unroll
            for (int q = 0; q < RPT; ++q) {
                acc_madd(v2[0], r[q], z[q]);
                acc_madd(v2[1], gam[q], gam[q]);
            }
            solver_allreduce<A, 2>(v2, slots, wscr, 1, tx, cluster, C, rank, halo_in);
            eta = v2[0];
            gg = v2[1];
        }
        const A thr = A(d.tol * d.tol * (double)gg);
        const A tol = A(d.tol);

        // ---- main loop   (include/pcg.cuh:154-208)
        uint32_t iter = 0;
        int32_t status = ST_MAX_ITER;
        A eta_new = A(0), rr = A(0);
        const uint32_t max_iter = d.max_iter;
        if constexpr (REC) {
            // y = S p0 (p0 = z0 and its halos are in vp after the barrier above)
            matS_rows(y);
            for (; iter < max_iter;) {
                if constexpr (PTRI) {  // neighbours need this CTA's boundary y for their r halo
                    if (first_knot) push_halo_tx<T, RPT>(uh + NP + i, rank - 1, y, tx, 0);
                    if (last_knot) push_halo_tx<T, RPT>(uh + i, rank + 1, y, tx, 0);
                }
                A pap;
                {
                    A v1[1] = {A(0)};
#pragma unroll
                    for (int q = 0; q < RPT; ++q) acc_madd(v1[0], p[q], y[q]);
                    solver_allreduce<A, 1>(v1, slots, wscr, 0, tx, cluster, C, rank, PTRI ? halo_in : 0u);
                    pap = v1[0];
                }
                const T alpha = (pap == A(0)) ? T(0) : acc_ratio<T>(eta, pap);
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    lam[q] = fma_rn(alpha, p[q], lam[q]);
                    r[q] = fma_rn(-alpha, y[q], r[q]);
                    if (act) my_r[q] = r[q];
                }
                if constexpr (PTRI) {
                    for (uint32_t t = tid; t < 2 * n; t += nthr) {
                        if (t < n && has_left) vr[t] = fma_rn(-alpha, uh[t], vr[t]);
                        if (t >= n && has_right) {
                            T *h = vr + (nk + 1) * NP + (t - n);
                            *h = fma_rn(-alpha, uh[NP + t - n], *h);
                        }
                    }
                }
                __syncthreads();
                matP_rows(z);
                // z into the vp window (own rows; boundary into the neighbours' halos)
                if (act) {
#pragma unroll
                    for (int q = 0; q < RPT; ++q) my_p[q] = z[q];
                }
                if (first_knot) push_halo_tx<T, RPT>(vp + (K + 1) * NP + i, rank - 1, z, tx, 1);
                if (last_knot) push_halo_tx<T, RPT>(vp + i, rank + 1, z, tx, 1);
                // w = S z is needed only after the reduction, and only the rows
                // next to a neighbour read its halo: the other warps form w
                // while the partials and halos travel (once this CTA's z rows
                // are all in the window), the rest after the wait.  Either
                // way, before the exit test, so that its loads and FMAs
                // interleave with the slot sums.
                T w[RPT];
                {
                    A v2[2] = {A(0), A(0)};
#pragma unroll
                    for (int q = 0; q < RPT; ++q) {
                        acc_madd(v2[0], r[q], z[q]);
                        if (relres) acc_madd(v2[1], r[q], r[q]);
                    }
                    if (C > 1) {
                        // its CTA barrier also completes this CTA's z rows in the window
                        cluster_allreduce_tx_send<A, 2>(v2, slots, wscr, 1, tx, C, rank, halo_in);
                        const bool halo_rows = __any_sync(0xffffffffu, first_knot || last_knot);
                        if (!halo_rows) matS_rows(w);
                        cluster_allreduce_tx_finish<A, 2>(v2, slots, 1, tx, C);
                        if (halo_rows) matS_rows(w);
                    } else {
                        cluster_allreduce<A, 2>(v2, slots, wscr, 1, cluster, C, rank);
                        matS_rows(w);
                    }
                    eta_new = v2[0];
                    rr = v2[1];
                }
                ++iter;
                if (!acc_finite(eta_new) || !acc_finite(pap)) { status = ST_BREAKDOWN; break; }
                if (relres ? (rr <= thr) : (acc_abs(eta_new) < tol)) { status = ST_CONVERGED; break; }
                const T beta = acc_ratio<T>(eta_new, eta);
                eta = eta_new;
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    p[q] = fma_rn(beta, p[q], z[q]);
                    y[q] = fma_rn(beta, y[q], w[q]);
                }
            }
        } else {
            for (; iter < max_iter;) {
                matS_rows(y);
                if constexpr (PTRI) {  // neighbours need this CTA's boundary upsilon for their r halo
                    if (first_knot) push_halo_tx<T, RPT>(uh + NP + i, rank - 1, y, tx, 0);
                    if (last_knot) push_halo_tx<T, RPT>(uh + i, rank + 1, y, tx, 0);
                }
                A pap;
                {
                    A v1[1] = {A(0)};
#pragma unroll
                    for (int q = 0; q < RPT; ++q) acc_madd(v1[0], p[q], y[q]);
                    solver_allreduce<A, 1>(v1, slots, wscr, 0, tx, cluster, C, rank, PTRI ? halo_in : 0u);
                    pap = v1[0];
                }
                const T alpha = (pap == A(0)) ? T(0) : acc_ratio<T>(eta, pap);
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    lam[q] = fma_rn(alpha, p[q], lam[q]);
                    r[q] = fma_rn(-alpha, y[q], r[q]);
                    if (act) my_r[q] = r[q];
                }
                if constexpr (PTRI) {
                    for (uint32_t t = tid; t < 2 * n; t += nthr) {
                        if (t < n && has_left) vr[t] = fma_rn(-alpha, uh[t], vr[t]);
                        if (t >= n && has_right) {
                            T *h = vr + (nk + 1) * NP + (t - n);
                            *h = fma_rn(-alpha, uh[NP + t - n], *h);
                        }
                    }
                }
                __syncthreads();
                matP_rows(z);
                if (first_knot) push_halo_tx<T, RPT>(zh + NP + i, rank - 1, z, tx, 1);
                if (last_knot) push_halo_tx<T, RPT>(zh + i, rank + 1, z, tx, 1);
                {
                    A v2[2] = {A(0), A(0)};
#pragma unroll
                    for (int q = 0; q < RPT; ++q) {
                        acc_madd(v2[0], r[q], z[q]);
                        if (relres) acc_madd(v2[1], r[q], r[q]);
                    }
                    solver_allreduce<A, 2>(v2, slots, wscr, 1, tx, cluster, C, rank, halo_in);
                    eta_new = v2[0];
                    rr = v2[1];
                }
                ++iter;
                if (!acc_finite(eta_new) || !acc_finite(pap)) { status = ST_BREAKDOWN; break; }
                if (relres ? (rr <= thr) : (acc_abs(eta_new) < tol)) { status = ST_CONVERGED; break; }
                const T beta = acc_ratio<T>(eta_new, eta);
                eta = eta_new;
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    p[q] = fma_rn(beta, p[q], z[q]);
                    if (act) my_p[q] = p[q];
                }
                for (uint32_t t = tid; t < 2 * n; t += nthr) {
                    if (t < n && has_left) vp[t] = fma_rn(beta, vp[t], zh[t]);
                    if (t >= n && has_right) {
                        T *h = vp + (nk + 1) * NP + (t - n);
                        *h = fma_rn(beta, *h, zh[NP + t - n]);
                    }
                }
                __syncthreads();
            }
        }

        // ---- outputs   (include/pcg.cuh:212-217)
        stamp.solved();
        const bool adj = adj_pass();
        // the output fields: read again now when pairs are possible, else as taken
        OutFields dd;
        if constexpr (FA) dd = reload_outputs(lp, item);
        else dd = OutFields{d.lambda, d.mu, d.dS, d.lam_fwd, d.flags, d.result, d.result_adj};
        T *lam_out = static_cast<T *>(adj ? dd.mu : dd.lambda);
        if (act) {
#pragma unroll
            for (int q = 0; q < RPT; ++q) lam_out[(size_t)k * n + i + q] = lam[q];
        }
        if (rank == 0 && tid == 0) {
            if (C > 1)  // a reduction wait of some CTA of the cluster gave up
                for (uint32_t c = 0; c < C; ++c)
                    if (*cluster.map_shared_rank(tx.timed_out, c)) status = ST_TIMEOUT;
            SysResult res;
            res.iters = iter;
            res.status = status;
            res.eta = (double)eta_new;
            res.rr = relres ? (double)rr : -1.0;
            res.gg = (double)gg;
            res.outer = 0;
            res.pad = 0;
            lp.results[adj ? dd.result_adj : dd.result] = res;
        }

        // ---- adjoint epilogue: dS = -1/2 (mu lam^T + lam mu^T) on the block pattern
        // (after an adjoint solve, or the adjoint pass of a pair)
        if ((dd.flags & SYS_ADJOINT) || adj) {
            const T *lf = static_cast<const T *>(dd.lam_fwd);
            T *dS = static_cast<T *>(dd.dS);
            group_sync(cluster, C);  // vp / vr free in every CTA
            T lfi[RPT];
#pragma unroll
            for (int q = 0; q < RPT; ++q) {
                lfi[q] = act ? lf[(size_t)k * n + i + q] : T(0);
                if (act) {
                    my_r[q] = lam[q];  // mu
                    my_p[q] = lfi[q];
                }
            }
            if (first_knot) {
                T *dst = cluster.map_shared_rank(vr, rank - 1) + (K + 1) * NP + i;
#pragma unroll
                for (int q = 0; q < RPT; ++q) dst[q] = lam[q];
            }
            if (last_knot) {
                T *dst = cluster.map_shared_rank(vr, rank + 1) + i;
#pragma unroll
                for (int q = 0; q < RPT; ++q) dst[q] = lam[q];
            }
            for (uint32_t t = tid; t < 2 * n; t += nthr) {
                if (t < n && has_left) vp[t] = lf[(size_t)(kb - 1) * n + t];
                if (t >= n && has_right) vp[(nk + 1) * NP + (t - n)] = lf[(size_t)ke * n + (t - n)];
            }
            group_sync(cluster, C);
            if (act) {
                for (uint32_t b = 0; b < 3; ++b) {
                    const bool present = (b != 0 || k > 0) && (b != 2 || k + 1 < N);
                    const T *lw = vp + (lk + b) * NP;
                    const T *mw = vr + (lk + b) * NP;
                    for (uint32_t j = 0; j < n; ++j) {
#pragma unroll
                        for (int q = 0; q < RPT; ++q) {
                            const T g = present ? T(-0.5) * fma_rn(lam[q], lw[j], lfi[q] * mw[j]) : T(0);
                            dS[(size_t)k * blkS + (b * n + j) * n + i + q] = g;
                        }
                    }
                }
            }
        }
        stamp.done(lp, item, iter);
        if constexpr (FA) {
            if ((dd.flags & SYS_FWD_ADJ) && lp.queue) {  // a pair: the adjoint pass next, then a new item
                __syncthreads();  // every thread has read this pass's word
                if (tid == 0) s_item[kAdjPassWord] = adj ? 0u : 1u;
            }
        }
    }
    if (C > 1) cluster.sync();  // every transaction-counted store into this CTA has landed
    if constexpr (S_TM) {  // every TMEM access of the CTA is done
        tmem_fence_before_sync();
        __syncthreads();
        tmem_fence_after_sync();
        if ((tid >> 5) == 0) tmem_dealloc(tbase, kTmemColumns);
    }
}

}  // namespace gbdpcg

namespace gbdpcg {

// Shared-memory plan of the single-reduction kernel: the standard plan plus
// the Phi^-1 blocks of the two halo knots and a second w-halo buffer.
template <typename T, typename A, int NP, int ST>
struct SmemPlanSR {
    using Base = SmemPlan<T, A, NP, false, ST>;
    __host__ __device__ static size_t mhalo() { return round_up((size_t)2 * NP * NP * sizeof(T), 32); }
    __host__ __device__ static size_t bytes(uint32_t kmax, uint32_t C, uint32_t nwarps) {
        return Base::bytes(kmax, C, nwarps) + mhalo() + 2 * Base::halo();
    }
};

// Single-reduction (Chronopoulos-Gear) PCG with a block-diagonal Phi^-1: the
// vectors s = S p and u = Phi^-1 r are carried by recurrences so that
// gamma = r.u, delta = (S u).u (and r.r) are reduced together: one cluster
// reduction per iteration instead of two (transaction-counted for C >= 2, the
// neighbours' boundary w travelling on the same mbarrier).
//   r0 = gamma - S x0, u0 = M r0, w0 = S u0, g0 = r0.u0, d0 = w0.u0,
//   alpha0 = g0/d0, beta0 = 0; per pass
//   p = u + beta p; s = w + beta s; x += alpha p; r -= alpha s; u = M r;
//   w = S u; g' = r.u; d' = w.u; beta = g'/g; alpha = g'/(d' - beta g'/alpha).
// Halos: a CTA needs u of its two halo knots for w = S u.  It receives the
// neighbours' boundary w with the reduction and repeats, on its copies, the
// owner's s_h = w_h + beta s_h, r_h -= alpha s_h and u_h = M_h r_h (the halo
// knots' Phi^-1 blocks are loaded once per system), with the same operations
// in the same order, so the halos equal the owner's values bit for bit.
// Iterates differ from the two-reduction kernel at roundoff level; the exit
// test (|g'| < tol, or ||r|| <= tol ||gamma||) and the pass count are the
// standard iteration's.
template <typename T, typename A, int NP, int ST, int RPT>
__global__ void __launch_bounds__((RegBudget<T, A, NP, false, ST, RPT>::max_threads), 1)
    pcg_sr_kernel(const LaunchParams lp) {
    using Plan = SmemPlan<T, A, NP, false, ST>;
    using PlanSR = SmemPlanSR<T, A, NP, ST>;
    constexpr bool S_REG = ST <= ST_REG_S, P_REG = ST == ST_REG;
    const cg::cluster_group cluster = cg::this_cluster();
    const uint32_t C = cluster.num_blocks();
    const uint32_t rank = cluster.block_rank();
    const uint32_t tid = threadIdx.x, nthr = blockDim.x;

    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *sp = smem_raw;
    T *vu = reinterpret_cast<T *>(sp); sp += Plan::vec(lp.kmax);   // u window (own + halos)
    T *vr = reinterpret_cast<T *>(sp); sp += Plan::vec(lp.kmax);   // r window (own + halos)
    T *sh = reinterpret_cast<T *>(sp); sp += Plan::halo();          // s of the halo knots
    T *wh0 = reinterpret_cast<T *>(sp); sp += Plan::halo();         // received w halos, buffer 0
    A *slots = reinterpret_cast<A *>(sp); sp += Plan::slots(C);
    A *wscr = reinterpret_cast<A *>(sp); sp += Plan::wscr(nthr >> 5);
    uint32_t *s_item = reinterpret_cast<uint32_t *>(sp); sp += kItemBytes;
    T *ms = reinterpret_cast<T *>(sp); sp += Plan::mat_s(lp.kmax);
    T *mp = reinterpret_cast<T *>(sp); sp += Plan::mat_p(lp.kmax);
    T *mh = reinterpret_cast<T *>(sp); sp += PlanSR::mhalo();       // Phi^-1 of the halo knots
    T *wh1 = reinterpret_cast<T *>(sp);                              // received w halos, buffer 1
    const uint32_t zero_elems = (uint32_t)((2 * Plan::vec(lp.kmax) + 2 * Plan::halo()) / sizeof(T));

    for (uint32_t e = tid; e < (uint32_t)(Plan::slots(C) / sizeof(A)); e += nthr) slots[e] = A(0);
    for (uint32_t e = tid; e < (uint32_t)(kMaxValues * 32); e += nthr) wscr[e] = A(0);  // local slots
    // transaction-counted reductions (C >= 2), as in pcg_cluster_kernel
    TxReduce tx{reinterpret_cast<uint64_t *>(s_item + 8), 0u, s_item + 12};
    if (C > 1) {
        if (tid == 0) {
            mbar_init(tx.bar, 1);
            mbar_init(tx.bar + 1, 1);
            *tx.timed_out = 0u;
            mbar_init_fence();
        }
        cluster.sync();
    }
    const uint32_t cluster_id = blockIdx.x / C, nclusters = gridDim.x / C;
    Stamper stamp(lp, rank);
    for (uint32_t pass = 0;; ++pass) {
        uint32_t item;
        if (lp.queue) {
            if (rank == 0 && tid == 0) {
                const uint32_t it = atomicAdd(lp.queue, 1u);
                for (uint32_t c = 0; c < C; ++c) *cluster.map_shared_rank(s_item, c) = it;
            }
            group_sync(cluster, C);
            item = *reinterpret_cast<volatile uint32_t *>(s_item);
        } else {
            item = cluster_id + pass * nclusters;
            __syncthreads();
        }
        if (item >= lp.count) break;
        stamp.pop();
        const SysDesc d = lp.descs ? lp.descs[lp.order ? lp.order[item] : item] : lp.one;
        const uint32_t n = d.n, N = d.N;
        const uint32_t K = (N + C - 1) / C;
        if (n == 0 || N == 0 || n > (uint32_t)NP || K > lp.kmax || (size_t)K * n > (size_t)nthr * RPT ||
            (RPT > 1 && (n % RPT) != 0) || (d.flags & (SYS_PINV_TRI | SYS_ADJOINT | SYS_FWD_ADJ))) {
            if (rank == 0 && tid == 0) {
                SysResult res = {};
                res.status = -1;
                lp.results[d.result] = res;
            }
            stamp.rejected();
            stamp.done(lp, item, 0);
            group_sync(cluster, C);
            continue;
        }
        const uint32_t kb = min(rank * K, N), ke = min(kb + K, N), nk = ke - kb;
        const uint32_t row0 = tid * RPT;
        const uint32_t lk = row0 / n, i = row0 - lk * n;
        const bool act = lk < nk;
        const uint32_t k = kb + lk;
        const bool relres = (d.flags & SYS_EXIT_RELRES) != 0;
        const T *__restrict__ S = static_cast<const T *>(d.S);
        const T *__restrict__ P = static_cast<const T *>(d.P);
        const T *__restrict__ gamma = static_cast<const T *>(d.gamma);
        const T *__restrict__ lam0 =
            (d.flags & SYS_LAMBDA0_ZERO) ? nullptr : static_cast<const T *>(d.lambda0);
        const uint32_t blkS = 3 * n * n, blkP = n * n;
        const uint32_t R = (K * n + 1) & ~1u;  // row stride of staged matrices (even)
        const bool has_left = nk > 0 && kb > 0, has_right = nk > 0 && ke < N;
        const bool first_knot = act && lk == 0 && kb > 0, last_knot = act && lk + 1 == nk && ke < N;
        // halo bytes the neighbours send to this CTA with each reduction (n values each)
        const uint32_t halo_in = ((has_left ? n : 0u) + (has_right ? n : 0u)) * (uint32_t)sizeof(T);
        if (tid == 0 && nk > 0) {  // this CTA's rows into L2 before they are staged
            prefetch_l2_range(S + (size_t)kb * blkS, (size_t)nk * blkS * sizeof(T));
            prefetch_l2_range(P + (size_t)kb * blkP, (size_t)nk * blkP * sizeof(T));
        }

        for (uint32_t e = tid; e < zero_elems; e += nthr) vu[e] = T(0);
        // Phi^-1 blocks of the halo knots (column-major n x n)
        for (uint32_t e = tid; e < 2 * n * n; e += nthr) {
            const uint32_t side = e / (n * n), w = e - side * n * n;
            if (side == 0 && has_left) mh[w] = __ldg(P + (size_t)(kb - 1) * blkP + w);
            if (side == 1 && has_right) mh[NP * NP + w] = __ldg(P + (size_t)ke * blkP + w);
        }

        T Sr[S_REG ? RPT : 1][S_REG ? 3 * NP : 1];
        T Pr[P_REG ? RPT : 1][P_REG ? NP : 1];
        if constexpr (S_REG) {
            const T *Sk = S + (size_t)k * blkS;
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const bool present = act && (b != 0 || k > 0) && (b != 2 || k + 1 < N);
#pragma unroll
                for (int j = 0; j < NP; ++j)
#pragma unroll
                    for (int q = 0; q < RPT; ++q)
                        Sr[q][b * NP + j] = (present && (uint32_t)j < n)
                                                ? __ldg(Sk + (b * n + j) * n + i + q)
                                                : T(0);
            }
        } else {
            const T *Sg = S + (size_t)kb * blkS;
            stage_rows(ms, R, Sg, nk, n, blkS, tid, nthr);
        }
        if constexpr (P_REG) {
            const T *Pk = P + (size_t)k * blkP;
#pragma unroll
            for (int j = 0; j < NP; ++j)
#pragma unroll
                for (int q = 0; q < RPT; ++q)
                    Pr[q][j] = (act && (uint32_t)j < n) ? __ldg(Pk + j * n + i + q) : T(0);
        } else {
            const T *Pg = P + (size_t)kb * blkP;
            stage_rows(mp, R, Pg, nk, n, blkP, tid, nthr);
        }
        const int sb0 = (k == 0) ? 1 : 0, sb1 = (k + 1 == N) ? 2 : 3;
        auto matS = [&](const T *x, T(&y)[RPT]) {
            if constexpr (S_REG) reg_matvec<T, NP, 3, RPT>(Sr, x, y);
            else smem_matvec<T, NP, 3, RPT>(ms, R, lk * n + i, sb0, sb1, x, n, y);
        };
        auto matP = [&](const T *x, T(&y)[RPT]) {
            if constexpr (P_REG) reg_matvec<T, NP, 1, RPT>(Pr, x + NP, y);
            else smem_matvec<T, NP, 1, RPT>(mp, R, lk * n + i, 0, 1, x + NP, n, y);
        };
        // u of halo row t (0..n-1 left knot, n..2n-1 right knot) from the r halo,
        // in the order of the owner's Phi^-1 matvec (j ascending from 0)
        auto halo_u = [&](uint32_t t) {
            const uint32_t side = t < n ? 0 : 1, row = t - side * n;
            const T *M = mh + side * NP * NP + row;
            const T *rw = vr + (side ? (nk + 1) * NP : 0);
            T acc = T(0);
#pragma unroll
            for (int j = 0; j < NP; ++j)  // unrolled to NP: every load issued ahead of the chain
                if ((uint32_t)j < n) acc = fma_rn(M[j * n], rw[j], acc);
            return acc;
        };
        T *my_u = vu + (lk + 1) * NP + i;
        T *my_r = vr + (lk + 1) * NP + i;
        stage_wait();
        __syncthreads();
        stamp.staged();

        // ---- r0 = gamma - S x0 (the u window holds x0 for this product)
        T gam[RPT], lam[RPT], r[RPT], u[RPT], w[RPT], p[RPT], s[RPT];
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
            gam[q] = act ? gamma[(size_t)k * n + i + q] : T(0);
            lam[q] = (act && lam0) ? lam0[(size_t)k * n + i + q] : T(0);
            if (act) my_u[q] = lam[q];
            p[q] = T(0);
            s[q] = T(0);
        }
        if (lam0) {
            for (uint32_t t = tid; t < 2 * n; t += nthr) {
                if (t < n && has_left) vu[t] = lam0[(size_t)(kb - 1) * n + t];
                if (t >= n && has_right) vu[(nk + 1) * NP + (t - n)] = lam0[(size_t)ke * n + (t - n)];
            }
        }
        __syncthreads();
        if (act) matS(vu + lk * NP, w);
#pragma unroll
        for (int q = 0; q < RPT; ++q) r[q] = act ? gam[q] - w[q] : T(0);
        group_sync(cluster, C);  // windows read before any neighbour writes into them
        if (act) {
#pragma unroll
            for (int q = 0; q < RPT; ++q) my_r[q] = r[q];
        }
        if (first_knot) {
            T *dst = cluster.map_shared_rank(vr, rank - 1) + (K + 1) * NP + i;
#pragma unroll
            for (int q = 0; q < RPT; ++q) dst[q] = r[q];
        }
        if (last_knot) {
            T *dst = cluster.map_shared_rank(vr, rank + 1) + i;
#pragma unroll
            for (int q = 0; q < RPT; ++q) dst[q] = r[q];
        }
        group_sync(cluster, C);
        // ---- u0 = M r0 (own rows and halo rows), w0 = S u0
        if (act) matP(vr + lk * NP, u);
        else {
#pragma unroll
            for (int q = 0; q < RPT; ++q) u[q] = T(0);
        }
        for (uint32_t t = tid; t < 2 * n; t += nthr) {
            if (t < n && has_left) vu[t] = halo_u(t);
            if (t >= n && has_right) vu[(nk + 1) * NP + (t - n)] = halo_u(t);
        }
        if (act) {
#pragma unroll
            for (int q = 0; q < RPT; ++q) my_u[q] = u[q];
        }
        __syncthreads();
        if (act) matS(vu + lk * NP, w);
        else {
#pragma unroll
            for (int q = 0; q < RPT; ++q) w[q] = T(0);
        }
        // boundary w into the neighbours' halo buffer 0, counted on their reduction buffer 0
        if (first_knot) push_halo_tx<T, RPT>(wh0 + NP + i, rank - 1, w, tx, 0);
        if (last_knot) push_halo_tx<T, RPT>(wh0 + i, rank + 1, w, tx, 0);
        A g, dlt, gg;
        {
            A v3[3] = {A(0), A(0), A(0)};
#pragma unroll
            for (int q = 0; q < RPT; ++q) {
                acc_madd(v3[0], r[q], u[q]);
                acc_madd(v3[1], w[q], u[q]);
                acc_madd(v3[2], gam[q], gam[q]);
            }
            solver_allreduce<A, 3>(v3, slots, wscr, 0, tx, cluster, C, rank, halo_in);
            g = v3[0];
            dlt = v3[1];
            gg = v3[2];
        }
        const A thr = A(d.tol * d.tol * (double)gg);
        const A tol = A(d.tol);
        T alpha = (dlt == A(0)) ? T(0) : T(g / dlt);
        T beta = T(0);

        uint32_t iter = 0;
        int32_t status = ST_MAX_ITER;
        A g_new = A(0), rr = A(0);
        const uint32_t max_iter = d.max_iter;
        for (; iter < max_iter;) {
            const T *wh = (iter & 1) ? wh1 : wh0;   // w halos received with the last reduction
            T *wh_next = (iter & 1) ? wh0 : wh1;
#pragma unroll
            for (int q = 0; q < RPT; ++q) {
                p[q] = fma_rn(beta, p[q], u[q]);
                s[q] = fma_rn(beta, s[q], w[q]);
                lam[q] = fma_rn(alpha, p[q], lam[q]);
                r[q] = fma_rn(-alpha, s[q], r[q]);
                if (act) my_r[q] = r[q];
            }
            for (uint32_t t = tid; t < 2 * n; t += nthr) {
                if (t < n && has_left) {
                    sh[t] = fma_rn(beta, sh[t], wh[t]);
                    vr[t] = fma_rn(-alpha, sh[t], vr[t]);
                }
                if (t >= n && has_right) {
                    const uint32_t j = t - n;
                    sh[NP + j] = fma_rn(beta, sh[NP + j], wh[NP + j]);
                    T *h = vr + (nk + 1) * NP + j;
                    *h = fma_rn(-alpha, sh[NP + j], *h);
                }
            }
            __syncthreads();
            if (act) matP(vr + lk * NP, u);
            else {
#pragma unroll
                for (int q = 0; q < RPT; ++q) u[q] = T(0);
            }
            for (uint32_t t = tid; t < 2 * n; t += nthr) {
                if (t < n && has_left) vu[t] = halo_u(t);
                if (t >= n && has_right) vu[(nk + 1) * NP + (t - n)] = halo_u(t);
            }
            if (act) {
#pragma unroll
                for (int q = 0; q < RPT; ++q) my_u[q] = u[q];
            }
            __syncthreads();
            if (act) matS(vu + lk * NP, w);
            else {
#pragma unroll
                for (int q = 0; q < RPT; ++q) w[q] = T(0);
            }
            // halo buffer b travels with reduction buffer b: (iter + 1) & 1
            const int buf = (int)((iter + 1) & 1);
            if (first_knot) push_halo_tx<T, RPT>(wh_next + NP + i, rank - 1, w, tx, buf);
            if (last_knot) push_halo_tx<T, RPT>(wh_next + i, rank + 1, w, tx, buf);
            A dn;
            {
                A v3[3] = {A(0), A(0), A(0)};
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    acc_madd(v3[0], r[q], u[q]);
                    acc_madd(v3[1], w[q], u[q]);
                    if (relres) acc_madd(v3[2], r[q], r[q]);
                }
                solver_allreduce<A, 3>(v3, slots, wscr, buf, tx, cluster, C, rank, halo_in);
                g_new = v3[0];
                dn = v3[1];
                rr = v3[2];
            }
            ++iter;
            if (!isfinite(g_new) || !isfinite(dn)) { status = ST_BREAKDOWN; break; }
            if (relres ? (rr <= thr) : (fabs(g_new) < tol)) { status = ST_CONVERGED; break; }
            const A b = g_new / g;
            const A den = dn - b * g_new / A(alpha);
            beta = T(b);
            alpha = (den == A(0)) ? T(0) : T(g_new / den);
            g = g_new;
        }

        stamp.solved();
        T *lam_out = static_cast<T *>(d.lambda);
        if (act) {
#pragma unroll
            for (int q = 0; q < RPT; ++q) lam_out[(size_t)k * n + i + q] = lam[q];
        }
        if (rank == 0 && tid == 0) {
            if (C > 1)  // a reduction wait of some CTA of the cluster gave up
                for (uint32_t c = 0; c < C; ++c)
                    if (*cluster.map_shared_rank(tx.timed_out, c)) status = ST_TIMEOUT;
            SysResult res;
            res.iters = iter;
            res.status = status;
            res.eta = (double)g_new;
            res.rr = relres ? (double)rr : -1.0;
            res.gg = (double)gg;
            res.outer = 0;
            res.pad = 0;
            lp.results[d.result] = res;
        }
        stamp.done(lp, item, iter);
    }
    if (C > 1) cluster.sync();  // every transaction-counted store into this CTA has landed
}

}  // namespace gbdpcg
