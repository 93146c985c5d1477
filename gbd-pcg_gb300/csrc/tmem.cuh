// Tensor memory (TMEM) as storage for matrix rows.
//
// Each SM of GB300 has 256 KB of tensor memory: 128 lanes x 512 columns of 32
// bits, allocated per CTA by column ranges (tcgen05.alloc) and moved to and
// from registers by tcgen05.st / tcgen05.ld.  A warp reaches only the 32
// lanes of its quarter, (warp % 4) * 32 .. + 31; with the 32x32b shape each
// thread of the warp owns one lane and moves N consecutive columns of it.
// The PCG kernels use it as a third on-chip tier beside registers and shared
// memory: matrix rows written once per system and read every iteration.
//
// Allocation can wait for columns that another CTA on the same SM holds, so
// a kernel that allocates all 512 columns must be the only such CTA on its
// SM.  The kernels that use these helpers guarantee that through their
// shared-memory request (more than half of an SM's), and deallocate before
// they exit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbdpcg {

constexpr uint32_t kTmemColumns = 512;

// Warp-wide (all 32 threads): allocate `ncols` columns, address written to smem.
__device__ __forceinline__ void tmem_alloc(uint32_t *smem_dst, uint32_t ncols) {
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(smem_dst);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

// Warp-wide: release the columns.
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// Ordering of TMEM accesses across a thread barrier.
__device__ __forceinline__ void tmem_fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Warp-wide: this thread's lane, columns [taddr, taddr+8) <- v.
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const float (&v)[8]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
        "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
        "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
        : "memory");
}

// Warp-wide: wait until this thread's TMEM stores have completed.
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Warp-wide: a <- columns [ta, ta+8), b <- columns [tb, tb+8) of this thread's
// lane; the wait is in the same statement, so the registers are ready when it
// returns.
__device__ __forceinline__ void tmem_ld8x2(uint32_t ta, uint32_t tb, float (&a)[8], float (&b)[8]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%16];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8, %9, %10, %11, %12, %13, %14, %15}, [%17];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(ta), "r"(tb)
        : "memory");
#pragma unroll
    for (int u = 0; u < 8; ++u) {
        a[u] = __uint_as_float(r[u]);
        b[u] = __uint_as_float(r[8 + u]);
    }
}

}  // namespace gbdpcg
