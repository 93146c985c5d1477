// Registry of the instantiated cluster-kernel variants (host side).
#pragma once
#include <stddef.h>
#include <stdint.h>

namespace gbdpcg {

struct KernelVariant {
    int f64;     // matrices and vectors in double
    int acc;     // dot-product accumulation: 0 in T (float), 1 double, 2 float-float
    int np;      // compile-time block-size bound (n <= np)
    int ptri;    // Phi^-1 block-tridiagonal (cbtd) instead of block-diagonal
    int st;      // storage: 0 S and Phi^-1 in registers, 1 S in registers and Phi^-1 in
                 // shared memory, 2 both in shared memory, 3 hybrid, 4 tensor memory,
                 // 5 streamed from global memory
    int rpt;     // matrix rows per thread (2 needs an even n)
    int alg;     // 0 two reductions per iteration, 1 single reduction (block-diagonal Phi^-1),
                 // 2 FP32 inner PCG with FP64 refinement, 3 recurrence form (three barriers
                 // per iteration)
    const void *func;
    size_t (*smem_bytes)(uint32_t kmax, uint32_t C, uint32_t nwarps);
    int fa = 0;  // runs forward + adjoint pairs (SYS_FWD_ADJ), for such plans only
};

// Each returns the number of variants written to `out` (at most kMaxVariantsPerNP).
constexpr int kMaxVariantsPerNP = 64;
int variants_np6(KernelVariant *out);
int variants_np8(KernelVariant *out);
int variants_np12(KernelVariant *out);
int variants_np14(KernelVariant *out);
int variants_np16(KernelVariant *out);
int variants_np24(KernelVariant *out);
int variants_np32(KernelVariant *out);
int variants_np6_ext(KernelVariant *out);
int variants_np8_ext(KernelVariant *out);
int variants_np12_ext(KernelVariant *out);
int variants_np14_ext(KernelVariant *out);
int variants_np16_ext(KernelVariant *out);
int variants_np24_ext(KernelVariant *out);
int variants_np32_ext(KernelVariant *out);
int variants_stream_small(KernelVariant *out);  // streamed rows, NP 6..14
int variants_fa_np6(KernelVariant *out);  // forward + adjoint pair variants, one unit per NP
int variants_fa_np8(KernelVariant *out);
int variants_fa_np12(KernelVariant *out);
int variants_fa_np14(KernelVariant *out);
int variants_fa_np16(KernelVariant *out);
int variants_fa_np24(KernelVariant *out);
int variants_fa_np32(KernelVariant *out);
int variants_stream_large(KernelVariant *out);  // streamed rows, NP 16..32

const void *plain_kernel_ptr(bool f64);
size_t plain_smem_bytes(bool f64, uint32_t n, uint32_t N);

}  // namespace gbdpcg
