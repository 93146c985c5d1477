// Test infrastructure only: a stand-in for the three device routines of the
// GLASS library (A2R-Lab/GLASS, a git submodule that the reference does not
// vendor; its pinned commit is unknown) that the reference PCG kernel calls.
// It exists so that the reference kernel (include/pcg.cuh of Sdevaud/GBD-PCG)
// can be rebuilt for sm_103a and run beside this project's kernels as a parity
// check and a GPU baseline. Nothing in the product links it.
//
// Semantics follow the reference's call sites:
//   glass::copy<T>(n, src, dst)        include/pcg.cuh:111,215  block-strided copy
//   glass::dot<T, n>(out, a, b)        include/pcg.cuh:144,163,187  out[0] = sum a_i b_i
//   glass::reduce<T>(out, n, d_in)     include/pcg.cuh:147,167,191  out[0] = sum d_in[0..n)
// The scratch `out` holds max(n, knot_points) elements (include/pcg.cuh:91-92),
// so dot stages the n products there and reduces them in place.
//
// Reduction order (written here, restated exactly by oracle/pcg_oracle.c):
// products are rounded to T, then a "halving fold" repeats
//     h = len / 2;  up = len - h;  x[i] += x[i + up]  for i < h;  len = up
// until len == 1.  Every step ends with __syncthreads(), so x[0] is visible to
// the whole block on return.
#pragma once
#include <stdint.h>

namespace glass {

template <typename T>
__device__ void copy(uint32_t n, const T *src, T *dst) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) dst[i] = src[i];
}

template <typename T>
__device__ void halving_fold(T *x, uint32_t len) {
    while (len > 1) {
        const uint32_t h = len / 2, up = len - h;
        for (uint32_t i = threadIdx.x; i < h; i += blockDim.x) x[i] = x[i] + x[i + up];
        __syncthreads();
        len = up;
    }
}

template <typename T, uint32_t n>
__device__ void dot(T *out, T *a, T *b) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const T prod = a[i] * b[i];
        out[i] = prod;
    }
    __syncthreads();
    halving_fold<T>(out, n);
}

template <typename T>
__device__ void reduce(T *out, uint32_t n, T *d_in) {
    copy<T>(n, d_in, out);
    __syncthreads();
    halving_fold<T>(out, n);
}

}  // namespace glass
