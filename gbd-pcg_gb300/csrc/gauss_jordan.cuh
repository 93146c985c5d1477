// Rotating Gauss-Jordan inverse of a small symmetric positive definite block
// held one row per lane of a warp (shared by the block-Jacobi builder and the
// fused Schur formation).  Lane r holds row r of the block in registers,
// padded with the identity to NP x NP; step j pivots on row j and on each
// row's first register, then every row shifts one column to the left and the
// column of the inverse being formed enters at the right, so all register
// indices are compile-time constants while the step loop stays rolled, and
// after NP steps the columns are back in order.  No pivoting (the block is
// symmetric positive definite); a zero pivot leaves its column unscaled.
#pragma once
#include <stdint.h>

namespace gbdpcg {

template <typename CT>
struct PrecVec;  // 16-byte shared-memory loads
template <>
struct PrecVec<float> {
    static constexpr int W = 4;
    __device__ static void get(const float *p, float *v) {
        const float4 t = *reinterpret_cast<const float4 *>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
    __device__ static void put(float *p, const float *v) {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};
template <>
struct PrecVec<double> {
    static constexpr int W = 2;
    __device__ static void get(const double *p, double *v) {
        const double2 t = *reinterpret_cast<const double2 *>(p);
        v[0] = t.x; v[1] = t.y;
    }
    __device__ static void put(double *p, const double *v) {
        *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]);
    }
};

// Rotating Gauss-Jordan inverse of the NP x NP block whose row `lane` is a
// (lanes >= NP hold nothing).  s_raw, s_t: NP-element, 16-byte aligned rows;
// NP a multiple of the 16-byte vector width.
template <typename CT, int NP>
__device__ __forceinline__ void gj_rotate(CT (&a)[NP], CT *s_raw, CT *s_t, uint32_t lane) {
    constexpr int W = PrecVec<CT>::W;
#pragma unroll 1
    for (uint32_t j = 0; j < (uint32_t)NP; ++j) {
        const bool pivot = lane == j;
        if (pivot) {  // the pivot row, 16 bytes a store
#pragma unroll
            for (int c = 0; c < NP; c += W) PrecVec<CT>::put(s_raw + c, a + c);
        }
        __syncwarp();
        CT piv = s_raw[0];
        if (piv == CT(0)) piv = CT(1);  // singular block: leave that column unscaled
        const CT inv = CT(1) / piv;
        // scaled pivot row, shifted one column left; the new last column is inv
        if (lane + 1 < (uint32_t)NP) s_t[lane] = s_raw[lane + 1] * inv;
        else if (lane + 1 == (uint32_t)NP) s_t[lane] = inv;
        __syncwarp();
        const CT m = a[0];
#pragma unroll
        for (int c = 0; c < NP; c += W) {
            CT t[W];
            PrecVec<CT>::get(s_t + c, t);
#pragma unroll
            for (int u = 0; u < W; ++u) {
                const int e = c + u;
                if (e + 1 < NP) a[e] = pivot ? t[u] : a[e + 1] - m * t[u];
                else a[e] = pivot ? t[u] : -(m * inv);
            }
        }
        __syncwarp();  // the rows are read before the next step overwrites them
    }
}

}  // namespace gbdpcg
