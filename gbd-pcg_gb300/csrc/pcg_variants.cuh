// Instantiation helper for the cluster-kernel variants (one translation unit
// per block-size bound, so that they compile in parallel).
#pragma once
#include "pcg_cluster.cuh"
#include "pcg_variants.h"

#define GBDPCG_VARIANT(T, A, NP, PTRI, MREG)                                                  \
    ::gbdpcg::KernelVariant {                                                                 \
        sizeof(T) == 8, sizeof(A) == 8, NP, PTRI, MREG,                                       \
            (const void *)&::gbdpcg::pcg_cluster_kernel<T, A, NP, PTRI, MREG>,                \
            &::gbdpcg::SmemPlan<T, A, NP, PTRI, MREG>::bytes                                  \
    }

// fp32 in registers (native and FP64 dot accumulation) and in shared memory;
// fp64 in shared memory, and in registers where the rows fit.
#define GBDPCG_VARIANTS_F32(NP)                                                               \
    out[c++] = GBDPCG_VARIANT(float, float, NP, false, true);                                 \
    out[c++] = GBDPCG_VARIANT(float, float, NP, true, true);                                  \
    out[c++] = GBDPCG_VARIANT(float, double, NP, false, true);                                \
    out[c++] = GBDPCG_VARIANT(float, double, NP, true, true);                                 \
    out[c++] = GBDPCG_VARIANT(float, float, NP, false, false);                                \
    out[c++] = GBDPCG_VARIANT(float, float, NP, true, false);
#define GBDPCG_VARIANTS_F64_SMEM(NP)                                                          \
    out[c++] = GBDPCG_VARIANT(double, double, NP, false, false);                              \
    out[c++] = GBDPCG_VARIANT(double, double, NP, true, false);
