// Instantiation helper for the cluster-kernel variants (one translation unit
// per block-size bound, so that they compile in parallel).
#pragma once
#include "pcg_cluster.cuh"
#include "pcg_refine.cuh"
#include "pcg_stream.cuh"
#include "pcg_variants.h"

#define GBDPCG_VARIANT(T, A, NP, PTRI, ST, RPT)                                               \
    ::gbdpcg::KernelVariant {                                                                 \
        sizeof(T) == 8, ::gbdpcg::acc_code<T, A>(), NP, PTRI, ST, RPT, 0,                     \
            (const void *)&::gbdpcg::pcg_cluster_kernel<T, A, NP, PTRI, ST, RPT, false>,      \
            &::gbdpcg::SmemPlan<T, A, NP, PTRI, ST>::bytes                                    \
    }
#define GBDPCG_VARIANT_REC(T, A, NP, PTRI, ST, RPT)                                           \
    ::gbdpcg::KernelVariant {                                                                 \
        sizeof(T) == 8, ::gbdpcg::acc_code<T, A>(), NP, PTRI, ST, RPT, 3,                     \
            (const void *)&::gbdpcg::pcg_cluster_kernel<T, A, NP, PTRI, ST, RPT, true>,       \
            &::gbdpcg::SmemPlan<T, A, NP, PTRI, ST>::bytes                                    \
    }
// recurrence form (three barriers per iteration)
#define GBDPCG_VARIANTS_REC(NP)                                                               \
    out[c++] = GBDPCG_VARIANT_REC(float, float, NP, false, ST_REG, 1);                        \
    out[c++] = GBDPCG_VARIANT_REC(float, float, NP, true, ST_REG, 1);                         \
    out[c++] = GBDPCG_VARIANT_REC(float, float, NP, false, ST_REG_S, 1);                      \
    out[c++] = GBDPCG_VARIANT_REC(float, float, NP, false, ST_SMEM, 1);                       \
    out[c++] = GBDPCG_VARIANT_REC(float, double, NP, false, ST_REG, 1);                       \
    out[c++] = GBDPCG_VARIANT_REC(double, double, NP, false, ST_SMEM, 1);
#define GBDPCG_VARIANTS_REC_RPT2(NP) out[c++] = GBDPCG_VARIANT_REC(float, float, NP, false, ST_REG_S, 2);
#define GBDPCG_VARIANT_SR(T, A, NP, ST, RPT)                                                  \
    ::gbdpcg::KernelVariant {                                                                 \
        sizeof(T) == 8, ::gbdpcg::acc_code<T, A>(), NP, false, ST, RPT, 1,                    \
            (const void *)&::gbdpcg::pcg_sr_kernel<T, A, NP, ST, RPT>,                        \
            &::gbdpcg::SmemPlanSR<T, A, NP, ST>::bytes                                        \
    }

#define GBDPCG_VARIANT_RF_ACC(NP, ST, RPT, AI)                                                \
    ::gbdpcg::KernelVariant {                                                                 \
        0, ::gbdpcg::acc_code<float, AI>(), NP, false, ST, RPT, 2,                            \
            (const void *)&::gbdpcg::pcg_refine_kernel<NP, ST, RPT, AI>,                      \
            &::gbdpcg::SmemPlanRF<NP, ST>::bytes                                              \
    }
#define GBDPCG_VARIANT_RF(NP, ST, RPT) GBDPCG_VARIANT_RF_ACC(NP, ST, RPT, double)
// FP32 inner solve with FP64 refinement
#define GBDPCG_VARIANTS_RF(NP)                                                                \
    out[c++] = GBDPCG_VARIANT_RF(NP, ST_REG, 1);                                              \
    out[c++] = GBDPCG_VARIANT_RF(NP, ST_REG_S, 1);                                            \
    out[c++] = GBDPCG_VARIANT_RF(NP, ST_SMEM, 1);
#define GBDPCG_VARIANTS_RF_RPT2(NP) out[c++] = GBDPCG_VARIANT_RF(NP, ST_REG_S, 2);

// FP32: rows in registers (RPT 1; RPT 2 for even bounds), S in registers with
// Phi^-1 in shared memory, both in shared memory; FP64 dot accumulation with
// rows in registers.
#define GBDPCG_VARIANTS_F32(NP)                                                               \
    out[c++] = GBDPCG_VARIANT(float, float, NP, false, ST_REG, 1);                            \
    out[c++] = GBDPCG_VARIANT(float, float, NP, true, ST_REG, 1);                             \
    out[c++] = GBDPCG_VARIANT(float, float, NP, false, ST_REG_S, 1);                          \
    out[c++] = GBDPCG_VARIANT(float, float, NP, false, ST_SMEM, 1);                           \
    out[c++] = GBDPCG_VARIANT(float, float, NP, true, ST_SMEM, 1);                            \
    out[c++] = GBDPCG_VARIANT(float, double, NP, false, ST_REG, 1);                           \
    out[c++] = GBDPCG_VARIANT(float, double, NP, true, ST_REG, 1);                            \
    out[c++] = GBDPCG_VARIANT_SR(float, float, NP, ST_REG, 1);                                \
    out[c++] = GBDPCG_VARIANT_SR(float, float, NP, ST_REG_S, 1);                              \
    out[c++] = GBDPCG_VARIANT_SR(float, float, NP, ST_SMEM, 1);                               \
    out[c++] = GBDPCG_VARIANT_SR(float, double, NP, ST_REG, 1);
#define GBDPCG_VARIANTS_F32_RPT2(NP)                                                          \
    out[c++] = GBDPCG_VARIANT(float, float, NP, false, ST_REG, 2);                            \
    out[c++] = GBDPCG_VARIANT(float, float, NP, false, ST_REG_S, 2);                          \
    out[c++] = GBDPCG_VARIANT_SR(float, float, NP, ST_REG_S, 2);
// FP64: rows in shared memory, and in registers where they fit.
#define GBDPCG_VARIANTS_F64_SMEM(NP)                                                          \
    out[c++] = GBDPCG_VARIANT(double, double, NP, false, ST_SMEM, 1);                         \
    out[c++] = GBDPCG_VARIANT(double, double, NP, true, ST_SMEM, 1);                          \
    out[c++] = GBDPCG_VARIANT_SR(double, double, NP, ST_SMEM, 1);

// FP32 systems with float-float dot accumulation (accum.cuh), and FP32 + FP64
// refinement whose inner dot products accumulate in float-float.
#define GBDPCG_VARIANTS_F2(NP)                                                                \
    out[c++] = GBDPCG_VARIANT(float, ::gbdpcg::f2acc, NP, false, ST_REG, 1);                  \
    out[c++] = GBDPCG_VARIANT(float, ::gbdpcg::f2acc, NP, true, ST_REG, 1);                   \
    out[c++] = GBDPCG_VARIANT(float, ::gbdpcg::f2acc, NP, false, ST_REG_S, 1);                \
    out[c++] = GBDPCG_VARIANT(float, ::gbdpcg::f2acc, NP, false, ST_SMEM, 1);                 \
    out[c++] = GBDPCG_VARIANT_REC(float, ::gbdpcg::f2acc, NP, false, ST_REG, 1);              \
    out[c++] = GBDPCG_VARIANT_RF_ACC(NP, ST_REG, 1, ::gbdpcg::f2acc);                         \
    out[c++] = GBDPCG_VARIANT_RF_ACC(NP, ST_REG_S, 1, ::gbdpcg::f2acc);                       \
    out[c++] = GBDPCG_VARIANT_RF_ACC(NP, ST_SMEM, 1, ::gbdpcg::f2acc);
#define GBDPCG_VARIANTS_F2_RPT2(NP)                                                           \
    out[c++] = GBDPCG_VARIANT(float, ::gbdpcg::f2acc, NP, false, ST_REG_S, 2);                \
    out[c++] = GBDPCG_VARIANT_REC(float, ::gbdpcg::f2acc, NP, false, ST_REG_S, 2);            \
    out[c++] = GBDPCG_VARIANT_RF_ACC(NP, ST_REG_S, 2, ::gbdpcg::f2acc);
// Hybrid storage (sub-diagonal and diagonal S blocks in registers, the
// super-diagonal block and Phi^-1 in shared memory), standard and recurrence forms.
#define GBDPCG_VARIANTS_HYB(NP)                                                               \
    out[c++] = GBDPCG_VARIANT(float, float, NP, false, ST_HYB, 1);                            \
    out[c++] = GBDPCG_VARIANT_REC(float, float, NP, false, ST_HYB, 1);
#define GBDPCG_VARIANTS_HYB_RPT2(NP)                                                          \
    out[c++] = GBDPCG_VARIANT(float, float, NP, false, ST_HYB, 2);                            \
    out[c++] = GBDPCG_VARIANT_REC(float, float, NP, false, ST_HYB, 2);
// Variants that run forward + adjoint pairs (FP32, native accumulation): the
// storages the planner and the autotuner choose from (registers, split,
// shared, hybrid, tensor memory), standard and recurrence forms, with a
// compact or a cbtd Phi^-1.
#define GBDPCG_VARIANT_FA(NP, PTRI, ST, RPT, REC)                                             \
    ::gbdpcg::KernelVariant {                                                                 \
        0, 0, NP, PTRI, ST, RPT, REC ? 3 : 0,                                                 \
            (const void *)&::gbdpcg::pcg_cluster_kernel<float, float, NP, PTRI, ST, RPT, REC, true>, \
            &::gbdpcg::SmemPlan<float, float, NP, PTRI, ST>::bytes, 1                         \
    }
#define GBDPCG_VARIANTS_FA(NP)                                                                \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_REG, 1, false);                                \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_REG_S, 1, false);                              \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_SMEM, 1, false);                               \
    out[c++] = GBDPCG_VARIANT_FA(NP, true, ST_REG, 1, false);                                 \
    out[c++] = GBDPCG_VARIANT_FA(NP, true, ST_SMEM, 1, false);                                \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_HYB, 1, false);                                \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_REG, 1, true);                                 \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_SMEM, 1, true);                                \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_HYB, 1, true);
#define GBDPCG_VARIANTS_FA_RPT2(NP)                                                           \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_REG_S, 2, false);                              \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_HYB, 2, false);                                \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_TMEM, 2, false);                               \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_REG_S, 2, true);                               \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_HYB, 2, true);                                 \
    out[c++] = GBDPCG_VARIANT_FA(NP, false, ST_TMEM, 2, true);
// Streamed rows (read from global memory in every product): FP32 with a compact
// Phi^-1 (one or two rows per thread) or a cbtd one, FP64 with either.
#define GBDPCG_VARIANT_STREAM(T, A, NP, PTRI, RPT)                                            \
    ::gbdpcg::KernelVariant {                                                                 \
        sizeof(T) == 8, ::gbdpcg::acc_code<T, A>(), NP, PTRI, ::gbdpcg::ST_STREAM, RPT, 0,    \
            (const void *)&::gbdpcg::pcg_stream_kernel<T, A, NP, PTRI, RPT>,                  \
            &::gbdpcg::SmemPlanStream<T, A, NP, PTRI>::bytes                                  \
    }
#define GBDPCG_VARIANTS_STREAM(NP)                                                            \
    out[c++] = GBDPCG_VARIANT_STREAM(float, float, NP, false, 1);                             \
    out[c++] = GBDPCG_VARIANT_STREAM(float, float, NP, false, 2);                             \
    out[c++] = GBDPCG_VARIANT_STREAM(float, float, NP, true, 1);                              \
    out[c++] = GBDPCG_VARIANT_STREAM(double, double, NP, false, 1);                           \
    out[c++] = GBDPCG_VARIANT_STREAM(double, double, NP, true, 1);
// Tensor-memory storage (diagonal S block in registers, off-diagonal blocks in
// TMEM, Phi^-1 in shared memory), two rows per thread, standard and recurrence forms.
#define GBDPCG_VARIANTS_TMEM(NP)                                                              \
    out[c++] = GBDPCG_VARIANT(float, float, NP, false, ST_TMEM, 2);                           \
    out[c++] = GBDPCG_VARIANT_REC(float, float, NP, false, ST_TMEM, 2);
