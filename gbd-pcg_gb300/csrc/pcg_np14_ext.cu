// Cluster-kernel variants for blocks of size n <= 14: the recurrence form,
// FP32 + FP64 refinement and float-float accumulation (a second translation
// unit so that the variants of one block size compile in parallel).
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np14_ext(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_RF(14)
    GBDPCG_VARIANTS_RF_RPT2(14)
    GBDPCG_VARIANTS_REC(14)
    GBDPCG_VARIANTS_REC_RPT2(14)
    out[c++] = GBDPCG_VARIANT_REC(double, double, 14, false, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT_REC(double, double, 14, false, ST_REG_S, 1);
    GBDPCG_VARIANTS_F2(14)
    GBDPCG_VARIANTS_F2_RPT2(14)
    GBDPCG_VARIANTS_HYB(14)
    GBDPCG_VARIANTS_HYB_RPT2(14)
    GBDPCG_VARIANTS_TMEM(14)
    return c;
}
}  // namespace gbdpcg
