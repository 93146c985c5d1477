// Cluster-kernel variants for blocks of size n <= 12: the recurrence form,
// FP32 + FP64 refinement and float-float accumulation (a second translation
// unit so that the variants of one block size compile in parallel).
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np12_ext(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_RF(12)
    GBDPCG_VARIANTS_RF_RPT2(12)
    GBDPCG_VARIANTS_REC(12)
    GBDPCG_VARIANTS_REC_RPT2(12)
    out[c++] = GBDPCG_VARIANT_REC(double, double, 12, false, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT_REC(double, double, 12, false, ST_REG_S, 1);
    GBDPCG_VARIANTS_F2(12)
    GBDPCG_VARIANTS_F2_RPT2(12)
    GBDPCG_VARIANTS_HYB(12)
    GBDPCG_VARIANTS_HYB_RPT2(12)
    GBDPCG_VARIANTS_TMEM(12)
    return c;
}
}  // namespace gbdpcg
