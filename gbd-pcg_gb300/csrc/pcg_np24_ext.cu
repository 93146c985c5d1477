// Cluster-kernel variants for blocks of size n <= 24: the recurrence form,
// FP32 + FP64 refinement and float-float accumulation (a second translation
// unit so that the variants of one block size compile in parallel).
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np24_ext(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_RF(24)
    GBDPCG_VARIANTS_RF_RPT2(24)
    GBDPCG_VARIANTS_REC(24)
    GBDPCG_VARIANTS_REC_RPT2(24)
    out[c++] = GBDPCG_VARIANT_REC(double, double, 24, false, ST_REG_S, 1);
    GBDPCG_VARIANTS_F2(24)
    GBDPCG_VARIANTS_F2_RPT2(24)
    GBDPCG_VARIANTS_HYB(24)
    GBDPCG_VARIANTS_HYB_RPT2(24)
    GBDPCG_VARIANTS_TMEM(24)
    return c;
}
}  // namespace gbdpcg
