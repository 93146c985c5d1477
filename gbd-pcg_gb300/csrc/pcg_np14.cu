// Cluster-kernel variants for blocks of size n <= 14.
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np14(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_F32(14)
    GBDPCG_VARIANTS_F32_RPT2(14)
    GBDPCG_VARIANTS_F64_SMEM(14)
    out[c++] = GBDPCG_VARIANT(double, double, 14, false, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT_SR(double, double, 14, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT(double, double, 14, false, ST_REG_S, 1);
    out[c++] = GBDPCG_VARIANT_SR(double, double, 14, ST_REG_S, 1);
    return c;
}
}  // namespace gbdpcg
