// Cluster-kernel variants for blocks of size n <= 12.
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np12(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_F32(12)
    GBDPCG_VARIANTS_F32_RPT2(12)
    GBDPCG_VARIANTS_F64_SMEM(12)
    out[c++] = GBDPCG_VARIANT(double, double, 12, false, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT_SR(double, double, 12, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT(double, double, 12, true, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT(double, double, 12, false, ST_REG_S, 1);
    out[c++] = GBDPCG_VARIANT_SR(double, double, 12, ST_REG_S, 1);
    return c;
}
}  // namespace gbdpcg
