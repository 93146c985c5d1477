// Cluster-kernel variants for blocks of size n <= 6.
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np6(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_F32(6)
    GBDPCG_VARIANTS_F32_RPT2(6)
    GBDPCG_VARIANTS_F64_SMEM(6)
    out[c++] = GBDPCG_VARIANT(double, double, 6, false, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT_SR(double, double, 6, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT(double, double, 6, true, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT(double, double, 6, false, ST_REG_S, 1);
    out[c++] = GBDPCG_VARIANT_SR(double, double, 6, ST_REG_S, 1);
    return c;
}
}  // namespace gbdpcg
