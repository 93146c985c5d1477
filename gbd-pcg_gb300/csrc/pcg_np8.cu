// Cluster-kernel variants for blocks of size n <= 8.
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np8(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_F32(8)
    GBDPCG_VARIANTS_F32_RPT2(8)
    GBDPCG_VARIANTS_F64_SMEM(8)
    out[c++] = GBDPCG_VARIANT(double, double, 8, false, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT_SR(double, double, 8, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT(double, double, 8, true, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT(double, double, 8, false, ST_REG_S, 1);
    out[c++] = GBDPCG_VARIANT_SR(double, double, 8, ST_REG_S, 1);
    return c;
}
}  // namespace gbdpcg
