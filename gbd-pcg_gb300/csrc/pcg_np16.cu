// Cluster-kernel variants for blocks of size n <= 16.
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np16(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_F32(16)
    GBDPCG_VARIANTS_F32_RPT2(16)
    GBDPCG_VARIANTS_F64_SMEM(16)
    out[c++] = GBDPCG_VARIANT(double, double, 16, false, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT_SR(double, double, 16, ST_REG, 1);
    out[c++] = GBDPCG_VARIANT(double, double, 16, false, ST_REG_S, 1);
    out[c++] = GBDPCG_VARIANT_SR(double, double, 16, ST_REG_S, 1);
    return c;
}
}  // namespace gbdpcg
