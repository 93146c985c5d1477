// Cluster-kernel variants for blocks of size n <= 24.
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np24(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_F32(24)
    GBDPCG_VARIANTS_F32_RPT2(24)
    GBDPCG_VARIANTS_F64_SMEM(24)
    out[c++] = GBDPCG_VARIANT(double, double, 24, false, ST_REG_S, 1);
    out[c++] = GBDPCG_VARIANT_SR(double, double, 24, ST_REG_S, 1);
    return c;
}
}  // namespace gbdpcg
