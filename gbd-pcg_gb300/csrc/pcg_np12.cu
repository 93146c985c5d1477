// Cluster-kernel variants for blocks of size n <= 12.
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np12(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_F32(12)
    GBDPCG_VARIANTS_F64_SMEM(12)
    out[c++] = GBDPCG_VARIANT(double, double, 12, false, true);
    out[c++] = GBDPCG_VARIANT(double, double, 12, true, true);
    return c;
}
}  // namespace gbdpcg
