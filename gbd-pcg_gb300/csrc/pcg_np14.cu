// Cluster-kernel variants for blocks of size n <= 14.
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np14(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_F32(14)
    GBDPCG_VARIANTS_F64_SMEM(14)
    out[c++] = GBDPCG_VARIANT(double, double, 14, false, true);
    return c;
}
}  // namespace gbdpcg
