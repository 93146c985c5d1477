// Cluster-kernel variants for blocks of size n <= 32.
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np32(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_F32(32)
    GBDPCG_VARIANTS_F64_SMEM(32)
    return c;
}
}  // namespace gbdpcg
