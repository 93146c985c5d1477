// Cluster-kernel variants for blocks of size n <= 12 that run forward +
// adjoint pairs (a translation unit of their own, compiled in parallel).
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_fa_np12(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_FA(12)
    GBDPCG_VARIANTS_FA_RPT2(12)
    return c;
}
}  // namespace gbdpcg
