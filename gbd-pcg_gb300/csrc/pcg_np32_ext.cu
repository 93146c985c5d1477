// Cluster-kernel variants for blocks of size n <= 32: the recurrence form,
// FP32 + FP64 refinement and float-float accumulation (a second translation
// unit so that the variants of one block size compile in parallel).
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_np32_ext(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_RF(32)
    GBDPCG_VARIANTS_REC(32)
    GBDPCG_VARIANTS_F2(32)
    GBDPCG_VARIANTS_HYB(32)
    return c;
}
}  // namespace gbdpcg
