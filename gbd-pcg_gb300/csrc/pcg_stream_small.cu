// Streamed-row cluster-kernel variants for blocks of size n <= 14.
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_stream_small(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_STREAM(6)
    GBDPCG_VARIANTS_STREAM(8)
    GBDPCG_VARIANTS_STREAM(12)
    GBDPCG_VARIANTS_STREAM(14)
    return c;
}
}  // namespace gbdpcg
