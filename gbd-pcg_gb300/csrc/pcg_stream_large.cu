// Streamed-row cluster-kernel variants for blocks of size 14 < n <= 32.
#include "pcg_variants.cuh"

namespace gbdpcg {
int variants_stream_large(KernelVariant *out) {
    int c = 0;
    GBDPCG_VARIANTS_STREAM(16)
    GBDPCG_VARIANTS_STREAM(24)
    GBDPCG_VARIANTS_STREAM(32)
    return c;
}
}  // namespace gbdpcg
