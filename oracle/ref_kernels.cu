// Test infrastructure only.  Rebuilds the reference kernel pcg<T, n, N>
// (include/pcg.cuh:54-218 of Sdevaud/GBD-PCG, included from the reference
// checkout at build time, never copied) for sm_103a, against the GLASS
// stand-in in oracle/glass/.  The reference takes its sizes as template
// arguments, so every (n, N) it is run at is listed here.  Its dynamic shared
// array is declared `extern __shared__ T s_temp[]` (include/pcg.cuh:79), so one
// translation unit can only hold one T: the recipe compiles this file twice,
// with and without REF_PCG_DOUBLE, into two device-only cubins in oracle/_ref/
// that ref_launcher.cu loads at run time.
#include "glass.cuh"
#include "pcg.cuh"

#ifdef REF_PCG_DOUBLE
typedef double ref_real;
#define REF_PCG_SIZES(X) X(2, 3) X(3, 5) X(14, 32) X(14, 128)
#else
typedef float ref_real;
#define REF_PCG_SIZES(X) \
    X(2, 3) X(3, 5) X(5, 2) X(14, 32) X(14, 64) X(14, 128) X(6, 64) X(12, 64) X(24, 128)
#endif

#define REF_PCG_INSTANTIATE(n, N)                                                   \
    template __global__ void pcg<ref_real, n##u, N##u>(                             \
        ref_real *, ref_real *, ref_real *, ref_real *, ref_real *, ref_real *,     \
        ref_real *, ref_real *, uint32_t *, bool *, uint32_t, ref_real);
REF_PCG_SIZES(REF_PCG_INSTANTIATE)
