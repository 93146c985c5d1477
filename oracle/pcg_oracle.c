/*
 * ORACLE — test infrastructure only.  CPU restatement of the reference PCG
 * solver (Sdevaud/GBD-PCG) used by tests/ as the parity oracle and by
 * bench.py as the timed host-core baseline.  The product never links it.
 *
 * Two families of functions:
 *
 * 1. oracle_ref_pcg_{f32,f64}: the reference kernel pcg<T,n,N>
 *    (include/pcg.cuh:54-218) restated in its exact arithmetic order:
 *      - the block-row matvec bdmv (include/utils.cuh:46-85): per row, a
 *        sequential fused multiply-add over the 2n or 3n columns of the
 *        column-major n x 3n block row, starting from 0;
 *      - the halo window loadbdVec (include/utils.cuh:9-40);
 *      - dot/reduce in the order of the GLASS stand-in in oracle/glass/glass.cuh
 *        (rounded products, then the halving fold);
 *      - updates lambda += alpha p, r -= alpha v, p = z + beta p as fused
 *        multiply-adds, as nvcc contracts them (include/pcg.cuh:173,174,204);
 *      - exit test |eta_new| < tol after which the pass is counted
 *        (include/pcg.cuh:195); at least one pass is always made.
 *    With the rebuilt reference kernel it agrees bit for bit (GPU test).
 *    Deviation: for knotPoints == 1 the reference reads past the end of the
 *    vectors (include/utils.cuh:21-24 takes the knot-0 branch); here knot 0
 *    of a one-knot system uses the diagonal block only.
 *
 * 2. oracle_pcg_{f32,f64} / oracle_pcg_batch: the same iteration with the
 *    product's options — block-diagonal or block-tridiagonal preconditioner
 *    storage, the reference exit test or a relative recursive-residual exit
 *    ||r||_2 <= tol ||gamma||_2, optional double accumulation of the dot
 *    products — with dots summed sequentially.  This is the host-core
 *    baseline (a port: the reference ships no CPU path) and the oracle for
 *    the product kernels, whose reduction order differs.
 *
 * Compile with -ffp-contract=off: every fused multiply-add is explicit.
 */
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "pcg_oracle.h"

static uint32_t umax(uint32_t a, uint32_t b) { return a > b ? a : b; }

#define DEFINE_ORACLE(T, SUF, FMA, FABS)                                                   \
    /* halving fold of oracle/glass/glass.cuh */                                          \
    static T fold_##SUF(T *x, uint32_t len) {                                              \
        while (len > 1) {                                                                  \
            const uint32_t h = len / 2, up = len - h;                                      \
            for (uint32_t i = 0; i < h; ++i) x[i] = x[i] + x[i + up];                      \
            len = up;                                                                      \
        }                                                                                  \
        return x[0];                                                                       \
    }                                                                                      \
    /* loadbdVec (include/utils.cuh:9-40): w = [v_{k-1} | v_k | v_{k+1}] */                \
    static void window_##SUF(T *w, const T *v, uint32_t n, uint32_t N, uint32_t k) {       \
        memcpy(w + n, v + (size_t)k * n, n * sizeof(T));                                   \
        if (k > 0) memcpy(w, v + (size_t)(k - 1) * n, n * sizeof(T));                      \
        if (k + 1 < N) memcpy(w + 2 * n, v + (size_t)(k + 1) * n, n * sizeof(T));          \
    }                                                                                      \
    /* bdmv (include/utils.cuh:46-85): y = M_k w over the present block columns */        \
    static void bdmv_##SUF(T *y, const T *M, const T *w, uint32_t n, uint32_t N,           \
                           uint32_t k) {                                                   \
        uint32_t c0 = 0, c1 = 3 * n;                                                       \
        if (k == 0) c0 = n;                                                                \
        if (k == N - 1) c1 = 2 * n;                                                        \
        for (uint32_t r = 0; r < n; ++r) {                                                 \
            T val = (T)0;                                                                  \
            for (uint32_t c = c0; c < c1; ++c) val = FMA(M[(size_t)n * c + r], w[c], val); \
            y[r] = val;                                                                    \
        }                                                                                  \
    }                                                                                      \
    static T ref_dot_##SUF(T *prod, const T *a, const T *b, uint32_t n) {                  \
        for (uint32_t i = 0; i < n; ++i) prod[i] = a[i] * b[i];                            \
        return fold_##SUF(prod, n);                                                        \
    }                                                                                      \
    uint32_t oracle_ref_pcg_##SUF(const T *S, const T *Pinv, const T *gamma, T *lambda,    \
                                  uint32_t n, uint32_t N, uint32_t max_iter, T tol,        \
                                  int *max_iter_exit) {                                    \
        const size_t nN = (size_t)n * N, blk = 3 * (size_t)n * n;                          \
        T *r = (T *)calloc(nN, sizeof(T)), *p = (T *)calloc(nN, sizeof(T));                \
        T *z = (T *)calloc(nN, sizeof(T)), *v = (T *)calloc(nN, sizeof(T));                \
        T *part = (T *)calloc(umax(n, N), sizeof(T)), *prod = (T *)calloc(n, sizeof(T));   \
        T *w = (T *)calloc(3 * (size_t)n, sizeof(T));                                      \
        T *lam = lambda;                                                                   \
        uint32_t iter;                                                                     \
        T eta, eta_new, alpha, beta;                                                       \
        /* r = gamma - S lambda   (include/pcg.cuh:119-126) */                             \
        for (uint32_t k = 0; k < N; ++k) {                                                 \
            window_##SUF(w, lam, n, N, k);                                                 \
            bdmv_##SUF(r + k * n, S + k * blk, w, n, N, k);                                \
            for (uint32_t i = 0; i < n; ++i) r[k * n + i] = gamma[k * n + i] - r[k * n + i]; \
        }                                                                                  \
        /* z = Pinv r, p = z, eta = r.z   (include/pcg.cuh:131-149) */                     \
        for (uint32_t k = 0; k < N; ++k) {                                                 \
            window_##SUF(w, r, n, N, k);                                                   \
            bdmv_##SUF(z + k * n, Pinv + k * blk, w, n, N, k);                             \
        }                                                                                  \
        memcpy(p, z, nN * sizeof(T));                                                      \
        for (uint32_t k = 0; k < N; ++k) part[k] = ref_dot_##SUF(prod, r + k * n, z + k * n, n); \
        eta = fold_##SUF(part, N);                                                         \
        *max_iter_exit = 1;                                                                \
        for (iter = 0; iter < max_iter; ++iter) {                                          \
            /* upsilon = S p; alpha = eta / p.upsilon   (:157-169) */                      \
            for (uint32_t k = 0; k < N; ++k) {                                             \
                window_##SUF(w, p, n, N, k);                                               \
                bdmv_##SUF(v + k * n, S + k * blk, w, n, N, k);                            \
            }                                                                              \
            for (uint32_t k = 0; k < N; ++k) part[k] = ref_dot_##SUF(prod, p + k * n, v + k * n, n); \
            alpha = eta / fold_##SUF(part, N);                                             \
            /* lambda += alpha p; r -= alpha upsilon   (:172-176) */                       \
            for (size_t i = 0; i < nN; ++i) {                                              \
                lam[i] = FMA(alpha, p[i], lam[i]);                                         \
                r[i] = FMA(-alpha, v[i], r[i]);                                            \
            }                                                                              \
            /* z = Pinv r; eta_new = r.z   (:181-193) */                                   \
            for (uint32_t k = 0; k < N; ++k) {                                             \
                window_##SUF(w, r, n, N, k);                                               \
                bdmv_##SUF(z + k * n, Pinv + k * blk, w, n, N, k);                         \
            }                                                                              \
            for (uint32_t k = 0; k < N; ++k) part[k] = ref_dot_##SUF(prod, r + k * n, z + k * n, n); \
            eta_new = fold_##SUF(part, N);                                                 \
            if (FABS(eta_new) < tol) { ++iter; *max_iter_exit = 0; break; }  /* :195 */   \
            beta = eta_new / eta;                                                          \
            eta = eta_new;                                                                 \
            for (size_t i = 0; i < nN; ++i) p[i] = FMA(beta, p[i], z[i]);  /* :203-206 */ \
        }                                                                                  \
        free(r); free(p); free(z); free(v); free(part); free(prod); free(w);               \
        return iter;                                                                       \
    }                                                                                      \
    /* ---- product-semantics PCG (sequential dot order) ---- */                          \
    static void matvec_##SUF(T *y, const T *M, const T *x, uint32_t n, uint32_t N,         \
                             int diag_only) {                                              \
        const size_t blk = diag_only ? (size_t)n * n : 3 * (size_t)n * n;                  \
        for (uint32_t k = 0; k < N; ++k) {                                                 \
            const T *Mk = M + k * blk;                                                     \
            T *yk = y + (size_t)k * n;                                                     \
            uint32_t b0 = (k == 0) ? 1 : 0, b1 = (k + 1 == N) ? 2 : 3;                     \
            if (diag_only) b0 = 1, b1 = 2;                                                 \
            for (uint32_t i = 0; i < n; ++i) yk[i] = (T)0;                                 \
            for (uint32_t b = b0; b < b1; ++b) {                                           \
                const T *xb = x + ((size_t)k + b - 1) * n;                                 \
                const T *Mb = diag_only ? Mk : Mk + (size_t)b * n * n;                     \
                for (uint32_t j = 0; j < n; ++j) {                                         \
                    const T xj = xb[j];                                                    \
                    const T *col = Mb + (size_t)j * n;                                     \
                    for (uint32_t i = 0; i < n; ++i) yk[i] = FMA(col[i], xj, yk[i]);       \
                }                                                                          \
            }                                                                              \
        }                                                                                  \
    }                                                                                      \
    static double dot_##SUF(const T *a, const T *b, size_t len, int acc64) {               \
        if (acc64) {                                                                       \
            double s = 0.0;                                                                \
            for (size_t i = 0; i < len; ++i) s = fma((double)a[i], (double)b[i], s);       \
            return s;                                                                      \
        }                                                                                  \
        T s = (T)0;                                                                        \
        for (size_t i = 0; i < len; ++i) s = FMA(a[i], b[i], s);                           \
        return (double)s;                                                                  \
    }                                                                                      \
    int oracle_pcg_##SUF(const T *S, const T *Pinv, const T *gamma, T *lam, uint32_t n,    \
                         uint32_t N, uint32_t max_iter, double tol, uint32_t flags,        \
                         uint32_t *iters_out, double *eta_out, double *rr_out) {           \
        const size_t nN = (size_t)n * N;                                                   \
        const int diag = (flags & ORACLE_PINV_BLOCKDIAG) != 0;                             \
        const int rel = (flags & ORACLE_EXIT_RELRES) != 0;                                 \
        const int acc64 = (flags & ORACLE_ACC64) != 0;                                     \
        T *r = (T *)malloc(nN * sizeof(T)), *p = (T *)malloc(nN * sizeof(T));              \
        T *z = (T *)malloc(nN * sizeof(T)), *v = (T *)malloc(nN * sizeof(T));              \
        int status = ORACLE_MAX_ITER;                                                      \
        uint32_t iter;                                                                     \
        double eta, eta_new = 0.0, rr = 0.0;                                               \
        const double gg = dot_##SUF(gamma, gamma, nN, 1);                                  \
        const double thr = tol * tol * gg;                                                 \
        matvec_##SUF(r, S, lam, n, N, 0);                                                  \
        for (size_t i = 0; i < nN; ++i) r[i] = gamma[i] - r[i];                            \
        matvec_##SUF(z, Pinv, r, n, N, diag);                                              \
        memcpy(p, z, nN * sizeof(T));                                                      \
        eta = dot_##SUF(r, z, nN, acc64);                                                  \
        for (iter = 0; iter < max_iter; ++iter) {                                          \
            matvec_##SUF(v, S, p, n, N, 0);                                                \
            const double pap = dot_##SUF(p, v, nN, acc64);                                 \
            const T alpha = (pap == 0.0) ? (T)0 : (T)(acc64 ? eta / pap                    \
                                                          : (double)((T)eta / (T)pap));    \
            for (size_t i = 0; i < nN; ++i) {                                              \
                lam[i] = FMA(alpha, p[i], lam[i]);                                         \
                r[i] = FMA(-alpha, v[i], r[i]);                                            \
            }                                                                              \
            matvec_##SUF(z, Pinv, r, n, N, diag);                                          \
            eta_new = dot_##SUF(r, z, nN, acc64);                                          \
            if (rel) rr = dot_##SUF(r, r, nN, acc64);                                      \
            if (!isfinite(eta_new) || !isfinite(pap)) { ++iter; status = ORACLE_BREAKDOWN; break; } \
            if (rel ? (rr <= thr) : (fabs(eta_new) < tol)) {                               \
                ++iter; status = ORACLE_CONVERGED; break;                                  \
            }                                                                              \
            const T beta = (T)(acc64 ? eta_new / eta : (double)((T)eta_new / (T)eta));     \
            eta = eta_new;                                                                 \
            for (size_t i = 0; i < nN; ++i) p[i] = FMA(beta, p[i], z[i]);                  \
        }                                                                                  \
        if (iters_out) *iters_out = iter;                                                  \
        if (eta_out) *eta_out = eta_new;                                                   \
        if (rr_out) *rr_out = rel ? rr : dot_##SUF(r, r, nN, 1);                           \
        free(r); free(p); free(z); free(v);                                                \
        return status;                                                                     \
    }                                                                                      \
    /* out = S x in double (the residual of the accuracy checks) */                       \
    void oracle_matvec_##SUF(double *y, const T *S, const T *x, uint32_t n, uint32_t N) {  \
        for (uint32_t k = 0; k < N; ++k) {                                                 \
            for (uint32_t i = 0; i < n; ++i) {                                             \
                double s = 0.0;                                                            \
                for (uint32_t b = (k == 0); b < (k + 1 == N ? 2u : 3u); ++b)               \
                    for (uint32_t j = 0; j < n; ++j)                                       \
                        s += (double)S[(size_t)k * 3 * n * n + (size_t)b * n * n +         \
                                       (size_t)j * n + i] *                                \
                             (double)x[((size_t)k + b - 1) * n + j];                       \
                y[(size_t)k * n + i] = s;                                                  \
            }                                                                              \
        }                                                                                  \
    }

DEFINE_ORACLE(float, f32, fmaf, fabsf)
DEFINE_ORACLE(double, f64, fma, fabs)

/* ---------------- batched host-core baseline (worker pool over a queue) --------------- */
typedef struct {
    oracle_system *sys;
    uint32_t count;
    int is_f64;
    uint32_t flags;
    atomic_uint next;
} batch_job;

static void *batch_worker(void *arg) {
    batch_job *job = (batch_job *)arg;
    for (;;) {
        const uint32_t i = atomic_fetch_add(&job->next, 1u);
        if (i >= job->count) break;
        oracle_system *s = &job->sys[i];
        if (job->is_f64)
            s->status = oracle_pcg_f64((const double *)s->S, (const double *)s->Pinv,
                                       (const double *)s->gamma, (double *)s->lambda, s->n, s->N,
                                       s->max_iter, s->tol, job->flags, &s->iters, NULL, NULL);
        else
            s->status = oracle_pcg_f32((const float *)s->S, (const float *)s->Pinv,
                                       (const float *)s->gamma, (float *)s->lambda, s->n, s->N,
                                       s->max_iter, s->tol, job->flags, &s->iters, NULL, NULL);
    }
    return NULL;
}

int oracle_pcg_batch(oracle_system *sys, uint32_t count, int is_f64, uint32_t flags,
                     int nthreads) {
    batch_job job;
    job.sys = sys;
    job.count = count;
    job.is_f64 = is_f64;
    job.flags = flags;
    atomic_init(&job.next, 0u);
    if (nthreads < 1) nthreads = 1;
    if (nthreads == 1) {
        batch_worker(&job);
        return 0;
    }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
    int started = 0;
    for (int t = 0; t < nthreads; ++t)
        if (pthread_create(&th[t], NULL, batch_worker, &job) == 0) ++started;
    if (started == 0) batch_worker(&job);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    free(th);
    return started;
}

/* ------------- single-reduction (Chronopoulos-Gear) PCG, block-diagonal Phi^-1 -------------
 * The product's opt-in single-reduction variant: s = S p and u = Phi^-1 r are
 * carried by recurrences so that gamma = r.u, delta = (S u).u (and r.r) are
 * reduced together, once per iteration:
 *   r0 = gamma - S x0, u0 = M r0, w0 = S u0, g0 = r0.u0, d0 = w0.u0,
 *   alpha0 = g0/d0, beta0 = 0, p_-1 = s_-1 = 0; then per pass
 *   p = u + beta p; s = w + beta s; x += alpha p; r -= alpha s; u = M r;
 *   w = S u; g' = r.u; d' = w.u; beta = g'/g; alpha = g'/(d' - beta g'/alpha).
 * The exit test and the pass count follow the standard iteration's. */
#define DEFINE_CG1(T, SUF, FMA)                                                            \
    int oracle_pcg_cg1_##SUF(const T *S, const T *Pinv, const T *gamma, T *lam, uint32_t n, \
                             uint32_t N, uint32_t max_iter, double tol, uint32_t flags,     \
                             uint32_t *iters_out, double *eta_out, double *rr_out) {        \
        const size_t nN = (size_t)n * N;                                                   \
        const int rel = (flags & ORACLE_EXIT_RELRES) != 0;                                 \
        const int acc64 = (flags & ORACLE_ACC64) != 0;                                     \
        T *r = (T *)malloc(nN * sizeof(T)), *u = (T *)malloc(nN * sizeof(T));              \
        T *w = (T *)malloc(nN * sizeof(T)), *p = (T *)calloc(nN, sizeof(T));               \
        T *s = (T *)calloc(nN, sizeof(T));                                                 \
        int status = ORACLE_MAX_ITER;                                                      \
        uint32_t iter;                                                                     \
        double g, d, gn = 0, dn, rr = 0;                                                   \
        const double gg = dot_##SUF(gamma, gamma, nN, 1);                                  \
        const double thr = tol * tol * gg;                                                 \
        matvec_##SUF(r, S, lam, n, N, 0);                                                  \
        for (size_t i = 0; i < nN; ++i) r[i] = gamma[i] - r[i];                            \
        matvec_##SUF(u, Pinv, r, n, N, 1);                                                 \
        matvec_##SUF(w, S, u, n, N, 0);                                                    \
        g = dot_##SUF(r, u, nN, acc64);                                                    \
        d = dot_##SUF(w, u, nN, acc64);                                                    \
        T alpha = (d == 0.0) ? (T)0 : (T)(acc64 ? g / d : (double)((T)g / (T)d));          \
        T beta = (T)0;                                                                     \
        for (iter = 0; iter < max_iter; ++iter) {                                          \
            for (size_t i = 0; i < nN; ++i) {                                              \
                p[i] = FMA(beta, p[i], u[i]);                                              \
                s[i] = FMA(beta, s[i], w[i]);                                              \
                lam[i] = FMA(alpha, p[i], lam[i]);                                         \
                r[i] = FMA(-alpha, s[i], r[i]);                                            \
            }                                                                              \
            matvec_##SUF(u, Pinv, r, n, N, 1);                                             \
            matvec_##SUF(w, S, u, n, N, 0);                                                \
            gn = dot_##SUF(r, u, nN, acc64);                                               \
            dn = dot_##SUF(w, u, nN, acc64);                                               \
            if (rel) rr = dot_##SUF(r, r, nN, acc64);                                      \
            if (!isfinite(gn) || !isfinite(dn)) { ++iter; status = ORACLE_BREAKDOWN; break; } \
            if (rel ? (rr <= thr) : (fabs(gn) < tol)) { ++iter; status = ORACLE_CONVERGED; break; } \
            if (acc64) {                                                                   \
                const double b = gn / g;                                                   \
                const double den = dn - b * gn / (double)alpha;                            \
                beta = (T)b;                                                               \
                alpha = (den == 0.0) ? (T)0 : (T)(gn / den);                               \
            } else {                                                                       \
                const T b = (T)gn / (T)g;                                                  \
                const T den = (T)dn - b * (T)gn / alpha;                                   \
                beta = b;                                                                  \
                alpha = (den == (T)0) ? (T)0 : (T)gn / den;                                \
            }                                                                              \
            g = gn;                                                                        \
        }                                                                                  \
        if (iters_out) *iters_out = iter;                                                  \
        if (eta_out) *eta_out = gn;                                                        \
        if (rr_out) *rr_out = rel ? rr : dot_##SUF(r, r, nN, 1);                           \
        free(r); free(u); free(w); free(p); free(s);                                       \
        return status;                                                                     \
    }
DEFINE_CG1(float, f32, fmaf)
DEFINE_CG1(double, f64, fma)
