/* ORACLE — test infrastructure only (see pcg_oracle.c). */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_PINV_BLOCKDIAG = 1u, ORACLE_EXIT_RELRES = 2u, ORACLE_ACC64 = 4u };
enum { ORACLE_CONVERGED = 0, ORACLE_MAX_ITER = 1, ORACLE_BREAKDOWN = 2 };

typedef struct {
    const void *S, *Pinv, *gamma;
    void *lambda;
    uint32_t n, N, max_iter;
    double tol;
    uint32_t iters;
    int status;
} oracle_system;

uint32_t oracle_ref_pcg_f32(const float *S, const float *Pinv, const float *gamma, float *lambda,
                            uint32_t n, uint32_t N, uint32_t max_iter, float tol,
                            int *max_iter_exit);
uint32_t oracle_ref_pcg_f64(const double *S, const double *Pinv, const double *gamma,
                            double *lambda, uint32_t n, uint32_t N, uint32_t max_iter, double tol,
                            int *max_iter_exit);
int oracle_pcg_f32(const float *S, const float *Pinv, const float *gamma, float *lambda,
                   uint32_t n, uint32_t N, uint32_t max_iter, double tol, uint32_t flags,
                   uint32_t *iters, double *eta, double *rr);
int oracle_pcg_f64(const double *S, const double *Pinv, const double *gamma, double *lambda,
                   uint32_t n, uint32_t N, uint32_t max_iter, double tol, uint32_t flags,
                   uint32_t *iters, double *eta, double *rr);
int oracle_pcg_cg1_f32(const float *S, const float *Pinv, const float *gamma, float *lambda,
                       uint32_t n, uint32_t N, uint32_t max_iter, double tol, uint32_t flags,
                       uint32_t *iters, double *eta, double *rr);
int oracle_pcg_cg1_f64(const double *S, const double *Pinv, const double *gamma, double *lambda,
                       uint32_t n, uint32_t N, uint32_t max_iter, double tol, uint32_t flags,
                       uint32_t *iters, double *eta, double *rr);
void oracle_matvec_f32(double *y, const float *S, const float *x, uint32_t n, uint32_t N);
void oracle_matvec_f64(double *y, const double *S, const double *x, uint32_t n, uint32_t N);
int oracle_pcg_batch(oracle_system *sys, uint32_t count, int is_f64, uint32_t flags,
                     int nthreads);

#ifdef __cplusplus
}
#endif
