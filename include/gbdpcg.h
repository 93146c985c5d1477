/*
 * gbdpcg — C ABI of the GB300 (sm_103a) PCG solver for the block-tridiagonal
 * Schur-complement systems  Phi^-1 S lambda = Phi^-1 gamma  of optimal control.
 *
 * It is the drop-in boundary for the reference's PCG path (Sdevaud/GBD-PCG):
 * the C++ templates of the reference's interface (solvePCG, pcg_solve,
 * pcg_config — see gpu_pcg.cuh in this directory) are inline wrappers over
 * these entry points.  Plain pointers and sizes only; every call returns a
 * status code (the reference exits the process instead,
 * include/gpuassert.cuh:5-14).
 *
 * Data layout (the reference's, include/pcg.cuh:104-110 and
 * include/utils.cuh:62,71,80): S and a block-tridiagonal Phi^-1 are
 * "compressed block-tridiagonal" (cbtd) arrays of N block rows, each an n x 3n
 * column-major matrix [S_{k,k-1} | S_{k,k} | S_{k,k+1}], element (r, c) of
 * block row k at k*3n^2 + c*n + r.  The blocks S_{0,-1} and S_{N-1,N} are
 * present as padding and never read.  A block-diagonal Phi^-1 may instead be
 * given compactly: n^2 per knot, column-major.  Vectors are n*N, knot-major.
 *
 * Supported sizes: 1 <= n <= 32 on the cluster solver: with the rows on chip
 * up to what 16 CTAs hold, with streamed rows up to the knots whose vectors
 * (three per knot) fit 16 CTAs' shared memory (n = 14 FP32: about 21000 knots;
 * n = 24 FP64: about 6000); larger n runs the plain algorithm (one CTA per
 * knot, all N co-resident); past those a call returns GBDPCG_ERR_UNSUPPORTED
 * before launching anything.
 *
 * Groups of entry points: single solves (host arrays, device pointers),
 * batched plans (graph replay, autotuner and its table, end-to-end pipelines
 * from host memory), the block-Jacobi builder, the adjoint, FP32 + FP64
 * refinement, an allocation-free solve, input adapters (CSR and dense to
 * cbtd), and the steps either side of the solve in a trajectory optimiser
 * (Schur-complement formation, optionally with the block-Jacobi Phi^-1, and
 * KKT back-substitution).
 */
#ifndef GBDPCG_H
#define GBDPCG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBDPCG_VERSION 1000

#if defined(__GNUC__)
#define GBDPCG_API __attribute__((visibility("default")))
#else
#define GBDPCG_API
#endif

/* ---- return codes of the API calls ---- */
typedef enum {
    GBDPCG_SUCCESS = 0,
    GBDPCG_ERR_INVALID_ARGUMENT = 1, /* null pointer, zero size, bad enum */
    GBDPCG_ERR_UNSUPPORTED = 2,      /* size or option combination not supported */
    GBDPCG_ERR_CUDA = 3,             /* a CUDA call failed; see gbdpcg_last_error() */
    GBDPCG_ERR_NO_MEMORY = 4,
    GBDPCG_ERR_NOT_CONVERGED = 5     /* a solve ended without meeting its exit test; the C ABI
                                        reports that per system (gbdpcg_result.status) and the
                                        C++ drop-in (gpu_pcg.cuh) raises this code for it when
                                        built with GBDPCG_ERROR_ON_MAX_ITER */
} gbdpcg_status;

/* ---- per-system outcome (gbdpcg_result.status) ---- */
enum {
    GBDPCG_CONVERGED = 0,   /* exit test met */
    GBDPCG_MAX_ITER = 1,    /* pcg_max_iter passes without meeting it (the reference's
                               d_max_iter_exit, include/pcg.cuh:101,212) */
    GBDPCG_BREAKDOWN = 2,   /* p^T S p or r^T Phi^-1 r not finite */
    GBDPCG_TIMEOUT = 3,     /* a wait inside the cluster solver's reductions gave up after about a
                               second; the system's outputs are not valid */
    GBDPCG_REJECTED = -1    /* the system did not fit the launch it was planned into */
};

/* exit criterion */
enum {
    GBDPCG_EXIT_REFERENCE = 0, /* |r^T Phi^-1 r| < exit_tol   (include/pcg.cuh:195) */
    GBDPCG_EXIT_RELRES = 1     /* ||r||_2 <= exit_tol ||gamma||_2 (recursive residual) */
};
/* Phi^-1 storage */
enum { GBDPCG_PINV_CBTD = 0, GBDPCG_PINV_BLOCKDIAG = 1 };
/* algorithm */
enum {
    GBDPCG_ALGO_AUTO = 0,    /* cluster solver when n <= 32, else plain */
    GBDPCG_ALGO_CLUSTER = 1, /* one thread-block cluster per system, DSMEM halos */
    GBDPCG_ALGO_PLAIN = 2,   /* one CTA per knot, grid-wide barriers (the reference's scheme) */
    GBDPCG_ALGO_SINGLE_REDUCTION = 3, /* cluster solver, Chronopoulos-Gear recurrences: one
                                         cluster-wide reduction per iteration; block-diagonal
                                         Phi^-1 only; iterates differ at roundoff level */
    GBDPCG_ALGO_RECURRENCE = 4 /* cluster solver with S p carried by a recurrence: three
                                  barriers per iteration instead of four; iterates differ at
                                  roundoff level */
};
/* dot-product accumulation for float systems (and for the FP32 inner solve of
 * a refined FP64 system, where NATIVE means FP64) */
enum {
    GBDPCG_DOT_NATIVE = 0,
    GBDPCG_DOT_FP64 = 1,  /* double */
    GBDPCG_DOT_FLOAT2 = 2 /* float-float: exact products, double-word sums with a 48-bit
                             significand, on the FP32 pipe (GB300's FP64 rate is a small
                             fraction of its FP32 rate); not with SINGLE_REDUCTION */
};
/* where the cluster solver keeps the matrix rows: AUTO picks; REGISTERS: S and
 * Phi^-1 rows in registers; SHARED: both staged in shared memory; SPLIT: S rows
 * in registers (two per thread for even n), Phi^-1 in shared memory; HYBRID:
 * the sub-diagonal and diagonal blocks of S in registers, its super-diagonal
 * block and Phi^-1 in shared memory (more rows per SM; FP32, block-diagonal
 * Phi^-1); TMEM: the diagonal block of S in registers, its off-diagonal
 * blocks in the SM's tensor memory, Phi^-1 in shared memory (the most rows
 * per SM; FP32, block-diagonal Phi^-1, even n; one CTA per SM); STREAM: no
 * storage, the rows are read from global memory (L2 or HBM) in every
 * product, so a cluster holds any system whose vectors fit its shared memory
 * (three vectors of its knots; AUTO's last choice before the plain algorithm) */
enum {
    GBDPCG_STORAGE_AUTO = 0,
    GBDPCG_STORAGE_REGISTERS = 1,
    GBDPCG_STORAGE_SHARED = 2,
    GBDPCG_STORAGE_SPLIT = 3,
    GBDPCG_STORAGE_HYBRID = 4,
    GBDPCG_STORAGE_TMEM = 5,
    GBDPCG_STORAGE_STREAM = 6
};

typedef struct {
    double exit_tol;         /* pcg_exit_tol, default 1e-6 (include/constants.cuh:17) */
    uint32_t max_iter;       /* pcg_max_iter, default 25  (include/constants.cuh:15) */
    uint32_t exit_mode;      /* GBDPCG_EXIT_*, default REFERENCE */
    uint32_t dot_precision;  /* GBDPCG_DOT_*, default NATIVE */
    uint32_t algorithm;      /* GBDPCG_ALGO_*, default AUTO */
    uint32_t cluster_size;   /* 0 = chosen by the tuner, else 1..16 CTAs per system */
    uint32_t max_threads;    /* 0 = chosen by the tuner, else a cap on threads per CTA */
    uint32_t storage;        /* GBDPCG_STORAGE_* */
    uint32_t use_graph;      /* plans: capture the launches in a CUDA graph (default 1) */
    uint32_t zero_guess;     /* 1: start from lambda = 0 and do not read lambda (default 0) */
    uint32_t max_outer;      /* refinement: outer steps (default 50) */
    uint32_t streams;        /* plans: streams the launches of one execution spread over (default 8) */
    uint32_t host_pieces;    /* packed plans: pieces gbdpcg_plan_execute_host pipelines (copies of
                                piece i+1 overlap the solve of piece i); 0 = automatic (about 512
                                systems a piece, at most 8), 1 = none */
    double inner_tol;        /* refinement: relative residual of each FP32 inner solve (default 0.05) */
} gbdpcg_config;

typedef struct {
    uint32_t iters;        /* PCG passes, the converging one included (include/pcg.cuh:195) */
    int32_t status;        /* GBDPCG_CONVERGED / _MAX_ITER / _BREAKDOWN / _REJECTED */
    double eta;            /* last r^T Phi^-1 r */
    double relres;         /* ||r||/||gamma||: recursive residual, or the true FP64 residual of
                              a refined solve (-1 if not tracked) */
    uint32_t outer;        /* refinement: outer steps taken (0 otherwise) */
    uint32_t reserved;
} gbdpcg_result;

/* One system of a batch.  Device pointers, element type of the batch.
 * Forward solve: lambda is in/out (initial guess, solution).
 * Adjoint solve: gamma = dL/dlambda, lambda = dL/dgamma (out), lambda_fwd = the
 * forward solution, dS = dL/dS (out, cbtd).  lambda_fwd and dS are NULL for a
 * forward solve. */
typedef struct {
    const void *S;
    const void *Pinv;
    const void *gamma;
    void *lambda;
    const void *lambda_fwd;
    void *dS;
    uint32_t n;
    uint32_t N;
} gbdpcg_system;

typedef struct gbdpcg_handle_s *gbdpcg_handle_t;
typedef struct gbdpcg_plan_s *gbdpcg_plan_t;
typedef void *gbdpcg_stream_t; /* a cudaStream_t; NULL is the legacy default stream */

GBDPCG_API int gbdpcg_version(void);
GBDPCG_API const char *gbdpcg_status_string(int status);
/* Message of the last failed call on this thread. */
GBDPCG_API const char *gbdpcg_last_error(void);
/* Defaults of pcg_config (include/types.cuh:18-34, include/constants.cuh:14-20). */
GBDPCG_API void gbdpcg_config_init(gbdpcg_config *cfg);

/* Handle: device, workspace, tuning table, launch cache.  One per thread of use. */
GBDPCG_API int gbdpcg_create(gbdpcg_handle_t *handle, int device);
GBDPCG_API int gbdpcg_destroy(gbdpcg_handle_t handle);

/* Host-pointer solve of one system; synchronous.  Replaces the host overload
 * solvePCG(h_S, h_Pinv, h_gamma, h_lambda, stateSize, knotPoints, config)
 * (include/interface.cuh:24-91).  Pinv is a cbtd array, or NULL to build the
 * block-Jacobi preconditioner on the GPU (the reference's documented
 * pcg_solve(S, gamma, lambda, ...) without Pinv, README.md:42).  S, Pinv and
 * gamma are not written (the reference copies them back, interface.cuh:77,79).
 * lambda is the initial guess on entry and the solution on return.  Uses a
 * per-thread handle on the current device. */
GBDPCG_API int gbdpcg_solve_f32(const float *S, const float *Pinv, const float *gamma, float *lambda,
                     uint32_t n, uint32_t N, const gbdpcg_config *cfg, gbdpcg_result *result);
GBDPCG_API int gbdpcg_solve_f64(const double *S, const double *Pinv, const double *gamma, double *lambda,
                     uint32_t n, uint32_t N, const gbdpcg_config *cfg, gbdpcg_result *result);

/* Device-pointer solve of one system, stream-ordered.  Replaces the device
 * overload solvePCG(state_size, knot_points, d_S, d_Pinv, d_gamma, d_lambda,
 * d_r, d_p, d_v_temp, d_eta_new_temp, config) (include/interface.cuh:94-146);
 * the cluster solver keeps r and p on chip, so no scratch is passed.  If
 * `result` is non-NULL the call waits for the stream and fills it; else the
 * result stays on the device (gbdpcg_last_result). */
GBDPCG_API int gbdpcg_solve_dev_f32(gbdpcg_handle_t h, const float *d_S, const float *d_Pinv,
                         uint32_t pinv_layout, const float *d_gamma, float *d_lambda, uint32_t n,
                         uint32_t N, const gbdpcg_config *cfg, gbdpcg_result *result,
                         gbdpcg_stream_t stream);
GBDPCG_API int gbdpcg_solve_dev_f64(gbdpcg_handle_t h, const double *d_S, const double *d_Pinv,
                         uint32_t pinv_layout, const double *d_gamma, double *d_lambda,
                         uint32_t n, uint32_t N, const gbdpcg_config *cfg,
                         gbdpcg_result *result, gbdpcg_stream_t stream);
/* Waits for the last device-pointer solve of this handle and returns its result. */
GBDPCG_API int gbdpcg_last_result(gbdpcg_handle_t h, gbdpcg_result *result);

/* Allocation-free solve of one FP32 system (no counterpart in the reference).
 * For callers that must not allocate device memory while they run: a
 * controller solving at a fixed rate, where an allocation in the loop costs
 * unbounded time; a process whose device memory another allocator already
 * owns; deployments that forbid allocation after start-up.  It runs the plain
 * algorithm (one CTA per knot, the reference's arithmetic order; cbtd Pinv)
 * with its scratch in one array of about 1 MiB compiled into the library's
 * device code.  CUDA loads that code into a device lazily, so the first call
 * on each device is what loads it and reserves the array there, and that call
 * can fail for want of device memory: make it at start-up, as a warm-up,
 * before other allocators take the memory and before any stream capture.
 * From then on the device holds the array until the process exits.  Every
 * call looks up the array's device address (cudaGetSymbolAddress, no
 * allocation) with the calling device current.  Limits: n*N <=
 * GBDPCG_NOALLOC_MAX_ELEMS and N <= GBDPCG_NOALLOC_MAX_KNOTS, else
 * GBDPCG_ERR_UNSUPPORTED.  The config is checked like the handle entry
 * points' configs.  No handle, no cudaMalloc/cudaFree.  Calls share the
 * array: calls that overlap on the GPU race.  If `result` is non-NULL the
 * call waits for the stream and fills it. */
#define GBDPCG_NOALLOC_MAX_ELEMS 131072
#define GBDPCG_NOALLOC_MAX_KNOTS 4096
GBDPCG_API int gbdpcg_solve_plain_noalloc_f32(const float *d_S, const float *d_Pinv,
                                              const float *d_gamma, float *d_lambda, uint32_t n,
                                              uint32_t N, const gbdpcg_config *cfg,
                                              gbdpcg_result *result, gbdpcg_stream_t stream);

/* FP64 solve by FP32 PCG with FP64 iterative refinement (no reference
 * counterpart).  S, gamma, lambda are double; Pinv is a compact block-diagonal
 * FP32 Phi^-1 (gbdpcg_block_jacobi_f64to32).  One persistent cluster kernel:
 * the rows of S are rounded to FP32 once and held on chip; each outer step
 * forms the true residual gamma - S lambda in FP64, solves the correction with
 * FP32 PCG (FP64 dot accumulation) to cfg->inner_tol relative residual, and
 * adds it in FP64; it stops when ||gamma - S lambda|| <= cfg->exit_tol ||gamma||
 * (exit_mode must be GBDPCG_EXIT_RELRES) or after cfg->max_iter inner passes /
 * cfg->max_outer outer steps.  result->iters counts inner passes. */
GBDPCG_API int gbdpcg_refine_solve_dev(gbdpcg_handle_t h, const double *d_S, const float *d_Pinv,
                                       const double *d_gamma, double *d_lambda, uint32_t n,
                                       uint32_t N, const gbdpcg_config *cfg,
                                       gbdpcg_result *result, gbdpcg_stream_t stream);
/* FP32 block-Jacobi Phi^-1 (compact) of an FP64 cbtd S, computed in FP64. */
GBDPCG_API int gbdpcg_block_jacobi_f64to32(gbdpcg_handle_t h, const double *d_S, float *d_Pinv,
                                           uint32_t n, uint32_t N, gbdpcg_stream_t stream);

/* Block-Jacobi preconditioner Phi^-1 = blockdiag(S_kk^-1) of a cbtd S, on the
 * GPU, in cbtd or compact layout; stream-ordered.  No reference counterpart:
 * the reference takes Phi^-1 from its caller. */
GBDPCG_API int gbdpcg_block_jacobi_f32(gbdpcg_handle_t h, const float *d_S, float *d_Pinv,
                            uint32_t pinv_layout, uint32_t n, uint32_t N,
                            gbdpcg_stream_t stream);
GBDPCG_API int gbdpcg_block_jacobi_f64(gbdpcg_handle_t h, const double *d_S, double *d_Pinv,
                            uint32_t pinv_layout, uint32_t n, uint32_t N,
                            gbdpcg_stream_t stream);

/* Adjoint of one solve S lambda = gamma (S symmetric): solves S mu = dL/dlambda
 * with the same PCG and writes dL/dgamma = mu and the block-tridiagonal
 * dL/dS = -1/2 (mu_i lambda_j^T + lambda_i mu_j^T) in cbtd layout (padding
 * blocks zero).  No reference counterpart. */
GBDPCG_API int gbdpcg_adjoint_dev_f32(gbdpcg_handle_t h, const float *d_S, const float *d_Pinv,
                           uint32_t pinv_layout, const float *d_lambda, const float *d_grad_lambda,
                           float *d_grad_gamma, float *d_grad_S, uint32_t n, uint32_t N,
                           const gbdpcg_config *cfg, gbdpcg_result *result,
                           gbdpcg_stream_t stream);

/* Batched solve of many independent systems of mixed n and N in persistent
 * cluster launches fed by device work queues (longest first), captured in one
 * CUDA graph.  No reference counterpart: the reference solves one system per
 * call.  `dtype` is 0 for float, 1 for double, 2 for FP64 systems solved by FP32
 * PCG with FP64 refinement (S, gamma, lambda double; Pinv compact FP32; see
 * gbdpcg_refine_solve_dev).  `systems` is a host array of
 * device pointers; all systems of a plan share pinv_layout and whether they
 * are adjoint solves (lambda_fwd != NULL).  The plan keeps the pointers: re-
 * executing it re-solves whatever the buffers hold. */
GBDPCG_API int gbdpcg_plan_create(gbdpcg_handle_t h, int dtype, const gbdpcg_system *systems, uint32_t count,
                       uint32_t pinv_layout, const gbdpcg_config *cfg, gbdpcg_plan_t *plan);
GBDPCG_API int gbdpcg_plan_execute(gbdpcg_plan_t plan, gbdpcg_stream_t stream);

/* Forward solve and adjoint of the loss L = 1/2 ||lambda - lambda*||^2 in one
 * launch (no reference counterpart).  Each cluster solves S lambda = gamma,
 * writes lambda, then, with the matrix rows still on chip, solves the adjoint
 * system S mu = lambda - lambda* (S is symmetric) from mu = 0 and writes
 * dL/dgamma = mu and the block-tridiagonal dL/dS = -1/2 (mu_i lambda_j^T +
 * lambda_i mu_j^T) in cbtd layout: the same results as a forward plan
 * followed by an adjoint plan (gbdpcg_system.lambda_fwd), without staging the
 * rows twice.  FP32 systems (dtype 0), device pointers.  The plan reports
 * 2 count results (gbdpcg_plan_results): the forward solves', then the
 * adjoint solves'.  Systems must fit the on-chip storages (else
 * GBDPCG_ERR_UNSUPPORTED). */
typedef struct {
    const void *S;
    const void *Pinv;
    const void *gamma;
    void *lambda;              /* forward solution (out; the initial guess unless cfg->zero_guess) */
    const void *lambda_target; /* lambda* */
    void *grad_gamma;          /* dL/dgamma = mu (out) */
    void *grad_S;              /* dL/dS, cbtd, padding blocks zero (out) */
    uint32_t n;
    uint32_t N;
} gbdpcg_fwd_adj_system;
GBDPCG_API int gbdpcg_plan_create_fwd_adj(gbdpcg_handle_t h, int dtype, const gbdpcg_fwd_adj_system *systems,
                                          uint32_t count, uint32_t pinv_layout, const gbdpcg_config *cfg,
                                          gbdpcg_plan_t *plan);

/* Split of one batch of independent systems over `parts` GPUs or ranks (no
 * reference counterpart: the reference solves one system per call; this is
 * the batch-level split of a multi-GPU deployment).  System i is estimated to
 * cost n[i]^2 N[i] iters[i] (iters NULL: 1 each); systems go, in decreasing
 * cost, to the part with the least cost so far (ties: the lowest index).
 * Writes part_of[count] and, if non-NULL, part_cost[parts].  Host code only:
 * no CUDA call, no GPU needed.  Each part is then solved by its own plan on
 * its own device, with no exchange of data between parts, and the results are
 * gathered in input order by the caller. */
GBDPCG_API int gbdpcg_partition(const uint32_t *n, const uint32_t *N, const float *iters, uint32_t count,
                                uint32_t parts, uint32_t *part_of, double *part_cost);

/* A system of a packed batch: element offsets into four device arenas
 * (S, Pinv, gamma, lambda; gamma and lambda share vec_off). */
typedef struct {
    uint32_t n;
    uint32_t N;
    uint64_t S_off;
    uint64_t Pinv_off;
    uint64_t vec_off;
} gbdpcg_packed_system;

/* Plan over packed device arenas (what a caller that keeps the batch in a few
 * large buffers uses).  The arena sizes are those the offsets reach. */
GBDPCG_API int gbdpcg_plan_create_packed(gbdpcg_handle_t h, int dtype,
                                         const gbdpcg_packed_system *systems, uint32_t count,
                                         const void *d_S, const void *d_Pinv, const void *d_gamma,
                                         void *d_lambda, uint32_t pinv_layout,
                                         const gbdpcg_config *cfg, gbdpcg_plan_t *plan);
/* End-to-end solve of a packed plan from host arenas: copies S, Pinv, gamma
 * (each skipped when NULL) host to device, executes, copies lambda (and, if
 * non-NULL, the per-system results) back, and waits.  Pinned host memory
 * makes the copies asynchronous DMA.  When the arenas hold the systems in
 * index order (offsets increasing), the batch is cut into pieces of
 * consecutive systems (config host_pieces): the copy of piece i+1 overlaps
 * the solve of piece i, and the solves of consecutive pieces overlap each
 * other, so the step costs about the copies plus the last piece's solve. */
GBDPCG_API int gbdpcg_plan_execute_host(gbdpcg_plan_t plan, const void *h_S, const void *h_Pinv,
                                        const void *h_gamma, void *h_lambda,
                                        gbdpcg_result *h_results, gbdpcg_stream_t stream);
/* Batched counterpart of the reference's documented pcg_solve(S, gamma,
 * lambda, stateSize, knotPoints, config) (README.md:42), which takes no Phi^-1:
 * copies S and gamma of a packed plan from the host, builds each system's
 * block-Jacobi Phi^-1 on the device into the plan's Pinv arena, solves, copies
 * lambda (and, if non-NULL, the results) back, and waits.  Pipelined in pieces
 * like gbdpcg_plan_execute_host (each piece's Phi^-1 is built right after its
 * copy).  n <= 32. */
GBDPCG_API int gbdpcg_plan_solve_host(gbdpcg_plan_t plan, const void *h_S, const void *h_gamma, void *h_lambda,
                                      gbdpcg_result *h_results, gbdpcg_stream_t stream);
/* Builds every system's block-Jacobi Phi^-1 into its Pinv pointer (stream-ordered). */
GBDPCG_API int gbdpcg_plan_build_block_jacobi(gbdpcg_plan_t plan, gbdpcg_stream_t stream);
/* Waits for the stream and copies the plan's results out: `count` of them
 * (2 count for a forward + adjoint plan). */
GBDPCG_API int gbdpcg_plan_results(gbdpcg_plan_t plan, gbdpcg_result *results, gbdpcg_stream_t stream);
/* Number of launches (cluster classes + plain systems) the plan makes per execution. */
GBDPCG_API int gbdpcg_plan_launch_count(gbdpcg_plan_t plan, uint32_t *launches);
/* Describes launch i: cluster size, threads per CTA, knots per CTA, systems, CTAs in the grid. */
GBDPCG_API int gbdpcg_plan_launch_info(gbdpcg_plan_t plan, uint32_t i, uint32_t *cluster, uint32_t *threads,
                            uint32_t *kmax, uint32_t *systems, uint32_t *ctas);
/* CSR -> cbtd on the device: the adapter behind the reference's solvePCG
 * overload for csr_t matrices (include/interface.cuh:8-20, whose body exits
 * with "NOT IMPLEMENTED"; csr_t at include/types.cuh:7-15).  A CSR matrix with
 * n N rows and columns (row_ptr: n N + 1 entries) whose entries lie in the
 * three diagonal blocks of their block row is scattered into d_out (3 n^2 N
 * elements, zeroed first; duplicates add).  d_err is one device word the call
 * uses as scratch.  Synchronous; an entry outside the band returns
 * GBDPCG_ERR_INVALID_ARGUMENT (the other entries are written). */
GBDPCG_API int gbdpcg_csr_to_cbtd_f32(const uint32_t *d_row_ptr, const uint32_t *d_col_ind, const float *d_val,
                                      uint32_t n, uint32_t N, float *d_out, uint32_t *d_err, gbdpcg_stream_t stream);
GBDPCG_API int gbdpcg_csr_to_cbtd_f64(const uint32_t *d_row_ptr, const uint32_t *d_col_ind, const double *d_val,
                                      uint32_t n, uint32_t N, double *d_out, uint32_t *d_err, gbdpcg_stream_t stream);
/* Dense -> cbtd on the device: the three diagonal blocks of every block row
 * of a dense n N x n N matrix (leading dimension ld >= n N; column-major, or
 * row-major when row_major != 0) into d_out (3 n^2 N elements; the padding
 * blocks of knots 0 and N-1 are written as zeros).  n <= 32.  With a non-NULL
 * d_err (one device word of scratch) the call also scans every entry outside
 * the band, waits, and returns GBDPCG_ERR_INVALID_ARGUMENT if one is nonzero;
 * with d_err NULL it is stream-ordered and checks nothing. */
GBDPCG_API int gbdpcg_dense_to_cbtd_f32(const float *d_D, uint64_t ld, int row_major, uint32_t n, uint32_t N,
                                        float *d_out, uint32_t *d_err, gbdpcg_stream_t stream);
GBDPCG_API int gbdpcg_dense_to_cbtd_f64(const double *d_D, uint64_t ld, int row_major, uint32_t n, uint32_t N,
                                        double *d_out, uint32_t *d_err, gbdpcg_stream_t stream);

/* The steps either side of the solve in a trajectory optimiser (no reference
 * counterpart: the callers of solvePCG in MPCGPU / GATO).  Problem: states
 * x_0..x_N (n), controls u_0..u_{N-1} (m), cost 1/2 z^T Theta z + g^T z with
 * Theta = blockdiag(diag(Qd_0)..diag(Qd_N), diag(Rd_0)..diag(Rd_{N-1})), g =
 * (q_0..q_N, r_0..r_{N-1}), constraints [A_k  B_k  -I] (x_k, u_k, x_{k+1}) = c_k,
 * KKT [Theta C^T; C 0][z; lambda] = [-g; c].  A_k (n x n) and B_k (n x m) are
 * column-major, knot-major.  n, m <= 32.  Stream-ordered.
 * form_schur: S = C Theta^-1 C^T (cbtd, N block rows) and gamma = -(c + C Theta^-1 g). */
GBDPCG_API int gbdpcg_form_schur_f32(const float *d_A, const float *d_B, const float *d_Qd, const float *d_Rd,
                                     const float *d_q, const float *d_r, const float *d_c, uint32_t n, uint32_t m,
                                     uint32_t N, float *d_S, float *d_gamma, gbdpcg_stream_t stream);
GBDPCG_API int gbdpcg_form_schur_f64(const double *d_A, const double *d_B, const double *d_Qd, const double *d_Rd,
                                     const double *d_q, const double *d_r, const double *d_c, uint32_t n, uint32_t m,
                                     uint32_t N, double *d_S, double *d_gamma, gbdpcg_stream_t stream);
/* form_schur_pinv: the same, and the block-Jacobi Phi^-1 = blockdiag(S_kk^-1)
 * (compact, n^2 per knot, column-major) from the same warp that formed S_kk:
 * bit for bit what gbdpcg_block_jacobi_* builds from the S written here, with
 * no second pass over S. */
GBDPCG_API int gbdpcg_form_schur_pinv_f32(const float *d_A, const float *d_B, const float *d_Qd, const float *d_Rd,
                                          const float *d_q, const float *d_r, const float *d_c, uint32_t n,
                                          uint32_t m, uint32_t N, float *d_S, float *d_gamma, float *d_Pinv,
                                          gbdpcg_stream_t stream);
GBDPCG_API int gbdpcg_form_schur_pinv_f64(const double *d_A, const double *d_B, const double *d_Qd,
                                          const double *d_Rd, const double *d_q, const double *d_r,
                                          const double *d_c, uint32_t n, uint32_t m, uint32_t N, double *d_S,
                                          double *d_gamma, double *d_Pinv, gbdpcg_stream_t stream);
/* kkt_backsub: z = -Theta^-1 (g + C^T lambda): x (n (N+1)) and u (m N). */
GBDPCG_API int gbdpcg_kkt_backsub_f32(const float *d_A, const float *d_B, const float *d_Qd, const float *d_Rd,
                                      const float *d_q, const float *d_r, const float *d_lambda, uint32_t n,
                                      uint32_t m, uint32_t N, float *d_x, float *d_u, gbdpcg_stream_t stream);
GBDPCG_API int gbdpcg_kkt_backsub_f64(const double *d_A, const double *d_B, const double *d_Qd, const double *d_Rd,
                                      const double *d_q, const double *d_r, const double *d_lambda, uint32_t n,
                                      uint32_t m, uint32_t N, double *d_x, double *d_u, gbdpcg_stream_t stream);

/* Kernel of launch i: storage (0 S and Phi^-1 in registers, 1 S in registers
 * and Phi^-1 in shared memory, 2 both in shared memory, 3 hybrid, 4 tensor memory), matrix rows per
 * thread, and algorithm (GBDPCG_ALGO_CLUSTER, _SINGLE_REDUCTION, _RECURRENCE,
 * or _PLAIN for a one-system plain launch; refinement launches report 0). */
GBDPCG_API int gbdpcg_plan_launch_kernel(gbdpcg_plan_t plan, uint32_t i, uint32_t *storage,
                                         uint32_t *rows_per_thread, uint32_t *algorithm);
GBDPCG_API int gbdpcg_plan_destroy(gbdpcg_plan_t plan);

/* Timeline of a plan's executions (no reference counterpart: measurement).
 * With the timeline on, every execution records for each system solved by a
 * cluster launch the GPU's global nanosecond clock (%globaltimer) at four
 * points, read by the leading thread of the cluster that solved it, and the
 * SM of every CTA of every launch.  It costs a few stores per system; the
 * launches are captured again when it is switched. */
typedef struct {
    uint64_t t_pop;     /* the cluster took the system from its launch's work list */
    uint64_t t_staged;  /* the system's matrix rows are on chip (the leading CTA's view) */
    uint64_t t_solved;  /* the PCG iteration has ended */
    uint64_t t_done;    /* lambda, the result and any adjoint output written */
    uint32_t system;    /* index of the system in the plan */
    uint32_t launch;    /* launch index (gbdpcg_plan_launch_info) */
    uint32_t cluster;   /* cluster of the launch's grid that solved it */
    uint32_t iters;     /* PCG passes (0: rejected by the launch) */
} gbdpcg_stamp;
GBDPCG_API int gbdpcg_plan_timeline(gbdpcg_plan_t plan, int enable);
/* Latency of the synchronisation primitives one cluster-solver iteration is
 * made of (no reference counterpart: measurement), on a grid of `clusters`
 * clusters of `cluster` CTAs of `threads` threads (clusters = 0: as many as
 * fit at once), each primitive repeated `reps` times in a dependent loop and
 * timed with CUDA events; nanoseconds per repetition, the loop's own cost
 * subtracted.  The cluster-barrier fields are 0 for cluster = 1.
 * Synchronous; allocates one word of device memory. */
typedef struct {
    double loop_ns;                 /* one repetition of the empty dependent loop */
    double syncthreads_ns;          /* __syncthreads */
    double cluster_barrier_ns;      /* barrier.cluster arrive (release) + wait (acquire) */
    double dsmem_store_barrier_ns;  /* one store into the next CTA's shared memory + the cluster barrier */
    double allreduce_ns[3];         /* cluster-wide reduction of 1, 2, 3 values behind a cluster barrier
                                       (the form of the single-reduction and refinement kernels) */
    double allreduce_tx_ns[3];      /* the same reduction by transaction-counted stores (st.async onto
                                       the receiving CTAs' mbarriers; the form of the cluster kernels
                                       for cluster >= 2; 0 for cluster = 1) */
} gbdpcg_probe;
GBDPCG_API int gbdpcg_probe_primitives(int device, uint32_t cluster, uint32_t threads, uint32_t clusters,
                                       uint32_t reps, gbdpcg_probe *out);
/* The cluster solver's failure path without a fault (no reference
 * counterpart: the reference's grid barriers wait without a limit): one
 * cluster of `cluster` CTAs (1..16) runs a wait that nothing completes, through
 * the solver's own bounded mbarrier wait (for cluster >= 2, a cluster-wide
 * reduction whose receivers also expect halo bytes no neighbour sends).  Every
 * CTA gives up after about a second; *status = GBDPCG_TIMEOUT when all of them
 * did (else the outcome of a CTA that did not), *waited_ms = the launch's
 * duration.  The context stays usable.  Synchronous; allocates `cluster`
 * words of device memory. */
GBDPCG_API int gbdpcg_probe_timeout(int device, uint32_t cluster, int *status, double *waited_ms);
/* Waits for the stream and copies the last execution's records (one per
 * system of the cluster launches, grouped by launch; at most `capacity`) and
 * the SM of each CTA (launch 0's CTAs first, in grid order; at most
 * `sm_capacity`).  *count and *sm_count receive the full sizes. */
GBDPCG_API int gbdpcg_plan_timeline_read(gbdpcg_plan_t plan, gbdpcg_stamp *stamps, uint32_t capacity,
                                         uint32_t *count, uint32_t *cta_sm, uint32_t sm_capacity,
                                         uint32_t *sm_count, gbdpcg_stream_t stream);

/* Autotuner (no reference counterpart: the reference fixes 64 threads per CTA
 * and one CTA per knot).  For every launch class of the plan it times, on the
 * plan's own systems, the class alone with each launch shape that holds all
 * of its systems — Phi^-1/S storage (registers, shared memory, split), rows
 * per thread, cluster size C (1-8, 16; every CTA owns at least one knot),
 * CTA size rounded to a warp — and keeps the fastest (a change must win by
 * more than 2%).  Classes that end up with the same shape are merged and the
 * plan's graph is rebuilt on its next execution.  Tuning solves from a zero
 * initial guess into scratch buffers: the plan's lambda, dS and results are
 * not written.  The choices are also stored in the handle's tuning table,
 * which later plans of the same handle use for systems of the same (n, N),
 * precision, Phi^-1 layout, algorithm and storage request when the config
 * leaves cluster_size and max_threads at 0.  `flags`: GBDPCG_TUNE_* bits.
 * `reps` timed launches per shape (0 means 2).  Synchronous. */
enum {
    GBDPCG_TUNE_RECURRENCE = 1,      /* with GBDPCG_ALGO_AUTO also try the recurrence form */
    GBDPCG_TUNE_SINGLE_REDUCTION = 2, /* with GBDPCG_ALGO_AUTO and a compact Phi^-1 also try the
                                         single-reduction (Chronopoulos-Gear) form */
    GBDPCG_TUNE_WHOLE_PLAN = 4        /* then time the whole plan as it runs (its classes side by
                                         side on the plan's streams, solving into scratch) and let
                                         each class, the longest first, take another of its shapes
                                         within 30% of its best alone when that makes the whole
                                         plan faster by more than 1% (forward plans of two or more
                                         classes) */
};
GBDPCG_API int gbdpcg_plan_autotune(gbdpcg_plan_t plan, uint32_t flags, uint32_t reps, gbdpcg_stream_t stream);
/* The handle's tuning table as text, one line per (n, N) entry:
 * "f64 refine acc64 ptri adjoint algorithm storage n N : st rpt alg C threads".
 * Writes at most `capacity` bytes including the terminating NUL and sets
 * *length to the full length without the NUL (call with capacity 0 to size). */
GBDPCG_API int gbdpcg_tune_export(gbdpcg_handle_t h, char *buffer, size_t capacity, size_t *length);
/* Adds the entries of a text produced by gbdpcg_tune_export (replacing equal
 * keys).  Entries naming a kernel variant this library does not contain are rejected. */
GBDPCG_API int gbdpcg_tune_import(gbdpcg_handle_t h, const char *text);
/* Empties the handle's tuning table. */
GBDPCG_API int gbdpcg_tune_clear(gbdpcg_handle_t h);

#ifdef __cplusplus
}
#endif

#endif /* GBDPCG_H */
