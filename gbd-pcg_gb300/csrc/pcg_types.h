// Device/host shared descriptors of the GB300 PCG solver.
//
// A "system" is one block-tridiagonal Schur-complement system S lambda = gamma
// with n x n blocks on N knots, stored in the compressed block-tridiagonal
// (cbtd) layout of the reference (include/pcg.cuh:104-110,
// include/utils.cuh:62,71,80): per knot k one n x 3n column-major block row
// [S_{k,k-1} | S_{k,k} | S_{k,k+1}], element (r, c) at k*3n^2 + c*n + r.
// The preconditioner Phi^-1 is either in the same layout (block-tridiagonal)
// or compact block-diagonal (n^2 per knot, column-major).
#pragma once
#include <stdint.h>

namespace gbdpcg {

enum : uint32_t {
    SYS_EXIT_RELRES = 1u,     // exit on ||r||_2 <= tol ||gamma||_2 (recursive residual)
    SYS_PINV_TRI = 2u,        // Phi^-1 stored as cbtd (3n^2 per knot), else compact
    SYS_ADJOINT = 4u,         // epilogue writes dS = -1/2 (mu lam^T + lam mu^T) and dgamma = mu
    SYS_LAMBDA0_ZERO = 8u,    // initial guess is zero (lambda0 pointer unused)
    SYS_REFINE = 16u,         // FP64 outer iterative refinement around the PCG
    SYS_FWD_ADJ = 32u,        // forward solve, then in the same launch the adjoint solve
                              // S mu = lambda - lambda* and the dS, dgamma epilogue
};

enum : int32_t {
    ST_CONVERGED = 0,
    ST_MAX_ITER = 1,
    ST_BREAKDOWN = 2,          // non-finite p.Sp or r.z
    ST_TIMEOUT = 3,            // a cluster reduction's wait gave up (about a second); results invalid
};

// One system of a work list.  All pointers are device pointers; element type is
// the launch's T (refinement: S, gamma and lambda are double, Pinv is float).
struct SysDesc {
    const void *S;        // cbtd, 3 n^2 N
    const void *P;        // Phi^-1, cbtd or compact
    const void *gamma;    // n N right-hand side
    const void *lambda0;  // n N initial guess (ignored with SYS_LAMBDA0_ZERO)
    void *lambda;         // n N solution (may alias lambda0)
    const void *lam_fwd;  // adjoint: forward solution lambda (n N)
    void *dS;             // adjoint: dL/dS in cbtd layout (3 n^2 N)
    double tol;           // exit tolerance (reference test or relative residual)
    double inner_tol;     // refinement: relative residual of each inner solve
    uint32_t n, N;
    uint32_t max_iter;    // PCG iterations (refinement: total inner iterations)
    uint32_t flags;
    uint32_t result;      // index into the result array
    uint32_t max_outer;   // refinement: outer steps
    const void *lstar;    // forward + adjoint: lambda* of L = 1/2 ||lambda - lambda*||^2
    void *mu;             // forward + adjoint: dL/dgamma = mu (n N)
    uint32_t result_adj;  // forward + adjoint: index of the adjoint solve's result
    uint32_t pad_;
};

struct SysResult {
    uint32_t iters;       // PCG iterations (reference counting: the converging pass counts)
    int32_t status;
    double eta;           // last r^T Phi^-1 r
    double rr;            // last ||r||^2 (recursive residual)
    double gg;            // ||gamma||^2
    uint32_t outer;       // refinement: outer steps taken
    uint32_t pad;
};

// Timeline record of one system in one launch (globaltimer nanoseconds),
// written by the leading thread of the cluster that solved it when a launch
// is given a stamp array.  Layout equals gbdpcg_stamp of gbdpcg.h.
struct StampRec {
    uint64_t t_pop;     // the cluster took the system from the work list
    uint64_t t_staged;  // its rows are on chip (the leading CTA's view)
    uint64_t t_solved;  // the PCG loop has ended
    uint64_t t_done;    // outputs (and any epilogue) written
    uint32_t system;    // index of the system in the plan
    uint32_t launch;    // launch (class) index
    uint32_t cluster;   // cluster index within the launch's grid
    uint32_t iters;
};

// Launch-wide parameters of the persistent cluster kernel.
struct LaunchParams {
    const SysDesc *descs;    // null: the single system `one` (passed by value)
    const uint32_t *order;   // work list: indices into descs, longest first
    uint32_t count;
    uint32_t kmax;           // knots per CTA the shared memory is sized for
    uint32_t *queue;         // work-queue head (zeroed before the launch); null: static
                             // round-robin of items over clusters
    SysResult *results;
    StampRec *stamps;        // null: no timeline; else one record per work-list item
    uint32_t *cta_sm;        // null, or the SM of every CTA of the grid (blockIdx.x order)
    uint32_t launch_id;      // launch index written into the stamps
    uint32_t pad_;
    SysDesc one;
};

}  // namespace gbdpcg
