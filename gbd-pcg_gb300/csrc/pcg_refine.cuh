// FP32 PCG with FP64 iterative refinement, fused in one persistent cluster
// kernel (no reference counterpart: the reference is FP32 or FP64 throughout,
// include/pcg.cuh:54 `template <typename T, ...>`).
//
// Per system (one cluster, knots split over its CTAs as in pcg_cluster.cuh):
//   * the rows of S are converted once from the FP64 input to FP32 and held on
//     chip (registers or shared memory), Phi^-1 is FP32 block-diagonal;
//   * lambda and gamma stay FP64 in registers;
//   * outer step: r64 = gamma - S64 lambda64, with S64 read from global memory
//     (FP64 FMAs, lambda halo through DSMEM), ||r64|| reduced in FP64; stop when
//     ||r64|| <= tol ||gamma|| — the exit test is on the true FP64 residual;
//   * inner solve: PCG in FP32 on S32 d = (float)r64 from d = 0, to
//     ||r_inner|| <= inner_tol ||r64||, its dot products accumulated in AI:
//     double, or f2acc (float-float, on the FP32 pipe; see accum.cuh);
//   * lambda64 += d.
// Result: iters = inner PCG passes summed over the outer steps, outer = outer
// steps, rr = the final ||r64||^2.
#pragma once
#include "pcg_cluster.cuh"

namespace gbdpcg {

template <int NP, int ST>
struct SmemPlanRF {
    using Base = SmemPlan<float, double, NP, false, ST>;
    __host__ __device__ static size_t dwin(uint32_t kmax) {
        return round_up((size_t)(kmax + 2) * NP * sizeof(double), 32);
    }
    __host__ __device__ static size_t bytes(uint32_t kmax, uint32_t C, uint32_t nwarps) {
        return Base::bytes(kmax, C, nwarps) + dwin(kmax);
    }
};

template <int NP, int ST, int RPT, typename AI>
__global__ void __launch_bounds__((RegBudget<float, double, NP, false, ST, RPT>::max_threads), 1)
    pcg_refine_kernel(const LaunchParams lp) {
    using T = float;
    static_assert(sizeof(AI) == sizeof(double), "inner and outer reductions share the slot arrays");
    using Plan = SmemPlan<T, double, NP, false, ST>;
    constexpr bool S_REG = ST <= ST_REG_S, P_REG = ST == ST_REG;
    const cg::cluster_group cluster = cg::this_cluster();
    const uint32_t C = cluster.num_blocks();
    const uint32_t rank = cluster.block_rank();
    const uint32_t tid = threadIdx.x, nthr = blockDim.x;

    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *sp = smem_raw;
    T *vp = reinterpret_cast<T *>(sp); sp += Plan::vec(lp.kmax);
    T *vr = reinterpret_cast<T *>(sp); sp += Plan::vec(lp.kmax);
    T *uh = reinterpret_cast<T *>(sp); sp += Plan::halo();  // unused (block-diagonal Phi^-1)
    T *zh = reinterpret_cast<T *>(sp); sp += Plan::halo();
    double *slots64 = reinterpret_cast<double *>(sp); sp += Plan::slots(C);  // FP64 reductions
    double *wscr64 = reinterpret_cast<double *>(sp); sp += Plan::wscr(nthr >> 5);
    AI *slots = reinterpret_cast<AI *>(slots64);  // the same bytes for the inner reductions
    AI *wscr = reinterpret_cast<AI *>(wscr64);
    uint32_t *s_item = reinterpret_cast<uint32_t *>(sp); sp += kItemBytes;
    T *ms = reinterpret_cast<T *>(sp); sp += Plan::mat_s(lp.kmax);
    T *mp = reinterpret_cast<T *>(sp); sp += Plan::mat_p(lp.kmax);
    double *vd = reinterpret_cast<double *>(sp);  // FP64 lambda window
    (void)uh;
    const uint32_t zero_elems = (uint32_t)((2 * Plan::vec(lp.kmax) + 2 * Plan::halo()) / sizeof(T));
    const uint32_t zero_d = (uint32_t)(SmemPlanRF<NP, ST>::dwin(lp.kmax) / sizeof(double));

    for (uint32_t e = tid; e < (uint32_t)(Plan::slots(C) / sizeof(double)); e += nthr) slots64[e] = 0.0;
    for (uint32_t e = tid; e < (uint32_t)(kMaxValues * 32); e += nthr) wscr64[e] = 0.0;  // local slots
    const uint32_t cluster_id = blockIdx.x / C, nclusters = gridDim.x / C;
    Stamper stamp(lp, rank);
    for (uint32_t pass = 0;; ++pass) {
        uint32_t item;
        if (lp.queue) {
            if (rank == 0 && tid == 0) {
                const uint32_t it = atomicAdd(lp.queue, 1u);
                for (uint32_t c = 0; c < C; ++c) *cluster.map_shared_rank(s_item, c) = it;
            }
            group_sync(cluster, C);
            item = *reinterpret_cast<volatile uint32_t *>(s_item);
        } else {
            item = cluster_id + pass * nclusters;
            __syncthreads();
        }
        if (item >= lp.count) break;
        stamp.pop();
        const SysDesc d = lp.descs ? lp.descs[lp.order ? lp.order[item] : item] : lp.one;
        const uint32_t n = d.n, N = d.N;
        const uint32_t K = (N + C - 1) / C;
        if (n == 0 || N == 0 || n > (uint32_t)NP || K > lp.kmax || (size_t)K * n > (size_t)nthr * RPT ||
            (RPT > 1 && (n % RPT) != 0) || (d.flags & (SYS_PINV_TRI | SYS_ADJOINT | SYS_FWD_ADJ))) {
            if (rank == 0 && tid == 0) {
                SysResult res = {};
                res.status = -1;
                lp.results[d.result] = res;
            }
            stamp.rejected();
            stamp.done(lp, item, 0);
            group_sync(cluster, C);
            continue;
        }
        const uint32_t kb = min(rank * K, N), ke = min(kb + K, N), nk = ke - kb;
        const uint32_t row0 = tid * RPT;
        const uint32_t lk = row0 / n, i = row0 - lk * n;
        const bool act = lk < nk;
        const uint32_t k = kb + lk;
        const double *__restrict__ S64 = static_cast<const double *>(d.S);
        const T *__restrict__ P = static_cast<const T *>(d.P);
        const double *__restrict__ gamma = static_cast<const double *>(d.gamma);
        const double *__restrict__ lam0 =
            (d.flags & SYS_LAMBDA0_ZERO) ? nullptr : static_cast<const double *>(d.lambda0);
        const uint32_t blkS = 3 * n * n, blkP = n * n;
        const uint32_t R = (K * n + 1) & ~1u;  // row stride of staged matrices (even)
        const bool has_left = nk > 0 && kb > 0, has_right = nk > 0 && ke < N;
        const bool first_knot = act && lk == 0 && kb > 0, last_knot = act && lk + 1 == nk && ke < N;
        const int sb0 = (k == 0) ? 1 : 0, sb1 = (k + 1 == N) ? 2 : 3;
        if (tid == 0 && nk > 0) {  // this CTA's rows into L2 before they are staged
            prefetch_l2_range(S64 + (size_t)kb * blkS, (size_t)nk * blkS * sizeof(double));
            prefetch_l2_range(P + (size_t)kb * blkP, (size_t)nk * blkP * sizeof(T));
        }

        for (uint32_t e = tid; e < zero_elems; e += nthr) vp[e] = T(0);
        for (uint32_t e = tid; e < zero_d; e += nthr) vd[e] = 0.0;

        // ---- FP32 copies of the rows of S (converted once), FP32 Phi^-1
        T Sr[S_REG ? RPT : 1][S_REG ? 3 * NP : 1];
        T Pr[P_REG ? RPT : 1][P_REG ? NP : 1];
        if constexpr (S_REG) {
            const double *Sk = S64 + (size_t)k * blkS;
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                const bool present = act && (b != 0 || k > 0) && (b != 2 || k + 1 < N);
#pragma unroll
                for (int j = 0; j < NP; ++j)
#pragma unroll
                    for (int q = 0; q < RPT; ++q)
                        Sr[q][b * NP + j] = (present && (uint32_t)j < n)
                                                ? __double2float_rn(__ldg(Sk + (b * n + j) * n + i + q))
                                                : T(0);
            }
        } else {
            const double *Sg = S64 + (size_t)kb * blkS;
            stage_rows(ms, R, Sg, nk, n, blkS, tid, nthr);
        }
        if constexpr (P_REG) {
            const T *Pk = P + (size_t)k * blkP;
#pragma unroll
            for (int j = 0; j < NP; ++j)
#pragma unroll
                for (int q = 0; q < RPT; ++q)
                    Pr[q][j] = (act && (uint32_t)j < n) ? __ldg(Pk + j * n + i + q) : T(0);
        } else {
            const T *Pg = P + (size_t)kb * blkP;
            stage_rows(mp, R, Pg, nk, n, blkP, tid, nthr);
        }
        auto matS = [&](const T *x, T(&y)[RPT]) {
            if constexpr (S_REG) reg_matvec<T, NP, 3, RPT>(Sr, x, y);
            else smem_matvec<T, NP, 3, RPT>(ms, R, lk * n + i, sb0, sb1, x, n, y);
        };
        auto matP = [&](const T *x, T(&y)[RPT]) {
            if constexpr (P_REG) reg_matvec<T, NP, 1, RPT>(Pr, x + NP, y);
            else smem_matvec<T, NP, 1, RPT>(mp, R, lk * n + i, 0, 1, x + NP, n, y);
        };
        T *my_p = vp + (lk + 1) * NP + i;
        T *my_r = vr + (lk + 1) * NP + i;
        double *my_d = vd + (lk + 1) * NP + i;

        stage_wait();
        __syncthreads();  // rows staged
        stamp.staged();
        double gam[RPT], lam[RPT], r64[RPT];
#pragma unroll
        for (int q = 0; q < RPT; ++q) {
            gam[q] = act ? gamma[(size_t)k * n + i + q] : 0.0;
            lam[q] = (act && lam0) ? lam0[(size_t)k * n + i + q] : 0.0;
        }
        int buf = 0;
        double gg;
        {
            double v1[1] = {0.0};
#pragma unroll
            for (int q = 0; q < RPT; ++q) v1[0] = fma(gam[q], gam[q], v1[0]);
            cluster_allreduce<double, 1>(v1, slots64, wscr64, buf, cluster, C, rank);
            buf ^= 1;
            gg = v1[0];
        }
        const double thr_out = d.tol * d.tol * gg;
        const double inner_tol2 = d.inner_tol * d.inner_tol;
        uint32_t iters = 0, outer = 0;
        int32_t status = ST_MAX_ITER;
        double rr64 = 0.0;
        AI eta_last = AI(0);
        for (;;) {
            // ---- r64 = gamma - S64 lambda64 (FP64, S64 from global memory)
            if (act) {
#pragma unroll
                for (int q = 0; q < RPT; ++q) my_d[q] = lam[q];
            }
            if (first_knot) {
                double *dst = cluster.map_shared_rank(vd, rank - 1) + (K + 1) * NP + i;
#pragma unroll
                for (int q = 0; q < RPT; ++q) dst[q] = lam[q];
            }
            if (last_knot) {
                double *dst = cluster.map_shared_rank(vd, rank + 1) + i;
#pragma unroll
                for (int q = 0; q < RPT; ++q) dst[q] = lam[q];
            }
            group_sync(cluster, C);
            if (act) {
                const double *Srow = S64 + (size_t)k * blkS + i;
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    double acc = 0.0;
                    for (int b = sb0; b < sb1; ++b) {
                        const double *col = Srow + (size_t)b * n * n + q;
                        const double *x = vd + (lk + b) * NP;
                        for (uint32_t j = 0; j < n; ++j) acc = fma(__ldg(col + (size_t)j * n), x[j], acc);
                    }
                    r64[q] = gam[q] - acc;
                }
            } else {
#pragma unroll
                for (int q = 0; q < RPT; ++q) r64[q] = 0.0;
            }
            {
                double v1[1] = {0.0};
#pragma unroll
                for (int q = 0; q < RPT; ++q) v1[0] = fma(r64[q], r64[q], v1[0]);
                cluster_allreduce<double, 1>(v1, slots64, wscr64, buf, cluster, C, rank);
                buf ^= 1;
                rr64 = v1[0];
            }
            if (!isfinite(rr64)) { status = ST_BREAKDOWN; break; }
            if (rr64 <= thr_out) { status = ST_CONVERGED; break; }
            if (iters >= d.max_iter || outer >= d.max_outer) break;

            // ---- inner FP32 PCG on S dx = r64 from dx = 0
            T r[RPT], x[RPT], p[RPT], z[RPT], y[RPT];
#pragma unroll
            for (int q = 0; q < RPT; ++q) {
                r[q] = __double2float_rn(r64[q]);
                x[q] = T(0);
                if (act) my_r[q] = r[q];
            }
            __syncthreads();
            if (act) matP(vr + lk * NP, z);
            else {
#pragma unroll
                for (int q = 0; q < RPT; ++q) z[q] = T(0);
            }
#pragma unroll
            for (int q = 0; q < RPT; ++q) {
                p[q] = z[q];
                if (act) my_p[q] = p[q];
            }
            if (first_knot) {
                T *dst = cluster.map_shared_rank(vp, rank - 1) + (K + 1) * NP + i;
#pragma unroll
                for (int q = 0; q < RPT; ++q) dst[q] = z[q];
            }
            if (last_knot) {
                T *dst = cluster.map_shared_rank(vp, rank + 1) + i;
#pragma unroll
                for (int q = 0; q < RPT; ++q) dst[q] = z[q];
            }
            AI eta, rr_in0;
            {
                AI v2[2] = {AI(0), AI(0)};
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    acc_madd(v2[0], r[q], z[q]);
                    acc_madd(v2[1], r[q], r[q]);
                }
                cluster_allreduce<AI, 2>(v2, slots, wscr, buf, cluster, C, rank);
                buf ^= 1;
                eta = v2[0];
                rr_in0 = v2[1];
            }
            const AI thr_in = AI(inner_tol2 * (double)rr_in0);
            const uint32_t budget = d.max_iter - iters;
            uint32_t it = 0;
            bool broke = false;
            for (; it < budget;) {
                if (act) matS(vp + lk * NP, y);
                else {
#pragma unroll
                    for (int q = 0; q < RPT; ++q) y[q] = T(0);
                }
                AI pap;
                {
                    AI v1[1] = {AI(0)};
#pragma unroll
                    for (int q = 0; q < RPT; ++q) acc_madd(v1[0], p[q], y[q]);
                    cluster_allreduce<AI, 1>(v1, slots, wscr, buf, cluster, C, rank);
                    buf ^= 1;
                    pap = v1[0];
                }
                const T alpha = (pap == AI(0)) ? T(0) : acc_ratio<T>(eta, pap);
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    x[q] = fma_rn(alpha, p[q], x[q]);
                    r[q] = fma_rn(-alpha, y[q], r[q]);
                    if (act) my_r[q] = r[q];
                }
                __syncthreads();
                if (act) matP(vr + lk * NP, z);
                else {
#pragma unroll
                    for (int q = 0; q < RPT; ++q) z[q] = T(0);
                }
                if (first_knot) {
                    T *dst = cluster.map_shared_rank(zh, rank - 1) + NP + i;
#pragma unroll
                    for (int q = 0; q < RPT; ++q) dst[q] = z[q];
                }
                if (last_knot) {
                    T *dst = cluster.map_shared_rank(zh, rank + 1) + i;
#pragma unroll
                    for (int q = 0; q < RPT; ++q) dst[q] = z[q];
                }
                AI eta_new, rr;
                {
                    AI v2[2] = {AI(0), AI(0)};
#pragma unroll
                    for (int q = 0; q < RPT; ++q) {
                        acc_madd(v2[0], r[q], z[q]);
                        acc_madd(v2[1], r[q], r[q]);
                    }
                    cluster_allreduce<AI, 2>(v2, slots, wscr, buf, cluster, C, rank);
                    buf ^= 1;
                    eta_new = v2[0];
                    rr = v2[1];
                }
                ++it;
                eta_last = eta_new;
                if (!acc_finite(eta_new) || !acc_finite(pap)) { broke = true; break; }
                if (rr <= thr_in) break;
                const T beta = acc_ratio<T>(eta_new, eta);
                eta = eta_new;
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    p[q] = fma_rn(beta, p[q], z[q]);
                    if (act) my_p[q] = p[q];
                }
                for (uint32_t t = tid; t < 2 * n; t += nthr) {
                    if (t < n && has_left) vp[t] = fma_rn(beta, vp[t], zh[t]);
                    if (t >= n && has_right) {
                        T *h = vp + (nk + 1) * NP + (t - n);
                        *h = fma_rn(beta, *h, zh[NP + t - n]);
                    }
                }
                __syncthreads();
            }
            iters += it;
            ++outer;
            if (broke) { status = ST_BREAKDOWN; break; }
#pragma unroll
            for (int q = 0; q < RPT; ++q) lam[q] += (double)x[q];
        }

        stamp.solved();
        double *lam_out = static_cast<double *>(d.lambda);
        if (act) {
#pragma unroll
            for (int q = 0; q < RPT; ++q) lam_out[(size_t)k * n + i + q] = lam[q];
        }
        if (rank == 0 && tid == 0) {
            SysResult res;
            res.iters = iters;
            res.status = status;
            res.eta = (double)eta_last;
            res.rr = rr64;
            res.gg = gg;
            res.outer = outer;
            res.pad = 0;
            lp.results[d.result] = res;
        }
        stamp.done(lp, item, iters);
    }
}

}  // namespace gbdpcg
