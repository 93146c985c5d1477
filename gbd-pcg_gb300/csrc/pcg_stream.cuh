// Cluster PCG with streamed matrix rows (storage ST_STREAM): for systems whose
// rows do not fit on chip.  Same mapping, halos, reductions and arithmetic as
// pcg_cluster_kernel's standard form (include/pcg.cuh:154-208), except that
//   * the block rows of S and Phi^-1 are read from global memory (L2, or HBM)
//     in every matrix-vector product instead of being held in registers,
//     shared or tensor memory;
//   * a thread owns one slot of RPT rows in each of G row groups (slot g*nthr +
//     tid, G = ceil(rows of the CTA / (RPT nthr))), so a CTA holds any number
//     of knots whose vectors fit its shared memory: the p and r windows (with
//     one halo knot on each side) and one more vector (S p, then Phi^-1 r) live
//     there, lambda lives in its output array and is updated in place;
//   * the dot-product partials of a thread run over its groups in order.
// With one group the products, updates and reductions are those of the
// shared-memory storage (ST_SMEM) at the same cluster and CTA size, in the
// same order, so the two agree bit for bit.  The adjoint epilogue is the
// cluster kernel's, over the row groups.
#pragma once
#include "pcg_cluster.cuh"

namespace gbdpcg {

// CTA size bound of the streamed kernel (its rows hold no registers).
constexpr int kStreamThreads = 512;

// Shared-memory plan: p and r windows, the product vector, two halos, the
// reduction slots and warp scratch, the item area.
template <typename T, typename A, int NP, bool PTRI>
struct SmemPlanStream {
    using Base = SmemPlan<T, A, NP, PTRI, ST_SMEM>;
    __host__ __device__ static size_t own(uint32_t kmax) { return round_up((size_t)kmax * NP * sizeof(T), 32); }
    __host__ __device__ static size_t bytes(uint32_t kmax, uint32_t C, uint32_t nwarps) {
        return 2 * Base::vec(kmax) + own(kmax) + 2 * Base::halo() + Base::slots(C) + Base::wscr(nwarps) + kItemBytes;
    }
};

// Block-row product of the RPT adjacent rows at M (the first row's element of
// column 0 of block 0 of its knot's block row, column-major with leading
// dimension n) over the present blocks [b0, b1), from global memory: one FMA
// chain per block in ascending column, summed in block order (smem_matvec's
// order).
template <typename T, int NP, int NB, int RPT>
__device__ __forceinline__ void gmem_matvec(const T *__restrict__ M, int b0, int b1, const T *x, uint32_t n,
                                            T (&y)[RPT]) {
    T acc[RPT][NB];
#pragma unroll
    for (int b = 0; b < NB; ++b) {
#pragma unroll
        for (int q = 0; q < RPT; ++q) acc[q][b] = T(0);
        if (b >= b0 && b < b1) {
            const T *col = M + (size_t)b * n * n;
#pragma unroll
            for (int j = 0; j < NP; ++j) {
                if ((uint32_t)j < n) {
                    const T xj = x[b * NP + j];
#pragma unroll
                    for (int q = 0; q < RPT; ++q) acc[q][b] = fma_rn(__ldg(col + (size_t)j * n + q), xj, acc[q][b]);
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
        T s = acc[q][0];
#pragma unroll
        for (int b = 1; b < NB; ++b) s += acc[q][b];
        y[q] = s;
    }
}

template <typename T, typename A, int NP, bool PTRI, int RPT>
__global__ void __launch_bounds__(kStreamThreads, 1) pcg_stream_kernel(const LaunchParams lp) {
    using Plan = SmemPlanStream<T, A, NP, PTRI>;
    using Base = typename Plan::Base;
    constexpr int NBP = PTRI ? 3 : 1;
    const cg::cluster_group cluster = cg::this_cluster();
    const uint32_t C = cluster.num_blocks();
    const uint32_t rank = cluster.block_rank();
    const uint32_t tid = threadIdx.x, nthr = blockDim.x;

    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *sp = smem_raw;
    T *vp = reinterpret_cast<T *>(sp); sp += Base::vec(lp.kmax);   // p window (lambda0 at the start)
    T *vr = reinterpret_cast<T *>(sp); sp += Base::vec(lp.kmax);   // r window
    T *vy = reinterpret_cast<T *>(sp); sp += Plan::own(lp.kmax);   // own rows: S p, then Phi^-1 r
    T *uh = reinterpret_cast<T *>(sp); sp += Base::halo();
    T *zh = reinterpret_cast<T *>(sp); sp += Base::halo();
    A *slots = reinterpret_cast<A *>(sp); sp += Base::slots(C);
    A *wscr = reinterpret_cast<A *>(sp); sp += Base::wscr(nthr >> 5);
    uint32_t *s_item = reinterpret_cast<uint32_t *>(sp);
    const uint32_t zero_elems =
        (uint32_t)((2 * Base::vec(lp.kmax) + Plan::own(lp.kmax) + 2 * Base::halo()) / sizeof(T));

    for (uint32_t e = tid; e < (uint32_t)(Base::slots(C) / sizeof(A)); e += nthr) slots[e] = A(0);
    for (uint32_t e = tid; e < (uint32_t)(kMaxValues * 32); e += nthr) wscr[e] = A(0);  // local slots
    TxReduce tx{reinterpret_cast<uint64_t *>(s_item + 8), 0u, s_item + 12};
    if (C > 1) {
        if (tid == 0) {
            mbar_init(tx.bar, 1);
            mbar_init(tx.bar + 1, 1);
            *tx.timed_out = 0u;
            mbar_init_fence();
        }
        cluster.sync();
    } else {
        __syncthreads();
    }
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
        // (a forward + adjoint pair runs on the on-chip storages only)
        if (n == 0 || N == 0 || n > (uint32_t)NP || K > lp.kmax || (RPT > 1 && (n % RPT) != 0) ||
            (d.flags & SYS_FWD_ADJ)) {
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
        const uint32_t nslots = nk * n / RPT, G = (nslots + nthr - 1) / nthr;
        const bool relres = (d.flags & SYS_EXIT_RELRES) != 0;
        const T *__restrict__ S = static_cast<const T *>(d.S);
        const T *__restrict__ P = static_cast<const T *>(d.P);
        const T *__restrict__ gamma = static_cast<const T *>(d.gamma);
        const T *lam0 = (d.flags & SYS_LAMBDA0_ZERO) ? nullptr : static_cast<const T *>(d.lambda0);
        T *lam = static_cast<T *>(d.lambda);
        const uint32_t blkS = 3 * n * n, blkP = NBP * n * n;
        const bool has_left = nk > 0 && kb > 0, has_right = nk > 0 && ke < N;
        const uint32_t halo_in = ((has_left ? n : 0u) + (has_right ? n : 0u)) * (uint32_t)sizeof(T);
        if (tid == 0 && nk > 0) {  // the first product's rows into L2 at once
            prefetch_l2_range(S + (size_t)kb * blkS, (size_t)nk * blkS * sizeof(T));
            prefetch_l2_range(P + (size_t)kb * blkP, (size_t)nk * blkP * sizeof(T));
        }
        for (uint32_t e = tid; e < zero_elems; e += nthr) vp[e] = T(0);

        // the RPT rows i.. of local knot lk that this thread owns in group g
        struct Slot {
            uint32_t lk, i, k;
            bool act, first, last;
            int sb0, sb1;
        };
        auto slot = [&](uint32_t g) {
            Slot s;
            const uint32_t row0 = (g * nthr + tid) * RPT;
            s.lk = row0 / n;
            s.i = row0 - s.lk * n;
            s.act = s.lk < nk;
            s.k = kb + s.lk;
            s.first = s.act && s.lk == 0 && kb > 0;
            s.last = s.act && s.lk + 1 == nk && ke < N;
            s.sb0 = (s.k == 0) ? 1 : 0;
            s.sb1 = (s.k + 1 == N) ? 2 : 3;
            return s;
        };
        auto matS = [&](const Slot &s, const T *x, T(&y)[RPT]) {
            gmem_matvec<T, NP, 3, RPT>(S + (size_t)s.k * blkS + s.i, s.sb0, s.sb1, x + s.lk * NP, n, y);
        };
        auto matP = [&](const Slot &s, const T *x, T(&y)[RPT]) {
            if constexpr (PTRI) gmem_matvec<T, NP, 3, RPT>(P + (size_t)s.k * blkP + s.i, s.sb0, s.sb1, x + s.lk * NP, n, y);
            else gmem_matvec<T, NP, 1, RPT>(P + (size_t)s.k * blkP + s.i, 0, 1, x + s.lk * NP + NP, n, y);
        };
        __syncthreads();

        // ---- lambda0 into the p window and into the solution array
        for (uint32_t g = 0; g < G; ++g) {
            const Slot s = slot(g);
            if (!s.act) continue;
#pragma unroll
            for (int q = 0; q < RPT; ++q) {
                const size_t row = (size_t)s.k * n + s.i + q;
                const T l = lam0 ? lam0[row] : T(0);
                vp[(s.lk + 1) * NP + s.i + q] = l;
                if (lam0 != lam) lam[row] = l;
            }
        }
        if (lam0) {
            for (uint32_t t = tid; t < 2 * n; t += nthr) {
                if (t < n && has_left) vp[t] = lam0[(size_t)(kb - 1) * n + t];
                if (t >= n && has_right) vp[(nk + 1) * NP + (t - n)] = lam0[(size_t)ke * n + (t - n)];
            }
        }
        __syncthreads();
        stamp.staged();

        // ---- r = gamma - S lambda0   (include/pcg.cuh:119-126), parked in vy
        A gg_acc = A(0);
        for (uint32_t g = 0; g < G; ++g) {
            const Slot s = slot(g);
            if (!s.act) continue;
            T y[RPT];
            matS(s, vp, y);
#pragma unroll
            for (int q = 0; q < RPT; ++q) {
                const T gm = gamma[(size_t)s.k * n + s.i + q];
                vy[s.lk * NP + s.i + q] = gm - y[q];
                acc_madd(gg_acc, gm, gm);
            }
        }
        group_sync(cluster, C);  // all windows read before any neighbour writes into them
        for (uint32_t g = 0; g < G; ++g) {
            const Slot s = slot(g);
            if (!s.act) continue;
            T r[RPT];
#pragma unroll
            for (int q = 0; q < RPT; ++q) {
                r[q] = vy[s.lk * NP + s.i + q];
                vr[(s.lk + 1) * NP + s.i + q] = r[q];
            }
            if constexpr (PTRI) {
                if (s.first) {
                    T *dst = cluster.map_shared_rank(vr, rank - 1) + (K + 1) * NP + s.i;
#pragma unroll
                    for (int q = 0; q < RPT; ++q) dst[q] = r[q];
                }
                if (s.last) {
                    T *dst = cluster.map_shared_rank(vr, rank + 1) + s.i;
#pragma unroll
                    for (int q = 0; q < RPT; ++q) dst[q] = r[q];
                }
            }
        }
        if constexpr (PTRI) group_sync(cluster, C);
        else __syncthreads();

        // ---- z = Phi^-1 r; p = z; eta = r.z   (include/pcg.cuh:131-149)
        A eta, gg;
        {
            A v2[2] = {A(0), gg_acc};
            for (uint32_t g = 0; g < G; ++g) {
                const Slot s = slot(g);
                if (!s.act) continue;
                T z[RPT];
                matP(s, vr, z);
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    vp[(s.lk + 1) * NP + s.i + q] = z[q];
                    acc_madd(v2[0], vr[(s.lk + 1) * NP + s.i + q], z[q]);
                }
                if (s.first) push_halo_tx<T, RPT>(vp + (K + 1) * NP + s.i, rank - 1, z, tx, 1);
                if (s.last) push_halo_tx<T, RPT>(vp + s.i, rank + 1, z, tx, 1);
            }
            solver_allreduce<A, 2>(v2, slots, wscr, 1, tx, cluster, C, rank, halo_in);
            eta = v2[0];
            gg = v2[1];
        }
        const A thr = A(d.tol * d.tol * (double)gg);
        const A tol = A(d.tol);

        // ---- main loop   (include/pcg.cuh:154-208)
        uint32_t iter = 0;
        int32_t status = ST_MAX_ITER;
        A eta_new = A(0), rr = A(0);
        const uint32_t max_iter = d.max_iter;
        for (; iter < max_iter;) {
            A pap;
            {
                A v1[1] = {A(0)};
                for (uint32_t g = 0; g < G; ++g) {
                    const Slot s = slot(g);
                    if (!s.act) continue;
                    T y[RPT];
                    matS(s, vp, y);
#pragma unroll
                    for (int q = 0; q < RPT; ++q) {
                        vy[s.lk * NP + s.i + q] = y[q];
                        acc_madd(v1[0], vp[(s.lk + 1) * NP + s.i + q], y[q]);
                    }
                    if constexpr (PTRI) {  // neighbours need the boundary upsilon for their r halo
                        if (s.first) push_halo_tx<T, RPT>(uh + NP + s.i, rank - 1, y, tx, 0);
                        if (s.last) push_halo_tx<T, RPT>(uh + s.i, rank + 1, y, tx, 0);
                    }
                }
                solver_allreduce<A, 1>(v1, slots, wscr, 0, tx, cluster, C, rank, PTRI ? halo_in : 0u);
                pap = v1[0];
            }
            const T alpha = (pap == A(0)) ? T(0) : acc_ratio<T>(eta, pap);
            for (uint32_t g = 0; g < G; ++g) {
                const Slot s = slot(g);
                if (!s.act) continue;
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    const size_t row = (size_t)s.k * n + s.i + q;
                    const uint32_t w = (s.lk + 1) * NP + s.i + q;
                    lam[row] = fma_rn(alpha, vp[w], lam[row]);
                    vr[w] = fma_rn(-alpha, vy[s.lk * NP + s.i + q], vr[w]);
                }
            }
            if constexpr (PTRI) {
                for (uint32_t t = tid; t < 2 * n; t += nthr) {
                    if (t < n && has_left) vr[t] = fma_rn(-alpha, uh[t], vr[t]);
                    if (t >= n && has_right) {
                        T *h = vr + (nk + 1) * NP + (t - n);
                        *h = fma_rn(-alpha, uh[NP + t - n], *h);
                    }
                }
            }
            __syncthreads();
            {
                A v2[2] = {A(0), A(0)};
                for (uint32_t g = 0; g < G; ++g) {
                    const Slot s = slot(g);
                    if (!s.act) continue;
                    T z[RPT];
                    matP(s, vr, z);
#pragma unroll
                    for (int q = 0; q < RPT; ++q) {
                        const T r = vr[(s.lk + 1) * NP + s.i + q];
                        vy[s.lk * NP + s.i + q] = z[q];
                        acc_madd(v2[0], r, z[q]);
                        if (relres) acc_madd(v2[1], r, r);
                    }
                    if (s.first) push_halo_tx<T, RPT>(zh + NP + s.i, rank - 1, z, tx, 1);
                    if (s.last) push_halo_tx<T, RPT>(zh + s.i, rank + 1, z, tx, 1);
                }
                solver_allreduce<A, 2>(v2, slots, wscr, 1, tx, cluster, C, rank, halo_in);
                eta_new = v2[0];
                rr = v2[1];
            }
            ++iter;
            if (!acc_finite(eta_new) || !acc_finite(pap)) { status = ST_BREAKDOWN; break; }
            if (relres ? (rr <= thr) : (acc_abs(eta_new) < tol)) { status = ST_CONVERGED; break; }
            const T beta = acc_ratio<T>(eta_new, eta);
            eta = eta_new;
            for (uint32_t g = 0; g < G; ++g) {
                const Slot s = slot(g);
                if (!s.act) continue;
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    const uint32_t w = (s.lk + 1) * NP + s.i + q;
                    vp[w] = fma_rn(beta, vp[w], vy[s.lk * NP + s.i + q]);
                }
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

        // ---- outputs: lambda is already in place   (include/pcg.cuh:212-217)
        stamp.solved();
        if (rank == 0 && tid == 0) {
            if (C > 1)
                for (uint32_t c = 0; c < C; ++c)
                    if (*cluster.map_shared_rank(tx.timed_out, c)) status = ST_TIMEOUT;
            SysResult res;
            res.iters = iter;
            res.status = status;
            res.eta = (double)eta_new;
            res.rr = relres ? (double)rr : -1.0;
            res.gg = (double)gg;
            res.outer = 0;
            res.pad = 0;
            lp.results[d.result] = res;
        }

        // ---- adjoint epilogue: dS = -1/2 (mu lam^T + lam mu^T) on the block pattern
        if (d.flags & SYS_ADJOINT) {
            const T *lf = static_cast<const T *>(d.lam_fwd);
            T *dS = static_cast<T *>(d.dS);
            group_sync(cluster, C);  // vp / vr free in every CTA, mu complete in lam
            for (uint32_t g = 0; g < G; ++g) {
                const Slot s = slot(g);
                if (!s.act) continue;
                T mu[RPT];
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    const size_t row = (size_t)s.k * n + s.i + q;
                    mu[q] = lam[row];
                    vr[(s.lk + 1) * NP + s.i + q] = mu[q];
                    vp[(s.lk + 1) * NP + s.i + q] = lf[row];
                }
                if (s.first) {
                    T *dst = cluster.map_shared_rank(vr, rank - 1) + (K + 1) * NP + s.i;
#pragma unroll
                    for (int q = 0; q < RPT; ++q) dst[q] = mu[q];
                }
                if (s.last) {
                    T *dst = cluster.map_shared_rank(vr, rank + 1) + s.i;
#pragma unroll
                    for (int q = 0; q < RPT; ++q) dst[q] = mu[q];
                }
            }
            for (uint32_t t = tid; t < 2 * n; t += nthr) {
                if (t < n && has_left) vp[t] = lf[(size_t)(kb - 1) * n + t];
                if (t >= n && has_right) vp[(nk + 1) * NP + (t - n)] = lf[(size_t)ke * n + (t - n)];
            }
            group_sync(cluster, C);
            for (uint32_t g = 0; g < G; ++g) {
                const Slot s = slot(g);
                if (!s.act) continue;
                for (uint32_t b = 0; b < 3; ++b) {
                    const bool present = (b != 0 || s.k > 0) && (b != 2 || s.k + 1 < N);
                    const T *lw = vp + (s.lk + b) * NP;
                    const T *mw = vr + (s.lk + b) * NP;
                    for (uint32_t j = 0; j < n; ++j) {
#pragma unroll
                        for (int q = 0; q < RPT; ++q) {
                            const T mq = vr[(s.lk + 1) * NP + s.i + q], lq = vp[(s.lk + 1) * NP + s.i + q];
                            const T gv = present ? T(-0.5) * fma_rn(mq, lw[j], lq * mw[j]) : T(0);
                            dS[(size_t)s.k * blkS + (b * n + j) * n + s.i + q] = gv;
                        }
                    }
                }
            }
        }
        stamp.done(lp, item, iter);
    }
    if (C > 1) cluster.sync();  // every transaction-counted store into this CTA has landed
}

}  // namespace gbdpcg
