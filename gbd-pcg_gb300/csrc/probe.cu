// Latency of the synchronisation primitives one PCG iteration of the cluster
// solver is built from (gbdpcg_probe_primitives): the CTA barrier, the
// cluster barrier, a distributed-shared-memory store followed by the cluster
// barrier, and the cluster-wide reductions of 1, 2 and 3 values the solver
// runs (pcg_cluster.cuh: cluster_allreduce, and cluster_allreduce_tx, the form
// the cluster kernels use for C >= 2), on the same shared-memory slot layout.
// Each probe kernel repeats one primitive `reps` times in a loop whose values
// depend on the previous repetition (nothing can be hoisted or overlapped),
// timed with CUDA events around the launch; the loop alone is measured the
// same way and subtracted.  Every loop is bounded; no probe waits on a flag.
// The iteration floor of the solver's forms is built from these numbers:
// standard form 2 reductions + 2 CTA barriers, recurrence form 2 reductions +
// 1 CTA barrier (the reference has 4 grid-wide barriers per iteration,
// include/pcg.cuh:166,178,190,207).
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/gbdpcg.h"
#include "pcg_cluster.cuh"

namespace gbdpcg {
void set_last_error(const std::string &msg);
}

namespace {

using namespace gbdpcg;

enum { PROBE_LOOP = 0, PROBE_SYNCTHREADS = 1, PROBE_CLUSTER = 2, PROBE_DSMEM = 3, PROBE_REDUCE = 4, PROBE_REDUCE_TX = 5 };

template <int KIND, int NQ>
__global__ void probe_kernel(uint32_t reps, float *sink) {
    const cg::cluster_group cluster = cg::this_cluster();
    const uint32_t C = cluster.num_blocks(), rank = cluster.block_rank();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t nwarps = blockDim.x >> 5;
    float *slots = reinterpret_cast<float *>(smem_raw);
    float *wscr = slots + 2 * kMaxValues * slot_stride(C);
    float *cell = wscr + nwarps * kMaxValues * 32;
    uint64_t *bar = reinterpret_cast<uint64_t *>(cell + 8);
    uint32_t *timed_out = reinterpret_cast<uint32_t *>(bar + 2);
    for (uint32_t e = threadIdx.x; e < 2 * kMaxValues * slot_stride(C); e += blockDim.x) slots[e] = 0.f;
    for (uint32_t e = threadIdx.x; e < kMaxValues * 32; e += blockDim.x) wscr[e] = 0.f;  // local slots
    if (threadIdx.x == 0) {
        cell[0] = 0.f;
        *timed_out = 0u;
        mbar_init(bar, 1);
        mbar_init(bar + 1, 1);
        mbar_init_fence();
    }
    if (C > 1)
        cluster.sync();
    else
        __syncthreads();
    TxReduce tx{bar, 0u, timed_out};
    float v = (float)(threadIdx.x & 7) * 1e-3f;
    for (uint32_t it = 0; it < reps; ++it) {
        if constexpr (KIND == PROBE_LOOP) {
            v = fmaf(v, 0.999f, 1e-3f);
        } else if constexpr (KIND == PROBE_SYNCTHREADS) {
            v = fmaf(v, 0.999f, 1e-3f);
            __syncthreads();
        } else if constexpr (KIND == PROBE_CLUSTER) {
            v = fmaf(v, 0.999f, 1e-3f);
            cluster.sync();
        } else if constexpr (KIND == PROBE_DSMEM) {
            // one boundary push to the next rank's shared memory, then the barrier
            // that makes it visible, as a halo push before a reduction
            if (threadIdx.x == 0) *cluster.map_shared_rank(cell, (rank + 1) % C) = v;
            cluster.sync();
            v = fmaf(cell[0], 0.5f, v);
        } else if constexpr (KIND == PROBE_REDUCE) {
            float q[NQ];
#pragma unroll
            for (int j = 0; j < NQ; ++j) q[j] = v + (float)j;
            cluster_allreduce<float, NQ>(q, slots, wscr, (int)(it & 1), cluster, C, rank);
            v = fmaf(q[0], 1e-9f, v * 0.5f);
        } else {
            float q[NQ];
#pragma unroll
            for (int j = 0; j < NQ; ++j) q[j] = v + (float)j;
            cluster_allreduce_tx<float, NQ>(q, slots, wscr, (int)(it & 1), tx, C, rank);
            v = fmaf(q[0], 1e-9f, v * 0.5f);
        }
    }
    if (*timed_out)
        sink[0] = 1.f;  // a reduction wait gave up
    else if (v == 12345.678f)
        sink[0] = v;  // keeps the chain alive
    if (C > 1) cluster.sync();  // no CTA leaves while a peer may still store into it
}

// A wait that nothing completes, through the solver's own bounded waits: for
// a cluster of C >= 2 CTAs, one transaction-counted reduction whose receivers
// also expect 16 bytes of halo that no neighbour sends (every real partial
// arrives); for C = 1, a wait on an mbarrier that expects 16 bytes nothing
// sends.  Each CTA gives up after about a second (mbar_wait_bounded) and
// writes its outcome to status[cta]: GBDPCG_TIMEOUT when the wait gave up.
// Nothing waits without a limit, and no CTA leaves before the cluster's last
// barrier, so no store is in flight into a CTA that has ended.
__global__ void probe_timeout_kernel(int *status) {
    const cg::cluster_group cluster = cg::this_cluster();
    const uint32_t C = cluster.num_blocks(), rank = cluster.block_rank();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t nwarps = blockDim.x >> 5;
    float *slots = reinterpret_cast<float *>(smem_raw);
    float *wscr = slots + 2 * kMaxValues * slot_stride(C);
    float *cell = wscr + nwarps * kMaxValues * 32;
    uint64_t *bar = reinterpret_cast<uint64_t *>(cell + 8);
    uint32_t *timed_out = reinterpret_cast<uint32_t *>(bar + 2);
    for (uint32_t e = threadIdx.x; e < kMaxValues * 32; e += blockDim.x) wscr[e] = 0.f;  // local slots
    if (threadIdx.x == 0) {
        *timed_out = 0u;
        mbar_init(bar, 1);
        mbar_init(bar + 1, 1);
        mbar_init_fence();
    }
    if (C > 1)
        cluster.sync();
    else
        __syncthreads();
    TxReduce tx{bar, 0u, timed_out};
    if (C > 1) {
        float q[1] = {(float)rank};
        cluster_allreduce_tx<float, 1>(q, slots, wscr, 0, tx, C, rank, 16u);
    } else {
        if (threadIdx.x == 0) mbar_arrive_expect_tx(bar, 16u);
        mbar_wait_bounded(bar, 0u, timed_out);
    }
    __syncthreads();
    if (threadIdx.x == 0) status[blockIdx.x] = *timed_out ? GBDPCG_TIMEOUT : GBDPCG_SUCCESS;
    if (C > 1) cluster.sync();
}

size_t probe_smem(uint32_t C, uint32_t threads) {
    // slots, warp scratch, then 32 words: a cell, two mbarriers, the timeout flag
    return (2 * kMaxValues * slot_stride(C) + (threads / 32) * kMaxValues * 32 + 32) * sizeof(float);
}

int probe_fail(int code, const std::string &msg) {
    set_last_error(msg);
    return code;
}

// ns per repetition of one probe kernel (grid of `clusters` clusters of C CTAs)
int time_probe(const void *func, uint32_t C, uint32_t threads, uint32_t clusters, uint32_t reps, float *sink,
               double *ns) {
    const size_t smem = probe_smem(C, threads);
    cudaError_t e = cudaSuccess;
    if (C > 8) e = cudaFuncSetAttribute(func, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return probe_fail(GBDPCG_ERR_CUDA, std::string("probe set-up: ") + cudaGetErrorString(e));
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (clusters == 0) {
        int active = 0;
        cfg.gridDim = dim3(C);
        e = cudaOccupancyMaxActiveClusters(&active, func, &cfg);
        if (e != cudaSuccess || active <= 0)
            return probe_fail(GBDPCG_ERR_UNSUPPORTED, "probe: cluster shape cannot be scheduled");
        clusters = (uint32_t)active;
    }
    cfg.gridDim = dim3(clusters * C);
    uint32_t r = reps;
    void *args[] = {&r, &sink};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.f;
    e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaLaunchKernelExC(&cfg, func, args);  // warm
    if (e == cudaSuccess) e = cudaEventRecord(e0, 0);
    if (e == cudaSuccess) e = cudaLaunchKernelExC(&cfg, func, args);
    if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess) return probe_fail(GBDPCG_ERR_CUDA, std::string("probe: ") + cudaGetErrorString(e));
    *ns = (double)ms * 1e6 / (double)reps;
    return GBDPCG_SUCCESS;
}

}  // namespace

extern "C" {

int gbdpcg_probe_primitives(int device, uint32_t cluster, uint32_t threads, uint32_t clusters, uint32_t reps,
                            gbdpcg_probe *out) {
    if (!out) return probe_fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (cluster < 1 || cluster > 16 || threads < 32 || threads > 1024 || threads % 32 || reps == 0)
        return probe_fail(GBDPCG_ERR_INVALID_ARGUMENT, "cluster 1..16, threads a multiple of 32 up to 1024, reps > 0");
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != device && cudaSetDevice(device) != cudaSuccess)
        return probe_fail(GBDPCG_ERR_INVALID_ARGUMENT, "bad device");
    float *sink = nullptr;
    int rc = GBDPCG_SUCCESS;
    if (cudaMalloc(&sink, sizeof(float)) != cudaSuccess || cudaMemset(sink, 0, sizeof(float)) != cudaSuccess)
        rc = probe_fail(GBDPCG_ERR_NO_MEMORY, "probe sink");
    double loop = 0, t[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const void *fns[10] = {(const void *)&probe_kernel<PROBE_LOOP, 1>, (const void *)&probe_kernel<PROBE_SYNCTHREADS, 1>,
                           (const void *)&probe_kernel<PROBE_CLUSTER, 1>, (const void *)&probe_kernel<PROBE_DSMEM, 1>,
                           (const void *)&probe_kernel<PROBE_REDUCE, 1>, (const void *)&probe_kernel<PROBE_REDUCE, 2>,
                           (const void *)&probe_kernel<PROBE_REDUCE, 3>, (const void *)&probe_kernel<PROBE_REDUCE_TX, 1>,
                           (const void *)&probe_kernel<PROBE_REDUCE_TX, 2>, (const void *)&probe_kernel<PROBE_REDUCE_TX, 3>};
    for (int k = 0; k < 10 && rc == GBDPCG_SUCCESS; ++k) {
        // no cluster barrier in a one-CTA cluster; the transaction-counted reduction is for C >= 2
        if ((k == 2 || k == 3 || k >= 7) && cluster == 1) continue;
        rc = time_probe(fns[k], cluster, threads, clusters, reps, sink, k == 0 ? &loop : &t[k]);
    }
    float flag = 0.f;
    if (rc == GBDPCG_SUCCESS && cudaMemcpy(&flag, sink, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
        rc = probe_fail(GBDPCG_ERR_CUDA, "probe read-back");
    if (rc == GBDPCG_SUCCESS && flag == 1.f) rc = probe_fail(GBDPCG_ERR_CUDA, "probe: a reduction wait timed out");
    if (sink) cudaFree(sink);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    if (rc) return rc;
    memset(out, 0, sizeof(*out));
    auto net = [&](double x) { return x > loop ? x - loop : 0.0; };
    out->loop_ns = loop;
    out->syncthreads_ns = net(t[1]);
    out->cluster_barrier_ns = cluster > 1 ? net(t[2]) : 0.0;
    out->dsmem_store_barrier_ns = cluster > 1 ? net(t[3]) : 0.0;
    for (int q = 0; q < 3; ++q) out->allreduce_ns[q] = net(t[4 + q]);
    for (int q = 0; q < 3; ++q) out->allreduce_tx_ns[q] = cluster > 1 ? net(t[7 + q]) : 0.0;
    return GBDPCG_SUCCESS;
}

int gbdpcg_probe_timeout(int device, uint32_t cluster, int *status, double *waited_ms) {
    if (!status || !waited_ms) return probe_fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (cluster < 1 || cluster > 16) return probe_fail(GBDPCG_ERR_INVALID_ARGUMENT, "cluster 1..16");
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != device && cudaSetDevice(device) != cudaSuccess)
        return probe_fail(GBDPCG_ERR_INVALID_ARGUMENT, "bad device");
    const uint32_t threads = 128;
    const void *func = (const void *)&probe_timeout_kernel;
    int *d_status = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc(&d_status, cluster * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(d_status, 0xff, cluster * sizeof(int));
    if (e == cudaSuccess && cluster > 8) e = cudaFuncSetAttribute(func, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = probe_smem(cluster, threads);
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void *args[] = {&d_status};
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaEventRecord(e0, 0);
    if (e == cudaSuccess) e = cudaLaunchKernelExC(&cfg, func, args);
    if (e == cudaSuccess) e = cudaEventRecord(e1, 0);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    std::vector<int> st(cluster, -2);
    if (e == cudaSuccess) e = cudaMemcpy(st.data(), d_status, cluster * sizeof(int), cudaMemcpyDeviceToHost);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (d_status) cudaFree(d_status);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    if (e != cudaSuccess) return probe_fail(GBDPCG_ERR_CUDA, std::string("timeout probe: ") + cudaGetErrorString(e));
    int worst = GBDPCG_TIMEOUT;
    for (int x : st)
        if (x != GBDPCG_TIMEOUT) worst = x;  // a CTA whose wait did not give up
    *status = worst;
    *waited_ms = (double)ms;
    return GBDPCG_SUCCESS;
}

}  // extern "C"
