// Host runtime and C ABI (include/gbdpcg.h) of the GB300 PCG solver.
//
//   * variant registry: the cluster-kernel instantiations, their register
//     budget (max threads per CTA) and shared-memory plans;
//   * planner: assigns each system a kernel variant (block-size bound NP,
//     Phi^-1 storage, precision), a cluster size C and a CTA size, groups
//     systems with the same launch shape into classes, sorts each class
//     longest first into a device work list;
//   * executor: one persistent cluster launch per class (fed by a device work
//     queue), the classes spread over a few streams, all captured in one CUDA
//     graph that also resets the queues;
//   * the single-system entry points (host and device pointers), which pass
//     the system descriptor by value and need no queue;
//   * the plain algorithm (one CTA per knot, cooperative launch) for n > 32.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/gbdpcg.h"
#include "pcg_types.h"
#include "pcg_variants.h"

namespace gbdpcg {
cudaError_t launch_block_jacobi(int kind, const SysDesc *d_descs, const uint64_t *d_prefix,
                                uint32_t nsys, uint64_t total_knots, int tri_layout,
                                cudaStream_t stream, const SysDesc *one = nullptr);
}

using namespace gbdpcg;

namespace {

thread_local std::string t_last_error;

size_t round_up(size_t x, size_t m) { return (x + m - 1) / m * m; }

int fail(int code, const std::string &msg) {
    t_last_error = msg;
    return code;
}

#define GB_CUDA(call)                                                                         \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(GBDPCG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// ------------------------------------------------------------------ variant registry
struct VariantInfo {
    KernelVariant v;
    int max_threads = 0;  // from the register budget (cudaFuncAttributes)
    int regs = 0;
    size_t smem_set = 0;  // max dynamic smem attribute already set
    bool nonportable = false;
};

struct Registry {
    std::vector<VariantInfo> list;
    int max_smem_optin = 0;
    int sm_count = 0;
    // the GPU reads pageable host memory through the host's page tables
    // (Grace: address translation services), so kernels may use host arrays
    // in place
    bool host_direct = false;
};

std::mutex g_reg_mu;
std::map<int, std::unique_ptr<Registry>> g_registries;  // per device

const int kNPs[] = {6, 8, 12, 14, 16, 24, 32};

int np_for(uint32_t n) {
    for (int np : kNPs)
        if ((int)n <= np) return np;
    return 0;
}

int get_registry(int device, Registry **out) {
    std::lock_guard<std::mutex> lk(g_reg_mu);
    auto it = g_registries.find(device);
    if (it != g_registries.end()) {
        *out = it->second.get();
        return GBDPCG_SUCCESS;
    }
    auto reg = std::make_unique<Registry>();
    KernelVariant buf[kMaxVariantsPerNP];
    int (*fns[])(KernelVariant *) = {variants_np6,      variants_np8,      variants_np12,
                                     variants_np14,     variants_np16,     variants_np24,
                                     variants_np32,     variants_np6_ext,  variants_np8_ext,
                                     variants_np12_ext, variants_np14_ext, variants_np16_ext,
                                     variants_np24_ext, variants_np32_ext,
                                     variants_stream_small, variants_stream_large,
                                     variants_fa_np6,   variants_fa_np8,   variants_fa_np12,
                                     variants_fa_np14,  variants_fa_np16,  variants_fa_np24,
                                     variants_fa_np32};
    for (auto fn : fns) {
        const int c = fn(buf);
        for (int i = 0; i < c; ++i) {
            VariantInfo vi;
            vi.v = buf[i];
            cudaFuncAttributes attr;
            GB_CUDA(cudaFuncGetAttributes(&attr, vi.v.func));
            vi.max_threads = attr.maxThreadsPerBlock / 32 * 32;
            vi.regs = attr.numRegs;
            reg->list.push_back(vi);
        }
    }
    GB_CUDA(cudaDeviceGetAttribute(&reg->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                   device));
    GB_CUDA(cudaDeviceGetAttribute(&reg->sm_count, cudaDevAttrMultiProcessorCount, device));
    int pageable = 0, host_tables = 0;
    GB_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device));
    GB_CUDA(cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device));
    reg->host_direct = pageable != 0 && host_tables != 0;
    *out = reg.get();
    g_registries[device] = std::move(reg);
    return GBDPCG_SUCCESS;
}

// acc: dot accumulation of FP32 systems (0 float, 1 double, 2 float-float);
// FP64 systems always accumulate in double.
// fa: a variant that runs forward + adjoint pairs (for such plans only).
VariantInfo *find_variant(Registry *reg, bool f64, int acc, int np, bool ptri, int st, int rpt,
                          int alg, bool fa = false) {
    for (auto &vi : reg->list)
        if (vi.v.f64 == (int)f64 && vi.v.acc == (f64 ? 1 : acc) && vi.v.np == np &&
            vi.v.ptri == (int)ptri && vi.v.st == st && vi.v.rpt == rpt && vi.v.alg == alg &&
            vi.v.fa == (int)fa)
            return &vi;
    return nullptr;
}

int prepare_variant(VariantInfo *vi, size_t smem, uint32_t C) {
    if (smem > 48 * 1024 && smem > vi->smem_set) {
        GB_CUDA(cudaFuncSetAttribute(vi->v.func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
        vi->smem_set = smem;
    }
    if (C > 8 && !vi->nonportable) {
        GB_CUDA(cudaFuncSetAttribute(vi->v.func, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        vi->nonportable = true;
    }
    return GBDPCG_SUCCESS;
}

// ------------------------------------------------------------------ device buffers
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    int ensure(size_t want) {
        if (want <= bytes) return GBDPCG_SUCCESS;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (cudaMalloc(&p, want) != cudaSuccess)
            return fail(GBDPCG_ERR_NO_MEMORY, "cudaMalloc of " + std::to_string(want) + " bytes");
        bytes = want;
        return GBDPCG_SUCCESS;
    }
    template <typename T>
    T *as(size_t byte_off = 0) const {
        return reinterpret_cast<T *>(static_cast<char *>(p) + byte_off);
    }
};

// ------------------------------------------------------------------ tuning table
// Key: what selects the kernel family (precision, refinement, dot precision,
// Phi^-1 layout, adjoint epilogue, the requested algorithm and storage) and
// the system size.  Value: the launch shape the autotuner measured fastest.
struct TuneKey {
    uint8_t f64, refine, acc, ptri, adjoint, alg_req, storage_req;
    uint32_t n, N;
    bool operator<(const TuneKey &o) const {
        return std::tie(f64, refine, acc, ptri, adjoint, alg_req, storage_req, n, N) <
               std::tie(o.f64, o.refine, o.acc, o.ptri, o.adjoint, o.alg_req, o.storage_req, o.n, o.N);
    }
};

struct TuneChoice {
    int st, rpt, alg;
    uint32_t C, threads;
};

// ------------------------------------------------------------------ launch shapes
struct Shape {
    VariantInfo *vi = nullptr;
    uint32_t C = 0, threads = 0, K = 0;
    bool plain = false;
};

// Storage / rows-per-thread candidates in order of preference: the first that
// holds the system wins.  Rows held in registers are the fastest; S in
// registers with Phi^-1 in shared memory holds 2 rows per thread (about 1.5x
// the rows per SM); rows in shared memory hold the most but read every matrix
// element from shared memory each iteration.
struct Pref {
    int st, rpt;
};

// A launch shape of the streamed storage may give a thread several row groups,
// so its CTA needs no thread per row (any CTA size holds the system).
bool streamed(int st) { return st == 5; }  // pcg_cluster.cuh ST_STREAM

std::vector<Pref> storage_prefs(bool f64, bool ptri, uint32_t storage) {
    if (storage == GBDPCG_STORAGE_STREAM) return f64 || ptri ? std::vector<Pref>{{5, 1}} : std::vector<Pref>{{5, 2}, {5, 1}};
    if (storage == GBDPCG_STORAGE_REGISTERS) return {{0, 1}, {0, 2}};
    if (storage == GBDPCG_STORAGE_SHARED) return {{2, 1}};
    if (storage == GBDPCG_STORAGE_SPLIT) return ptri ? std::vector<Pref>{} : std::vector<Pref>{{1, 2}, {1, 1}};
    if (storage == GBDPCG_STORAGE_HYBRID) return ptri ? std::vector<Pref>{} : std::vector<Pref>{{3, 2}, {3, 1}};
    if (storage == GBDPCG_STORAGE_TMEM) return ptri || f64 ? std::vector<Pref>{} : std::vector<Pref>{{4, 2}};
    // AUTO: rows on chip where they fit; streamed rows for larger systems
    if (f64) return ptri ? std::vector<Pref>{{0, 1}, {2, 1}, {5, 1}} : std::vector<Pref>{{0, 1}, {1, 1}, {2, 1}, {5, 1}};
    return ptri ? std::vector<Pref>{{0, 1}, {2, 1}, {5, 1}}
                : std::vector<Pref>{{1, 2}, {0, 1}, {1, 1}, {2, 1}, {3, 2}, {3, 1}, {5, 2}, {5, 1}};
}

// A tuned shape for one system, if its variant exists and holds the system.
bool tuned_shape(Registry *reg, bool f64, int acc, int np, bool ptri, uint32_t n, uint32_t N,
                 const TuneChoice &tc, Shape *out, bool fa = false) {
    if (tc.rpt < 1 || n % tc.rpt || tc.C < 1 || tc.C > 16 || tc.threads == 0 || tc.threads % 32) return false;
    VariantInfo *vi = find_variant(reg, f64, acc, np, ptri, tc.st, tc.rpt, tc.alg, fa);
    if (!vi) return false;
    const uint32_t K = (N + tc.C - 1) / tc.C;
    const uint32_t thr = (K * n + tc.rpt - 1) / tc.rpt;
    if ((!streamed(tc.st) && thr > tc.threads) || tc.threads > (uint32_t)vi->max_threads) return false;
    if (vi->v.smem_bytes(K, tc.C, tc.threads / 32) > (size_t)reg->max_smem_optin) return false;
    out->vi = vi;
    out->C = tc.C;
    out->K = K;
    out->threads = tc.threads;
    out->plain = false;
    return true;
}

// Dot accumulation of a launch: FP64 systems in double; refinement's inner
// solve in double unless float-float is asked for; FP32 systems as configured.
int acc_kind(bool f64_system, bool refine, uint32_t dot_precision) {
    if (f64_system) return 1;
    if (refine) return dot_precision == GBDPCG_DOT_FLOAT2 ? 2 : 1;
    return (int)dot_precision;
}

// Cluster size a lone system (latency, not throughput) starts its search at:
// C = 1 up to 40 knots (no cluster barriers), else about 16 knots a CTA (8 for
// FP64 rows), rounded up to a power of two.  Measured on n = 14: N = 32 is
// fastest at C = 1, N = 128 at C = 8 (FP32) and C = 16 (FP64).
uint32_t lone_cluster_pref(bool f64_rows, uint32_t N) {
    if (N <= 40) return 1;
    const uint32_t per = f64_rows ? 8 : 16;
    const uint32_t want = (N + per - 1) / per;
    uint32_t p = 1;
    while (p < want) p <<= 1;
    return std::min<uint32_t>(16, p);
}

// Whether the plain algorithm's N CTAs of 64 threads can all be resident at
// once (its cooperative launch needs that).
bool plain_fits(Registry *reg, bool f64, uint32_t n, uint32_t N) {
    const size_t smem = plain_smem_bytes(f64, n, N);
    if (smem > (size_t)reg->max_smem_optin) return false;
    const void *func = plain_kernel_ptr(f64);
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, 64, smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (int64_t)per_sm * reg->sm_count >= (int64_t)N;
}

// c_pref > 1 (lone systems, cluster size not pinned): clusters from c_pref up
// are tried first, then the smallest that fits.  `lone`: a single system
// solved by itself.  For such a system with a cbtd Phi^-1 that no on-chip
// shape holds, AUTO prefers the plain algorithm (all SMs, one CTA per knot)
// to streamed rows (one cluster of at most 16 SMs) whenever the plain
// kernel's CTAs fit at once; batches take streamed rows, which keep the whole
// batch in one persistent launch.
int choose_shape(Registry *reg, bool f64, uint32_t n, uint32_t N, uint32_t layout,
                 const gbdpcg_config &cfg, Shape *out, bool refine = false,
                 const TuneChoice *tuned = nullptr, uint32_t c_pref = 1, bool lone = false,
                 bool fa = false) {
    Shape s;
    const int np = np_for(n);
    if (refine) {
        if (np == 0 || layout != GBDPCG_PINV_BLOCKDIAG || cfg.algorithm == GBDPCG_ALGO_PLAIN)
            return fail(GBDPCG_ERR_UNSUPPORTED, "refinement needs n <= 32 and a compact Phi^-1");
    }
    const bool want_plain = !refine && (cfg.algorithm == GBDPCG_ALGO_PLAIN || np == 0);
    if (want_plain) {
        if (layout != GBDPCG_PINV_CBTD)
            return fail(GBDPCG_ERR_UNSUPPORTED, "plain algorithm needs a cbtd Phi^-1");
        s.plain = true;
        *out = s;
        return GBDPCG_SUCCESS;
    }
    const bool ptri = layout == GBDPCG_PINV_CBTD;
    const int acc = acc_kind(f64 && !refine, refine, cfg.dot_precision);
    const int alg = refine ? 2
                           : (cfg.algorithm == GBDPCG_ALGO_SINGLE_REDUCTION ? 1
                                                                             : (cfg.algorithm == GBDPCG_ALGO_RECURRENCE ? 3 : 0));
    if (alg == 1 && ptri)
        return fail(GBDPCG_ERR_UNSUPPORTED, "the single-reduction algorithm needs a block-diagonal Phi^-1");
    if (alg == 1 && acc == 2)
        return fail(GBDPCG_ERR_UNSUPPORTED, "the single-reduction algorithm has no float-float accumulation");
    if (tuned && tuned_shape(reg, f64 && !refine, acc, np, ptri, n, N, *tuned, out, fa)) return GBDPCG_SUCCESS;
    const uint32_t first_lo = (cfg.cluster_size == 0 && c_pref > 1) ? c_pref : 1;
    std::vector<Pref> prefs = storage_prefs(f64 && !refine, ptri, cfg.storage);
    // A lone FP32 system takes tensor-memory rows first where they fit: its
    // CTAs have their SMs to themselves anyway (the exclusive tensor-memory
    // allocation is what keeps that storage out of AUTO for batches), and its
    // iteration is the shortest there (n = 14, N = 32: 1.1-1.3 us against
    // 1.4-1.6 us with S in registers and Phi^-1 in shared memory).
    if (lone && cfg.storage == GBDPCG_STORAGE_AUTO && !f64 && !refine && !ptri)
        prefs.insert(prefs.begin(), Pref{4, 2});
    for (uint32_t from : {first_lo, 1u}) {
        for (const Pref &pf : prefs) {
            if (pf.rpt > 1 && (n % pf.rpt) != 0) continue;
            if (streamed(pf.st) && lone && ptri && cfg.storage == GBDPCG_STORAGE_AUTO &&
                cfg.algorithm == GBDPCG_ALGO_AUTO && cfg.cluster_size == 0 && plain_fits(reg, f64, n, N)) {
                s.plain = true;
                *out = s;
                return GBDPCG_SUCCESS;
            }
            VariantInfo *vi = find_variant(reg, f64 && !refine, acc, np, ptri, pf.st, pf.rpt, alg, fa);
            if (!vi) continue;
            uint32_t cap = cfg.max_threads ? cfg.max_threads : (uint32_t)vi->max_threads;
            cap = std::min<uint32_t>(cap, (uint32_t)vi->max_threads);
            const uint32_t c_lo = cfg.cluster_size ? cfg.cluster_size : from;
            const uint32_t c_hi = cfg.cluster_size ? cfg.cluster_size : 16;
            for (uint32_t C = c_lo; C <= c_hi; ++C) {
                if (C > 8 && (C & (C - 1))) continue;  // large clusters: powers of two only
                const uint32_t K = (N + C - 1) / C;
                const uint32_t thr = (K * n + pf.rpt - 1) / pf.rpt;
                if (thr > cap && !streamed(pf.st)) continue;
                // CTA sizes are rounded to 64 threads so that systems of similar
                // size share a launch (streamed rows: up to the cap, in row groups)
                uint32_t threads = std::min<uint32_t>(cap, std::max<uint32_t>(64, (thr + 63) / 64 * 64));
                if (threads < thr && !streamed(pf.st)) threads = (thr + 31) / 32 * 32;
                // shared memory at the largest CTA the class may get (streamed rows:
                // at this CTA, whose vectors are what bound the system)
                const uint32_t chk_warps = streamed(pf.st) ? threads / 32 : 32;
                if (vi->v.smem_bytes(K, C, chk_warps) > (size_t)reg->max_smem_optin) continue;
                s.vi = vi;
                s.C = C;
                s.K = K;
                s.threads = threads;
                *out = s;
                return GBDPCG_SUCCESS;
            }
        }
        if (from == 1) break;  // the second pass would repeat the first
    }
    if (cfg.algorithm == GBDPCG_ALGO_AUTO && layout == GBDPCG_PINV_CBTD) {
        s.plain = true;  // too large for 16 CTAs of rows: one CTA per knot
        *out = s;
        return GBDPCG_SUCCESS;
    }
    return fail(GBDPCG_ERR_UNSUPPORTED, "no cluster shape holds n=" + std::to_string(n) +
                                            " N=" + std::to_string(N));
}

}  // namespace

namespace gbdpcg {
// Message returned by gbdpcg_last_error() on this thread (for entry points in
// other translation units).
void set_last_error(const std::string &msg) { t_last_error = msg; }
}  // namespace gbdpcg

// ------------------------------------------------------------------ handle
constexpr size_t kWorkspaceBytes = 4096;  // 2 result slots + 256 pad + descriptor + prefix

struct gbdpcg_handle_s {
    int device = 0;
    Registry *reg = nullptr;
    DevBuf ws;          // fixed-size: result slots, one descriptor (never reallocated)
    DevBuf host_io;     // host-pointer solve: S, Pinv, gamma, lambda
    DevBuf plain_scratch;  // plain algorithm: r, p, dot partials
    SysResult *d_last = nullptr;
    cudaStream_t last_stream = nullptr;
    bool last_f64 = false;
    std::mutex tune_mu;  // guards `tune`
    std::map<TuneKey, TuneChoice> tune;
};

namespace {

struct HandleScope {  // makes the handle's device current for the duration of a call
    int prev = -1;
    explicit HandleScope(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~HandleScope() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

void to_public(const SysResult &r, gbdpcg_result *o) {
    o->iters = r.iters;
    o->status = r.status;
    o->eta = r.eta;
    o->relres = (r.rr >= 0 && r.gg > 0) ? sqrt(r.rr / r.gg) : (r.rr >= 0 ? 0.0 : -1.0);
    o->outer = r.outer;
    o->reserved = 0;
}

SysDesc make_desc(const void *S, const void *P, const void *g, const void *l0, void *l,
                  uint32_t n, uint32_t N, const gbdpcg_config &cfg, uint32_t layout,
                  uint32_t result_slot) {
    SysDesc d;
    memset(&d, 0, sizeof(d));
    d.S = S;
    d.P = P;
    d.gamma = g;
    d.lambda0 = l0;
    d.lambda = l;
    d.tol = cfg.exit_tol;
    d.inner_tol = cfg.inner_tol;
    d.max_outer = cfg.max_outer;
    d.n = n;
    d.N = N;
    d.max_iter = cfg.max_iter;
    d.flags = (cfg.exit_mode == GBDPCG_EXIT_RELRES ? SYS_EXIT_RELRES : 0u) |
              (layout == GBDPCG_PINV_CBTD ? SYS_PINV_TRI : 0u) |
              (cfg.zero_guess ? SYS_LAMBDA0_ZERO : 0u);
    d.result = result_slot;
    return d;
}

int check_cfg(const gbdpcg_config *cfg, uint32_t layout) {
    if (!cfg) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "config is NULL");
    if (layout > GBDPCG_PINV_BLOCKDIAG) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "bad pinv_layout");
    if (cfg->exit_mode > GBDPCG_EXIT_RELRES || cfg->dot_precision > GBDPCG_DOT_FLOAT2 ||
        cfg->algorithm > GBDPCG_ALGO_RECURRENCE || cfg->storage > GBDPCG_STORAGE_STREAM ||
        cfg->cluster_size > 16 || cfg->max_threads > 1024 || cfg->zero_guess > 1 ||
        !(cfg->inner_tol >= 0) || cfg->inner_tol >= 1)
        return fail(GBDPCG_ERR_INVALID_ARGUMENT, "bad config field");
    if (!(cfg->exit_tol >= 0)) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "exit_tol must be >= 0");
    return GBDPCG_SUCCESS;
}

}  // namespace

namespace gbdpcg {
// The config checks of the handle entry points, for entry points in other
// translation units (a config one entry point rejects, every one rejects).
int check_config(const gbdpcg_config *cfg, uint32_t layout) { return check_cfg(cfg, layout); }
}  // namespace gbdpcg

namespace {

// Launch the plain algorithm for one system (cooperative, N CTAs of 64 threads).
int launch_plain(gbdpcg_handle_s *h, bool f64, const SysDesc &d, SysResult *d_res,
                 cudaStream_t stream, DevBuf &scratch) {
    const size_t s = f64 ? 8 : 4;
    const size_t vec = (size_t)d.n * d.N * s;
    const size_t need = 2 * vec + 2 * (size_t)d.N * s + 256;
    int rc = scratch.ensure(need);
    if (rc) return rc;
    char *base = scratch.as<char>();
    void *d_r = base, *d_p = base + vec, *d_p1 = base + 2 * vec, *d_p2 = base + 2 * vec + d.N * s;
    const void *func = plain_kernel_ptr(f64);
    const size_t smem = plain_smem_bytes(f64, d.n, d.N);
    if (smem > (size_t)h->reg->max_smem_optin)
        return fail(GBDPCG_ERR_UNSUPPORTED, "plain algorithm: block row exceeds shared memory");
    if (smem > 48 * 1024)
        GB_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, 64, smem));
    if ((int64_t)per_sm * h->reg->sm_count < (int64_t)d.N)
        return fail(GBDPCG_ERR_UNSUPPORTED, "plain algorithm: knots exceed co-resident CTAs");
    uint32_t n = d.n, N = d.N, mi = d.max_iter, fl = d.flags;
    double tol = d.tol;
    const void *S = d.S, *P = d.P, *g = d.gamma, *l0 = d.lambda0;
    void *l = d.lambda;
    void *args[] = {&S, &P, &g, &l0, &l, &d_r, &d_p, &d_p1, &d_p2, &n, &N, &mi, &tol, &fl, &d_res};
    GB_CUDA(cudaLaunchCooperativeKernel(func, dim3(N), dim3(64), args, smem, stream));
    return GBDPCG_SUCCESS;
}

int launch_cluster(const Shape &sh, const LaunchParams &lp, uint32_t grid_clusters,
                   cudaStream_t stream) {
    const size_t smem = sh.vi->v.smem_bytes(lp.kmax, sh.C, sh.threads / 32);
    int rc = prepare_variant(sh.vi, smem, sh.C);
    if (rc) return rc;
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = sh.C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(grid_clusters * sh.C);
    cfg.blockDim = dim3(sh.threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void *args[] = {const_cast<LaunchParams *>(&lp)};
    GB_CUDA(cudaLaunchKernelExC(&cfg, sh.vi->v.func, args));
    return GBDPCG_SUCCESS;
}

int max_active_clusters(const Shape &sh, size_t smem, int *out) {
    int rc = prepare_variant(sh.vi, smem, sh.C);
    if (rc) return rc;
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = sh.C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(sh.C);
    cfg.blockDim = dim3(sh.threads);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    GB_CUDA(cudaOccupancyMaxActiveClusters(out, sh.vi->v.func, &cfg));
    return GBDPCG_SUCCESS;
}

// One system, device pointers; result left in h->d_last.
int solve_one(gbdpcg_handle_s *h, bool f64, const SysDesc &d0, const gbdpcg_config &cfg,
              uint32_t layout, cudaStream_t stream, bool refine = false) {
    SysResult *d_res = h->ws.as<SysResult>();
    int rc;
    SysDesc d = d0;
    d.result = 0;
    Shape sh;
    rc = choose_shape(h->reg, f64, d.n, d.N, layout, cfg, &sh, refine, nullptr,
                      lone_cluster_pref(f64 && !refine, d.N), true);
    if (rc) return rc;
    h->d_last = d_res;
    h->last_stream = stream;
    if (sh.plain) {
        return launch_plain(h, f64, d, d_res, stream, h->plain_scratch);
    }
    LaunchParams lp;
    memset(&lp, 0, sizeof(lp));
    lp.descs = nullptr;
    lp.order = nullptr;
    lp.count = 1;
    lp.kmax = sh.K;
    lp.queue = nullptr;
    lp.results = d_res;
    lp.one = d;
    return launch_cluster(sh, lp, 1, stream);
}

}  // namespace

// ------------------------------------------------------------------ plan
struct PlanClass {
    Shape sh;
    uint32_t kmax = 0;
    std::vector<uint32_t> items;  // indices into descs
    uint32_t order_off = 0;
    uint32_t grid_clusters = 0;
};

struct gbdpcg_plan_s {
    gbdpcg_handle_s *h = nullptr;
    bool f64 = false;
    bool refine = false;  // FP64 systems by FP32 PCG + FP64 refinement
    uint32_t layout = 0;
    gbdpcg_config cfg;
    uint32_t count = 0;
    std::vector<SysDesc> descs;
    std::vector<PlanClass> classes;
    std::vector<uint32_t> plain_items;
    DevBuf d_descs, d_order, d_queues, d_results, d_prefix;
    DevBuf plain_scratch;
    uint64_t total_knots = 0;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    // packed plans: the device arenas and their sizes in bytes
    bool packed = false;
    int dtype = 0;
    const void *arena_S = nullptr, *arena_P = nullptr, *arena_g = nullptr;
    void *arena_l = nullptr;
    size_t bytes_S = 0, bytes_P = 0, bytes_vec = 0;
    std::vector<gbdpcg_packed_system> packed_list;
    // execute_host pipeline (built on first use): pieces of consecutive systems,
    // each a plan of its own over the same arenas, with byte ranges [lo, hi)
    bool pieces_built = false;
    struct Piece {
        gbdpcg_plan_s *plan = nullptr;
        uint32_t first = 0, count = 0;
        size_t S0 = 0, S1 = 0, P0 = 0, P1 = 0, V0 = 0, V1 = 0;
    };
    std::vector<Piece> pieces;
    cudaStream_t copy_stream = nullptr;
    cudaStream_t build_stream = nullptr;  // highest priority: the Phi^-1 builds of solve_host
    std::vector<cudaStream_t> piece_streams;
    std::vector<cudaEvent_t> piece_events;  // [copied i], [solved i], start, [built i]
    // forward + adjoint pairs (gbdpcg_plan_create_fwd_adj): results [0, count)
    // are the forward solves', [count, 2 count) the adjoint solves'
    bool fused = false;
    uint32_t nresults = 0;
    // timeline (gbdpcg_plan_timeline): one record per work-list item, and the
    // SM of every CTA of every launch (launch c's CTAs from cta_off[c])
    bool timeline = false;
    DevBuf d_stamps, d_ctasm;
    std::vector<uint32_t> cta_off;
    ~gbdpcg_plan_s() {
        for (auto &pc : pieces) delete pc.plan;
        if (copy_stream) cudaStreamDestroy(copy_stream);
        if (build_stream) cudaStreamDestroy(build_stream);
        for (auto s : piece_streams) cudaStreamDestroy(s);
        for (auto e : piece_events) cudaEventDestroy(e);
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        for (auto s : streams) cudaStreamDestroy(s);
        for (auto e : events) cudaEventDestroy(e);
    }
};

namespace {

// adjoint: 0 forward solves, 1 adjoint solves, 2 forward + adjoint pairs
TuneKey tune_key(const gbdpcg_plan_s *p, uint8_t adjoint, uint32_t n, uint32_t N) {
    TuneKey k;
    memset(&k, 0, sizeof(k));
    k.f64 = p->f64;
    k.refine = p->refine;
    k.acc = (uint8_t)acc_kind(p->f64, p->refine, p->cfg.dot_precision);
    k.ptri = p->layout == GBDPCG_PINV_CBTD;
    k.adjoint = adjoint;
    k.alg_req = (uint8_t)p->cfg.algorithm;
    k.storage_req = (uint8_t)p->cfg.storage;
    k.n = n;
    k.N = N;
    return k;
}

int timeline_buffers(gbdpcg_plan_s *p);

// Merges classes with the same launch shape, orders each class's systems
// longest first and the classes by their largest system, builds the device
// work list, sizes each persistent grid to the clusters that fit at once, and
// drops a captured graph (the next execution captures the new launches).
// Merges the classes that share a launch shape, orders each class's systems
// by decreasing cost n^2 N (the queue hands out the longest first) and the
// classes by their largest system, and sizes each grid to the clusters that
// fit at once; `order` receives the work list of all classes.
int layout_classes(const std::vector<SysDesc> &descs, std::vector<PlanClass> &classes,
                   std::vector<uint32_t> &order) {
    std::vector<PlanClass> merged;
    std::map<std::tuple<const void *, uint32_t, uint32_t>, size_t> index;
    for (auto &pc : classes) {
        auto key = std::make_tuple((const void *)pc.sh.vi, pc.sh.C, pc.sh.threads);
        auto it = index.find(key);
        if (it == index.end()) {
            index.emplace(key, merged.size());
            merged.push_back(pc);
        } else {
            PlanClass &m = merged[it->second];
            m.items.insert(m.items.end(), pc.items.begin(), pc.items.end());
            m.kmax = std::max(m.kmax, pc.kmax);
        }
    }
    classes.swap(merged);
    auto cost = [&](uint32_t i) { return (double)descs[i].n * descs[i].n * descs[i].N; };
    for (auto &pc : classes)
        std::stable_sort(pc.items.begin(), pc.items.end(),
                         [&](uint32_t a, uint32_t b) { return cost(a) > cost(b); });
    std::stable_sort(classes.begin(), classes.end(),
                     [&](const PlanClass &a, const PlanClass &b) {
                         return cost(a.items[0]) > cost(b.items[0]);
                     });
    order.clear();
    for (auto &pc : classes) {
        pc.order_off = (uint32_t)order.size();
        order.insert(order.end(), pc.items.begin(), pc.items.end());
        int active = 0;
        int rc = max_active_clusters(pc.sh, pc.sh.vi->v.smem_bytes(pc.kmax, pc.sh.C, pc.sh.threads / 32), &active);
        if (rc) return rc;
        if (active <= 0)
            return fail(GBDPCG_ERR_UNSUPPORTED, "cluster shape cannot be scheduled (C=" +
                                                    std::to_string(pc.sh.C) + ")");
        pc.grid_clusters = std::min<uint32_t>((uint32_t)pc.items.size(), (uint32_t)active);
    }
    return GBDPCG_SUCCESS;
}

int plan_layout(gbdpcg_plan_s *p) {
    std::vector<uint32_t> order;
    if (int lrc = layout_classes(p->descs, p->classes, order)) return lrc;
    int rc;
    if ((rc = p->d_order.ensure(sizeof(uint32_t) * std::max<size_t>(1, order.size())))) return rc;
    if ((rc = p->d_queues.ensure(sizeof(uint32_t) * std::max<size_t>(1, p->classes.size())))) return rc;
    if (!order.empty())
        GB_CUDA(cudaMemcpy(p->d_order.p, order.data(), sizeof(uint32_t) * order.size(),
                           cudaMemcpyHostToDevice));
    if (p->timeline && (rc = timeline_buffers(p))) return rc;
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    if (p->graph) cudaGraphDestroy(p->graph);
    p->gexec = nullptr;
    p->graph = nullptr;
    return GBDPCG_SUCCESS;
}

// Sizes the timeline buffers to the current launch classes (called whenever
// the layout changes while the timeline is on, never during a capture).
int timeline_buffers(gbdpcg_plan_s *p) {
    p->cta_off.assign(p->classes.size() + 1, 0);
    size_t items = 0;
    for (size_t c = 0; c < p->classes.size(); ++c) {
        items += p->classes[c].items.size();
        p->cta_off[c + 1] = p->cta_off[c] + p->classes[c].grid_clusters * p->classes[c].sh.C;
    }
    int rc;
    if ((rc = p->d_stamps.ensure(sizeof(StampRec) * std::max<size_t>(1, items)))) return rc;
    if ((rc = p->d_ctasm.ensure(sizeof(uint32_t) * std::max<size_t>(1, p->cta_off.back())))) return rc;
    GB_CUDA(cudaMemset(p->d_stamps.p, 0, sizeof(StampRec) * std::max<size_t>(1, items)));
    return GBDPCG_SUCCESS;
}

int plan_enqueue(gbdpcg_plan_s *p, cudaStream_t stream) {
    const uint32_t nc = (uint32_t)p->classes.size();
    if (nc) GB_CUDA(cudaMemsetAsync(p->d_queues.p, 0, sizeof(uint32_t) * nc, stream));
    GB_CUDA(cudaEventRecord(p->events[0], stream));
    const uint32_t ns = (uint32_t)p->streams.size();
    for (uint32_t c = 0; c < nc; ++c) {
        cudaStream_t s = p->streams[c % ns];
        if (c < ns) GB_CUDA(cudaStreamWaitEvent(s, p->events[0], 0));
        const PlanClass &pc = p->classes[c];
        LaunchParams lp;
        memset(&lp, 0, sizeof(lp));
        lp.descs = p->d_descs.as<SysDesc>();
        lp.order = p->d_order.as<uint32_t>() + pc.order_off;
        lp.count = (uint32_t)pc.items.size();
        lp.kmax = pc.kmax;
        lp.queue = p->d_queues.as<uint32_t>() + c;
        lp.results = p->d_results.as<SysResult>();
        lp.launch_id = c;
        if (p->timeline) {
            lp.stamps = p->d_stamps.as<StampRec>() + pc.order_off;
            lp.cta_sm = p->d_ctasm.as<uint32_t>() + p->cta_off[c];
        }
        int rc = launch_cluster(pc.sh, lp, pc.grid_clusters, s);
        if (rc) return rc;
    }
    for (uint32_t s = 0; s < std::min(ns, nc); ++s) {
        GB_CUDA(cudaEventRecord(p->events[1 + s], p->streams[s]));
        GB_CUDA(cudaStreamWaitEvent(stream, p->events[1 + s], 0));
    }
    for (uint32_t idx : p->plain_items) {
        int rc = launch_plain(p->h, p->f64, p->descs[idx], p->d_results.as<SysResult>() + idx,
                              stream, p->plain_scratch);
        if (rc) return rc;
    }
    return GBDPCG_SUCCESS;
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" {

int gbdpcg_version(void) { return GBDPCG_VERSION; }

const char *gbdpcg_status_string(int s) {
    switch (s) {
        case GBDPCG_SUCCESS: return "success";
        case GBDPCG_ERR_INVALID_ARGUMENT: return "invalid argument";
        case GBDPCG_ERR_UNSUPPORTED: return "unsupported size or option";
        case GBDPCG_ERR_CUDA: return "CUDA error";
        case GBDPCG_ERR_NO_MEMORY: return "out of device memory";
        case GBDPCG_ERR_NOT_CONVERGED: return "not converged";
        default: return "unknown status";
    }
}

const char *gbdpcg_last_error(void) { return t_last_error.c_str(); }

void gbdpcg_config_init(gbdpcg_config *cfg) {
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->exit_tol = 1e-6;
    cfg->max_iter = 25;
    cfg->exit_mode = GBDPCG_EXIT_REFERENCE;
    cfg->dot_precision = GBDPCG_DOT_NATIVE;
    cfg->algorithm = GBDPCG_ALGO_AUTO;
    cfg->use_graph = 1;
    cfg->max_outer = 50;
    cfg->streams = 8;
    cfg->inner_tol = 0.05;
}

int gbdpcg_create(gbdpcg_handle_t *handle, int device) {
    if (!handle) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "handle is NULL");
    int ndev = 0;
    GB_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "bad device");
    HandleScope scope(device);
    auto h = std::make_unique<gbdpcg_handle_s>();
    h->device = device;
    int rc = get_registry(device, &h->reg);
    if (rc) return rc;
    rc = h->ws.ensure(kWorkspaceBytes);
    if (rc) return rc;
    *handle = h.release();
    return GBDPCG_SUCCESS;
}

int gbdpcg_destroy(gbdpcg_handle_t handle) {
    if (!handle) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "handle is NULL");
    HandleScope scope(handle->device);
    delete handle;
    return GBDPCG_SUCCESS;
}

static int solve_dev(gbdpcg_handle_t h, bool f64, const void *S, const void *P, uint32_t layout,
                     const void *g, void *l, uint32_t n, uint32_t N, const gbdpcg_config *cfg,
                     gbdpcg_result *result, cudaStream_t stream) {
    if (!h || !S || !P || !g || !l) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (n == 0 || N == 0) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "n and N must be positive");
    int rc = check_cfg(cfg, layout);
    if (rc) return rc;
    HandleScope scope(h->device);
    SysDesc d = make_desc(S, P, g, l, l, n, N, *cfg, layout, 0);
    rc = solve_one(h, f64, d, *cfg, layout, stream);
    if (rc) return rc;
    h->last_f64 = f64;
    if (result) return gbdpcg_last_result(h, result);
    return GBDPCG_SUCCESS;
}

int gbdpcg_solve_dev_f32(gbdpcg_handle_t h, const float *d_S, const float *d_Pinv,
                         uint32_t pinv_layout, const float *d_gamma, float *d_lambda, uint32_t n,
                         uint32_t N, const gbdpcg_config *cfg, gbdpcg_result *result,
                         gbdpcg_stream_t stream) {
    return solve_dev(h, false, d_S, d_Pinv, pinv_layout, d_gamma, d_lambda, n, N, cfg, result,
                     (cudaStream_t)stream);
}

int gbdpcg_solve_dev_f64(gbdpcg_handle_t h, const double *d_S, const double *d_Pinv,
                         uint32_t pinv_layout, const double *d_gamma, double *d_lambda,
                         uint32_t n, uint32_t N, const gbdpcg_config *cfg,
                         gbdpcg_result *result, gbdpcg_stream_t stream) {
    return solve_dev(h, true, d_S, d_Pinv, pinv_layout, d_gamma, d_lambda, n, N, cfg, result,
                     (cudaStream_t)stream);
}

int gbdpcg_last_result(gbdpcg_handle_t h, gbdpcg_result *result) {
    if (!h || !result || !h->d_last) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "no result");
    HandleScope scope(h->device);
    SysResult r;
    GB_CUDA(cudaMemcpyAsync(&r, h->d_last, sizeof(r), cudaMemcpyDeviceToHost, h->last_stream));
    GB_CUDA(cudaStreamSynchronize(h->last_stream));
    to_public(r, result);
    return GBDPCG_SUCCESS;
}

static int block_jacobi(gbdpcg_handle_t h, int kind, const void *S, void *P, uint32_t layout,
                        uint32_t n, uint32_t N, cudaStream_t stream) {
    if (!h || !S || !P) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (n == 0 || N == 0 || n > 32) return fail(GBDPCG_ERR_UNSUPPORTED, "block-Jacobi needs 1 <= n <= 32");
    if (layout > GBDPCG_PINV_BLOCKDIAG) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "bad layout");
    HandleScope scope(h->device);
    // the one descriptor goes to the kernel by value: stream-ordered, no upload
    SysDesc d;
    memset(&d, 0, sizeof(d));
    d.S = S;
    d.P = P;
    d.n = n;
    d.N = N;
    GB_CUDA(launch_block_jacobi(kind, nullptr, nullptr, 1, N, layout == GBDPCG_PINV_CBTD, stream, &d));
    return GBDPCG_SUCCESS;
}

int gbdpcg_block_jacobi_f32(gbdpcg_handle_t h, const float *d_S, float *d_Pinv,
                            uint32_t pinv_layout, uint32_t n, uint32_t N,
                            gbdpcg_stream_t stream) {
    return block_jacobi(h, 0, d_S, d_Pinv, pinv_layout, n, N, (cudaStream_t)stream);
}

int gbdpcg_block_jacobi_f64(gbdpcg_handle_t h, const double *d_S, double *d_Pinv,
                            uint32_t pinv_layout, uint32_t n, uint32_t N,
                            gbdpcg_stream_t stream) {
    return block_jacobi(h, 1, d_S, d_Pinv, pinv_layout, n, N, (cudaStream_t)stream);
}

int gbdpcg_block_jacobi_f64to32(gbdpcg_handle_t h, const double *d_S, float *d_Pinv, uint32_t n,
                                uint32_t N, gbdpcg_stream_t stream) {
    return block_jacobi(h, 2, d_S, d_Pinv, GBDPCG_PINV_BLOCKDIAG, n, N, (cudaStream_t)stream);
}

int gbdpcg_refine_solve_dev(gbdpcg_handle_t h, const double *d_S, const float *d_Pinv,
                            const double *d_gamma, double *d_lambda, uint32_t n, uint32_t N,
                            const gbdpcg_config *cfg, gbdpcg_result *result,
                            gbdpcg_stream_t stream) {
    if (!h || !d_S || !d_Pinv || !d_gamma || !d_lambda)
        return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (n == 0 || N == 0) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "n and N must be positive");
    int rc = check_cfg(cfg, GBDPCG_PINV_BLOCKDIAG);
    if (rc) return rc;
    if (cfg->exit_mode != GBDPCG_EXIT_RELRES)
        return fail(GBDPCG_ERR_UNSUPPORTED, "refinement exits on the relative residual");
    HandleScope scope(h->device);
    SysDesc d = make_desc(d_S, d_Pinv, d_gamma, d_lambda, d_lambda, n, N, *cfg,
                          GBDPCG_PINV_BLOCKDIAG, 0);
    d.flags |= SYS_REFINE;
    rc = solve_one(h, false, d, *cfg, GBDPCG_PINV_BLOCKDIAG, (cudaStream_t)stream, true);
    if (rc) return rc;
    h->last_f64 = true;
    if (result) return gbdpcg_last_result(h, result);
    return GBDPCG_SUCCESS;
}

// ---- host-pointer solves (per-thread handle on the current device)
static int thread_handle(gbdpcg_handle_t *out) {
    static thread_local std::map<int, gbdpcg_handle_t> handles;
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    auto it = handles.find(dev);
    if (it != handles.end()) {
        *out = it->second;
        return GBDPCG_SUCCESS;
    }
    gbdpcg_handle_t h = nullptr;
    int rc = gbdpcg_create(&h, dev);
    if (rc) return rc;
    handles[dev] = h;
    *out = h;
    return GBDPCG_SUCCESS;
}

static int solve_host(bool f64, const void *S, const void *P, const void *g, void *l, uint32_t n,
                      uint32_t N, const gbdpcg_config *cfg, gbdpcg_result *result) {
    if (!S || !g || !l) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (n == 0 || N == 0) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "n and N must be positive");
    gbdpcg_config c;
    if (cfg) c = *cfg;
    else gbdpcg_config_init(&c);
    const uint32_t layout = P ? GBDPCG_PINV_CBTD : GBDPCG_PINV_BLOCKDIAG;
    int rc = check_cfg(&c, layout);
    if (rc) return rc;
    gbdpcg_handle_t h = nullptr;
    rc = thread_handle(&h);
    if (rc) return rc;
    const size_t s = f64 ? 8 : 4;
    const size_t mat = (size_t)3 * n * n * N * s, vec = (size_t)n * N * s;
    // when Phi^-1 is built here, the plain algorithm still needs the cbtd layout
    const uint32_t build_layout =
        (!P && (c.algorithm == GBDPCG_ALGO_PLAIN || n > 32)) ? GBDPCG_PINV_CBTD : layout;
    const size_t pmat = P || build_layout == GBDPCG_PINV_CBTD ? mat : (size_t)n * n * N * s;
    cudaStream_t st = nullptr;
    // Where the GPU reads host memory through the host's page tables, the
    // kernels use the caller's arrays in place: S, Phi^-1 and gamma are read
    // once per solve and lambda is written once, so there are no staging
    // copies (GBDPCG_HOST_STAGING=1 forces the copies).  The results are the
    // same bits either way.
    const char *stage_env = getenv("GBDPCG_HOST_STAGING");
    const bool direct = h->reg->host_direct && !(stage_env && stage_env[0] == '1');
    char *dS, *dP, *dg, *dl;
    if (direct) {
        if (!P) {
            rc = h->host_io.ensure(pmat + 256);
            if (rc) return rc;
        }
        dS = static_cast<char *>(const_cast<void *>(S));
        dP = P ? static_cast<char *>(const_cast<void *>(P)) : h->host_io.as<char>();
        dg = static_cast<char *>(const_cast<void *>(g));
        dl = static_cast<char *>(l);
    } else {
        rc = h->host_io.ensure(mat + pmat + 2 * vec + 1024);
        if (rc) return rc;
        dS = h->host_io.as<char>();
        dP = dS + round_up(mat, 256);
        dg = dP + round_up(pmat, 256);
        dl = dg + round_up(vec, 256);
        GB_CUDA(cudaMemcpyAsync(dS, S, mat, cudaMemcpyHostToDevice, st));
        if (P) GB_CUDA(cudaMemcpyAsync(dP, P, mat, cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaMemcpyAsync(dg, g, vec, cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaMemcpyAsync(dl, l, vec, cudaMemcpyHostToDevice, st));
    }
    if (!P) {
        if (n > 32) return fail(GBDPCG_ERR_UNSUPPORTED, "block-Jacobi builder needs n <= 32");
        rc = block_jacobi(h, f64 ? 1 : 0, dS, dP, build_layout, n, N, st);
        if (rc) return rc;
    }
    rc = solve_dev(h, f64, dS, dP, build_layout, dg, dl, n, N, &c, nullptr, st);
    if (rc) return rc;
    if (!direct) GB_CUDA(cudaMemcpyAsync(l, dl, vec, cudaMemcpyDeviceToHost, st));
    gbdpcg_result r;
    rc = gbdpcg_last_result(h, &r);
    if (rc) return rc;
    if (result) *result = r;
    return GBDPCG_SUCCESS;
}

int gbdpcg_solve_f32(const float *S, const float *Pinv, const float *gamma, float *lambda,
                     uint32_t n, uint32_t N, const gbdpcg_config *cfg, gbdpcg_result *result) {
    return solve_host(false, S, Pinv, gamma, lambda, n, N, cfg, result);
}

int gbdpcg_solve_f64(const double *S, const double *Pinv, const double *gamma, double *lambda,
                     uint32_t n, uint32_t N, const gbdpcg_config *cfg, gbdpcg_result *result) {
    return solve_host(true, S, Pinv, gamma, lambda, n, N, cfg, result);
}

int gbdpcg_adjoint_dev_f32(gbdpcg_handle_t h, const float *d_S, const float *d_Pinv,
                           uint32_t pinv_layout, const float *d_lambda, const float *d_grad_lambda,
                           float *d_grad_gamma, float *d_grad_S, uint32_t n, uint32_t N,
                           const gbdpcg_config *cfg, gbdpcg_result *result,
                           gbdpcg_stream_t stream) {
    if (!h || !d_S || !d_Pinv || !d_lambda || !d_grad_lambda || !d_grad_gamma || !d_grad_S)
        return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (n == 0 || N == 0) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "n and N must be positive");
    int rc = check_cfg(cfg, pinv_layout);
    if (rc) return rc;
    if (cfg->algorithm == GBDPCG_ALGO_PLAIN || n > 32)
        return fail(GBDPCG_ERR_UNSUPPORTED, "adjoint runs on the cluster solver (n <= 32)");
    HandleScope scope(h->device);
    SysDesc d = make_desc(d_S, d_Pinv, d_grad_lambda, nullptr, d_grad_gamma, n, N, *cfg,
                          pinv_layout, 0);
    d.flags |= SYS_ADJOINT | SYS_LAMBDA0_ZERO;
    d.lam_fwd = d_lambda;
    d.dS = d_grad_S;
    rc = solve_one(h, false, d, *cfg, pinv_layout, (cudaStream_t)stream);
    if (rc) return rc;
    h->last_f64 = false;
    if (result) return gbdpcg_last_result(h, result);
    return GBDPCG_SUCCESS;
}

// ---- plans
}  // extern "C"

namespace {

// Builds a plan.  With `fa`, every system is a forward + adjoint pair (the
// forward fields are in `systems`, the adjoint's outputs and lambda* in fa).
int plan_create_impl(gbdpcg_handle_t h, int dtype, const gbdpcg_system *systems, uint32_t count,
                     uint32_t pinv_layout, const gbdpcg_config *cfg, gbdpcg_plan_t *plan,
                     const gbdpcg_fwd_adj_system *fa) {
    if (!h || !systems || !plan || count == 0)
        return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer or empty batch");
    if (dtype < 0 || dtype > 2) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "dtype must be 0, 1 or 2");
    int rc = check_cfg(cfg, pinv_layout);
    if (rc) return rc;
    if (dtype == 2 && (pinv_layout != GBDPCG_PINV_BLOCKDIAG || cfg->exit_mode != GBDPCG_EXIT_RELRES))
        return fail(GBDPCG_ERR_UNSUPPORTED, "refinement needs a compact Phi^-1 and the relative-residual exit");
    HandleScope scope(h->device);
    auto p = std::make_unique<gbdpcg_plan_s>();
    p->h = h;
    p->f64 = dtype == 1;
    p->refine = dtype == 2;
    p->layout = pinv_layout;
    p->cfg = *cfg;
    p->count = count;
    p->fused = fa != nullptr;
    p->nresults = fa ? 2 * count : count;
    if (fa && p->refine) return fail(GBDPCG_ERR_UNSUPPORTED, "no adjoint of a refined solve");
    const bool adjoint = systems[0].lambda_fwd != nullptr;
    std::map<std::tuple<const void *, uint32_t, uint32_t>, uint32_t> class_of;
    std::vector<uint64_t> prefix(count);
    // tuned shapes apply unless the config pins the cluster or CTA size
    const bool use_table = !cfg->cluster_size && !cfg->max_threads;
    std::unique_lock<std::mutex> tune_lock(h->tune_mu);
    for (uint32_t i = 0; i < count; ++i) {
        const gbdpcg_system &s = systems[i];
        if (!s.S || !s.Pinv || !s.gamma || !s.lambda || s.n == 0 || s.N == 0)
            return fail(GBDPCG_ERR_INVALID_ARGUMENT, "system " + std::to_string(i) + " is incomplete");
        if ((s.lambda_fwd != nullptr) != adjoint || (adjoint && !s.dS))
            return fail(GBDPCG_ERR_INVALID_ARGUMENT, "mixed forward and adjoint systems");
        SysDesc d = make_desc(s.S, s.Pinv, s.gamma, s.lambda, s.lambda, s.n, s.N, *cfg,
                              pinv_layout, i);
        if (adjoint) {
            if (p->refine) return fail(GBDPCG_ERR_UNSUPPORTED, "no adjoint of a refined solve");
            d.flags |= SYS_ADJOINT | SYS_LAMBDA0_ZERO;
            d.lam_fwd = s.lambda_fwd;
            d.dS = s.dS;
        }
        if (p->refine) d.flags |= SYS_REFINE;
        if (fa) {
            const gbdpcg_fwd_adj_system &f = fa[i];
            if (!f.lambda_target || !f.grad_gamma || !f.grad_S)
                return fail(GBDPCG_ERR_INVALID_ARGUMENT, "system " + std::to_string(i) + " is incomplete");
            d.flags |= SYS_FWD_ADJ;
            d.lstar = f.lambda_target;
            d.mu = f.grad_gamma;
            d.dS = f.grad_S;
            d.lam_fwd = f.lambda;  // the epilogue's forward solution is the lambda output
            d.result_adj = count + i;
        }
        prefix[i] = p->total_knots;
        p->total_knots += s.N;
        p->descs.push_back(d);
        Shape sh;
        const TuneChoice *tc = nullptr;
        TuneChoice tcv;
        if (use_table) {
            auto tt = h->tune.find(tune_key(p.get(), fa ? 2 : (adjoint ? 1 : 0), s.n, s.N));
            if (tt != h->tune.end()) {
                tcv = tt->second;
                tc = &tcv;
            }
        }
        rc = choose_shape(h->reg, p->f64, s.n, s.N, pinv_layout, *cfg, &sh, p->refine, tc, 1, false, fa != nullptr);
        if (rc) return rc;
        if (fa && (sh.plain || streamed(sh.vi->v.st)))
            return fail(GBDPCG_ERR_UNSUPPORTED, "a forward + adjoint pair needs the rows on chip (system " +
                                                    std::to_string(i) + ")");
        if (sh.plain) {
            if (adjoint) return fail(GBDPCG_ERR_UNSUPPORTED, "adjoint needs n <= 32");
            p->plain_items.push_back(i);
            continue;
        }
        auto key = std::make_tuple((const void *)sh.vi, sh.C, sh.threads);
        auto it = class_of.find(key);
        if (it == class_of.end()) {
            PlanClass pc;
            pc.sh = sh;
            it = class_of.emplace(key, (uint32_t)p->classes.size()).first;
            p->classes.push_back(pc);
        }
        PlanClass &pc = p->classes[it->second];
        pc.items.push_back(i);
        pc.kmax = std::max(pc.kmax, sh.K);
    }
    tune_lock.unlock();
    if ((rc = p->d_descs.ensure(sizeof(SysDesc) * count))) return rc;
    if ((rc = p->d_results.ensure(sizeof(SysResult) * p->nresults))) return rc;
    if ((rc = p->d_prefix.ensure(sizeof(uint64_t) * count))) return rc;
    GB_CUDA(cudaMemcpy(p->d_descs.p, p->descs.data(), sizeof(SysDesc) * count, cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(p->d_prefix.p, prefix.data(), sizeof(uint64_t) * count, cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemset(p->d_results.p, 0, sizeof(SysResult) * p->nresults));
    if ((rc = plan_layout(p.get()))) return rc;
    const size_t nc = p->classes.size();
    const uint32_t ns = (uint32_t)std::min<size_t>(std::max<uint32_t>(1, std::min<uint32_t>(cfg->streams, 32)),
                                                   std::max<size_t>(1, nc));
    for (uint32_t s = 0; s < ns; ++s) {
        cudaStream_t st;
        GB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        p->streams.push_back(st);
    }
    for (uint32_t e = 0; e < ns + 1; ++e) {
        cudaEvent_t ev;
        GB_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        p->events.push_back(ev);
    }
    *plan = p.release();
    return GBDPCG_SUCCESS;
}

}  // namespace

extern "C" {

int gbdpcg_plan_create(gbdpcg_handle_t h, int dtype, const gbdpcg_system *systems, uint32_t count,
                       uint32_t pinv_layout, const gbdpcg_config *cfg, gbdpcg_plan_t *plan) {
    return plan_create_impl(h, dtype, systems, count, pinv_layout, cfg, plan, nullptr);
}

int gbdpcg_plan_create_fwd_adj(gbdpcg_handle_t h, int dtype, const gbdpcg_fwd_adj_system *systems,
                               uint32_t count, uint32_t pinv_layout, const gbdpcg_config *cfg,
                               gbdpcg_plan_t *plan) {
    if (!systems || count == 0) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer or empty batch");
    if (dtype != 0) return fail(GBDPCG_ERR_UNSUPPORTED, "forward + adjoint pairs are float systems");
    std::vector<gbdpcg_system> fwd(count);
    for (uint32_t i = 0; i < count; ++i) {
        const gbdpcg_fwd_adj_system &f = systems[i];
        fwd[i] = gbdpcg_system{f.S, f.Pinv, f.gamma, f.lambda, nullptr, nullptr, f.n, f.N};
    }
    return plan_create_impl(h, dtype, fwd.data(), count, pinv_layout, cfg, plan, systems);
}

int gbdpcg_plan_execute(gbdpcg_plan_t p, gbdpcg_stream_t stream_) {
    if (!p) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "plan is NULL");
    HandleScope scope(p->h->device);
    cudaStream_t stream = (cudaStream_t)stream_;
    const bool graph = p->cfg.use_graph && p->plain_items.empty();
    if (!graph) return plan_enqueue(p, stream);
    if (!p->gexec) {
        cudaStream_t cap;
        GB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaStreamDestroy(cap);
            GB_CUDA(e);
        }
        int rc = plan_enqueue(p, cap);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(cap, &g);
        cudaStreamDestroy(cap);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        GB_CUDA(e);
        p->graph = g;
        GB_CUDA(cudaGraphInstantiate(&p->gexec, g, 0));
    }
    GB_CUDA(cudaGraphLaunch(p->gexec, stream));
    return GBDPCG_SUCCESS;
}

int gbdpcg_plan_create_packed(gbdpcg_handle_t h, int dtype, const gbdpcg_packed_system *systems,
                              uint32_t count, const void *d_S, const void *d_Pinv,
                              const void *d_gamma, void *d_lambda, uint32_t pinv_layout,
                              const gbdpcg_config *cfg, gbdpcg_plan_t *plan) {
    if (!systems || !d_S || !d_Pinv || !d_gamma || !d_lambda || !plan || count == 0)
        return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer or empty batch");
    if (dtype != 0 && dtype != 1) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "dtype must be 0 or 1");
    const size_t s = dtype ? 8 : 4;  // refinement: S, gamma, lambda double, Pinv float
    const size_t sP = dtype == 1 ? 8 : 4;
    std::vector<gbdpcg_system> sys(count);
    size_t eS = 0, eP = 0, eV = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const gbdpcg_packed_system &q = systems[i];
        const size_t n = q.n, N = q.N;
        const size_t pm = pinv_layout == GBDPCG_PINV_CBTD ? 3 * n * n * N : n * n * N;
        sys[i].S = static_cast<const char *>(d_S) + q.S_off * s;
        sys[i].Pinv = static_cast<const char *>(d_Pinv) + q.Pinv_off * sP;
        sys[i].gamma = static_cast<const char *>(d_gamma) + q.vec_off * s;
        sys[i].lambda = static_cast<char *>(d_lambda) + q.vec_off * s;
        sys[i].lambda_fwd = nullptr;
        sys[i].dS = nullptr;
        sys[i].n = q.n;
        sys[i].N = q.N;
        eS = std::max(eS, (size_t)q.S_off + 3 * n * n * N);
        eP = std::max(eP, (size_t)q.Pinv_off + pm);
        eV = std::max(eV, (size_t)q.vec_off + n * N);
    }
    int rc = gbdpcg_plan_create(h, dtype, sys.data(), count, pinv_layout, cfg, plan);
    if (rc) return rc;
    gbdpcg_plan_s *p = *plan;
    p->packed = true;
    p->dtype = dtype;
    p->packed_list.assign(systems, systems + count);
    p->arena_S = d_S;
    p->arena_P = d_Pinv;
    p->arena_g = d_gamma;
    p->arena_l = d_lambda;
    p->bytes_S = eS * s;
    p->bytes_P = eP * sP;
    p->bytes_vec = eV * s;
    return GBDPCG_SUCCESS;
}

}  // extern "C"

namespace {

// Forgets the execute_host pieces (rebuilt on the next call, e.g. with the
// shapes a new autotuning chose).
void drop_pieces(gbdpcg_plan_s *p) {
    for (auto &pc : p->pieces) delete pc.plan;
    p->pieces.clear();
    if (p->copy_stream) cudaStreamDestroy(p->copy_stream);
    p->copy_stream = nullptr;
    if (p->build_stream) cudaStreamDestroy(p->build_stream);
    p->build_stream = nullptr;
    for (auto s : p->piece_streams) cudaStreamDestroy(s);
    p->piece_streams.clear();
    for (auto e : p->piece_events) cudaEventDestroy(e);
    p->piece_events.clear();
    p->pieces_built = false;
}

// Cuts a packed plan into pieces of consecutive systems for execute_host.
// Needs offsets that increase with the system index in all three arenas, so
// that each piece is one contiguous byte range of each; otherwise (or with one
// piece) execute_host copies the arenas whole.
int build_pieces(gbdpcg_plan_s *p) {
    p->pieces_built = true;
    const uint32_t count = p->count;
    uint32_t k = p->cfg.host_pieces;
    if (k == 0) k = std::min<uint32_t>(8, std::max<uint32_t>(1, count / 512));
    k = std::min(k, count);
    if (k <= 1 || !p->plain_items.empty()) return GBDPCG_SUCCESS;
    const auto &L = p->packed_list;
    for (uint32_t i = 1; i < count; ++i)
        if (L[i].S_off <= L[i - 1].S_off || L[i].Pinv_off <= L[i - 1].Pinv_off || L[i].vec_off <= L[i - 1].vec_off)
            return GBDPCG_SUCCESS;
    const size_t s = p->dtype ? 8 : 4;
    // shares of S bytes, equal but for the last two pieces (3/4 and 1/2 of the
    // others): the solve of the last piece is the one no copy hides, so a
    // shorter last piece ends the pipeline sooner
    std::vector<double> bound(k);
    {
        std::vector<double> w(k, 1.0);
        if (k >= 4) {
            w[k - 2] = 0.75;
            w[k - 1] = 0.5;
        }
        double sum = 0, acc = 0;
        for (double x : w) sum += x;
        for (uint32_t j = 0; j < k; ++j) {
            bound[j] = acc / sum;  // piece j starts at this share
            acc += w[j];
        }
    }
    std::vector<uint32_t> cut = {0};
    const double total = (double)p->bytes_S;
    for (uint32_t i = 1; i < count && cut.size() < k; ++i)
        if ((double)L[i].S_off * s >= total * bound[cut.size()]) cut.push_back(i);
    cut.push_back(count);
    gbdpcg_config cfg = p->cfg;
    cfg.host_pieces = 1;
    for (size_t j = 0; j + 1 < cut.size(); ++j) {
        gbdpcg_plan_s::Piece pc;
        pc.first = cut[j];
        pc.count = cut[j + 1] - cut[j];
        pc.S0 = L[pc.first].S_off * s;
        pc.P0 = L[pc.first].Pinv_off * s;
        pc.V0 = L[pc.first].vec_off * s;
        const bool last = j + 2 == cut.size();
        pc.S1 = last ? p->bytes_S : L[cut[j + 1]].S_off * s;
        pc.P1 = last ? p->bytes_P : L[cut[j + 1]].Pinv_off * s;
        pc.V1 = last ? p->bytes_vec : L[cut[j + 1]].vec_off * s;
        gbdpcg_plan_t sub = nullptr;
        int rc = gbdpcg_plan_create_packed(p->h, p->dtype, L.data() + pc.first, pc.count, p->arena_S,
                                           p->arena_P, p->arena_g, p->arena_l, p->layout, &cfg, &sub);
        if (rc) return rc;
        pc.plan = sub;
        p->pieces.push_back(pc);
    }
    GB_CUDA(cudaStreamCreateWithFlags(&p->copy_stream, cudaStreamNonBlocking));
    // A Phi^-1 build waits for SMs that the previous piece's persistent solver
    // grids hold; at the highest priority it gets the first SMs they free.
    int lo_prio = 0, hi_prio = 0;
    GB_CUDA(cudaDeviceGetStreamPriorityRange(&lo_prio, &hi_prio));
    GB_CUDA(cudaStreamCreateWithPriority(&p->build_stream, cudaStreamNonBlocking, hi_prio));
    for (int j = 0; j < 2; ++j) {  // consecutive pieces overlap
        cudaStream_t st;
        GB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        p->piece_streams.push_back(st);
    }
    for (size_t j = 0; j < 3 * p->pieces.size() + 1; ++j) {
        cudaEvent_t ev;
        GB_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        p->piece_events.push_back(ev);
    }
    return GBDPCG_SUCCESS;
}

}  // namespace

extern "C" {

}  // extern "C"

namespace {

// End-to-end execution of a packed plan from host arenas; with build_pinv the
// block-Jacobi Phi^-1 is built on the device from the copied S (per piece,
// right before that piece's solve) instead of being copied.
int host_run(gbdpcg_plan_s *p, const void *h_S, const void *h_Pinv, const void *h_gamma, void *h_lambda,
             gbdpcg_result *h_results, gbdpcg_stream_t stream_, bool build_pinv) {
    if (!p || !h_lambda) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (!p->packed) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "plan was not created packed");
    if (build_pinv)
        for (auto &d : p->descs)
            if (d.n > 32) return fail(GBDPCG_ERR_UNSUPPORTED, "block-Jacobi builder needs n <= 32");
    HandleScope scope(p->h->device);
    cudaStream_t st = (cudaStream_t)stream_;
    if (!p->pieces_built) {
        int rc = build_pieces(p);
        if (rc) return rc;
    }
    if (!p->pieces.empty()) {
        const size_t np = p->pieces.size();
        cudaEvent_t start = p->piece_events[2 * np];
        GB_CUDA(cudaEventRecord(start, st));
        GB_CUDA(cudaStreamWaitEvent(p->copy_stream, start, 0));
        GB_CUDA(cudaStreamWaitEvent(p->build_stream, start, 0));
        for (auto s : p->piece_streams) GB_CUDA(cudaStreamWaitEvent(s, start, 0));
        auto h2d = [&](const void *dst, const void *src, size_t lo, size_t hi) -> cudaError_t {
            if (!src || hi <= lo) return cudaSuccess;
            return cudaMemcpyAsync(static_cast<char *>(const_cast<void *>(dst)) + lo,
                                   static_cast<const char *>(src) + lo, hi - lo, cudaMemcpyHostToDevice,
                                   p->copy_stream);
        };
        // GBDPCG_PIPE_LOG=1: when each piece's copies, Phi^-1 build and solve
        // end, on stderr (diagnostics)
        const char *log_env = getenv("GBDPCG_PIPE_LOG");
        std::vector<cudaEvent_t> tl;
        if (log_env && log_env[0] == '1') {
            tl.resize(3 * np + 1);
            for (auto &e : tl) GB_CUDA(cudaEventCreate(&e));
            GB_CUDA(cudaEventRecord(tl[3 * np], p->copy_stream));
        }
        for (size_t j = 0; j < np; ++j) {
            const auto &pc = p->pieces[j];
            GB_CUDA(h2d(p->arena_S, h_S, pc.S0, pc.S1));
            GB_CUDA(h2d(p->arena_P, h_Pinv, pc.P0, pc.P1));
            GB_CUDA(h2d(p->arena_g, h_gamma, pc.V0, pc.V1));
            if (!p->cfg.zero_guess) GB_CUDA(h2d(p->arena_l, h_lambda, pc.V0, pc.V1));
            GB_CUDA(cudaEventRecord(p->piece_events[j], p->copy_stream));
            if (!tl.empty()) GB_CUDA(cudaEventRecord(tl[j], p->copy_stream));
        }
        for (size_t j = 0; j < np; ++j) {
            const auto &pc = p->pieces[j];
            cudaStream_t cs = p->piece_streams[j % p->piece_streams.size()];
            int rc;
            if (build_pinv) {
                GB_CUDA(cudaStreamWaitEvent(p->build_stream, p->piece_events[j], 0));
                if ((rc = gbdpcg_plan_build_block_jacobi(pc.plan, p->build_stream))) return rc;
                GB_CUDA(cudaEventRecord(p->piece_events[2 * np + 1 + j], p->build_stream));
                GB_CUDA(cudaStreamWaitEvent(cs, p->piece_events[2 * np + 1 + j], 0));
            } else {
                GB_CUDA(cudaStreamWaitEvent(cs, p->piece_events[j], 0));
            }
            if (!tl.empty()) GB_CUDA(cudaEventRecord(tl[np + j], cs));
            rc = gbdpcg_plan_execute(pc.plan, cs);
            if (rc) return rc;
            if (!tl.empty()) GB_CUDA(cudaEventRecord(tl[2 * np + j], cs));
            if (pc.V1 > pc.V0)
                GB_CUDA(cudaMemcpyAsync(static_cast<char *>(h_lambda) + pc.V0,
                                        static_cast<char *>(p->arena_l) + pc.V0, pc.V1 - pc.V0,
                                        cudaMemcpyDeviceToHost, cs));
            GB_CUDA(cudaMemcpyAsync(p->d_results.as<SysResult>() + pc.first, pc.plan->d_results.p,
                                    sizeof(SysResult) * pc.count, cudaMemcpyDeviceToDevice, cs));
            GB_CUDA(cudaEventRecord(p->piece_events[np + j], cs));
        }
        for (size_t j = 0; j < np; ++j) GB_CUDA(cudaStreamWaitEvent(st, p->piece_events[np + j], 0));
        if (!tl.empty()) {
            GB_CUDA(cudaStreamSynchronize(st));
            for (size_t j = 0; j < np; ++j) {
                float t[3];
                for (int q = 0; q < 3; ++q) GB_CUDA(cudaEventElapsedTime(&t[q], tl[3 * np], tl[q * np + j]));
                fprintf(stderr, "gbdpcg pipe: piece %zu systems %u copied %.3f ms built %.3f ms solved %.3f ms\n", j,
                        p->pieces[j].count, t[0], t[1], t[2]);
            }
            for (auto e : tl) cudaEventDestroy(e);
        }
        if (h_results) return gbdpcg_plan_results(p, h_results, stream_);
        GB_CUDA(cudaStreamSynchronize(st));
        return GBDPCG_SUCCESS;
    }
    if (h_S) GB_CUDA(cudaMemcpyAsync(const_cast<void *>(p->arena_S), h_S, p->bytes_S,
                                     cudaMemcpyHostToDevice, st));
    if (h_Pinv) GB_CUDA(cudaMemcpyAsync(const_cast<void *>(p->arena_P), h_Pinv, p->bytes_P,
                                        cudaMemcpyHostToDevice, st));
    if (h_gamma) GB_CUDA(cudaMemcpyAsync(const_cast<void *>(p->arena_g), h_gamma, p->bytes_vec,
                                         cudaMemcpyHostToDevice, st));
    if (!p->cfg.zero_guess)
        GB_CUDA(cudaMemcpyAsync(p->arena_l, h_lambda, p->bytes_vec, cudaMemcpyHostToDevice, st));
    int rc;
    if (build_pinv && (rc = gbdpcg_plan_build_block_jacobi(p, stream_))) return rc;
    rc = gbdpcg_plan_execute(p, stream_);
    if (rc) return rc;
    GB_CUDA(cudaMemcpyAsync(h_lambda, p->arena_l, p->bytes_vec, cudaMemcpyDeviceToHost, st));
    if (h_results) return gbdpcg_plan_results(p, h_results, stream_);
    GB_CUDA(cudaStreamSynchronize(st));
    return GBDPCG_SUCCESS;
}

}  // namespace

extern "C" {

int gbdpcg_plan_execute_host(gbdpcg_plan_t p, const void *h_S, const void *h_Pinv,
                             const void *h_gamma, void *h_lambda, gbdpcg_result *h_results,
                             gbdpcg_stream_t stream) {
    return host_run(p, h_S, h_Pinv, h_gamma, h_lambda, h_results, stream, false);
}

int gbdpcg_plan_solve_host(gbdpcg_plan_t p, const void *h_S, const void *h_gamma, void *h_lambda,
                           gbdpcg_result *h_results, gbdpcg_stream_t stream) {
    if (!h_S || !h_gamma) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    return host_run(p, h_S, nullptr, h_gamma, h_lambda, h_results, stream, true);
}

int gbdpcg_plan_build_block_jacobi(gbdpcg_plan_t p, gbdpcg_stream_t stream) {
    if (!p) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "plan is NULL");
    for (auto &d : p->descs)
        if (d.n > 32) return fail(GBDPCG_ERR_UNSUPPORTED, "block-Jacobi builder needs n <= 32");
    HandleScope scope(p->h->device);
    GB_CUDA(launch_block_jacobi(p->refine ? 2 : (p->f64 ? 1 : 0), p->d_descs.as<SysDesc>(), p->d_prefix.as<uint64_t>(),
                                p->count, p->total_knots, p->layout == GBDPCG_PINV_CBTD,
                                (cudaStream_t)stream));
    return GBDPCG_SUCCESS;
}

int gbdpcg_plan_results(gbdpcg_plan_t p, gbdpcg_result *results, gbdpcg_stream_t stream) {
    if (!p || !results) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    HandleScope scope(p->h->device);
    std::vector<SysResult> r(p->nresults);
    GB_CUDA(cudaMemcpyAsync(r.data(), p->d_results.p, sizeof(SysResult) * p->nresults,
                            cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    GB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    for (uint32_t i = 0; i < p->nresults; ++i) to_public(r[i], &results[i]);
    return GBDPCG_SUCCESS;
}

int gbdpcg_plan_launch_count(gbdpcg_plan_t p, uint32_t *launches) {
    if (!p || !launches) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    *launches = (uint32_t)(p->classes.size() + p->plain_items.size());
    return GBDPCG_SUCCESS;
}

int gbdpcg_plan_launch_info(gbdpcg_plan_t p, uint32_t i, uint32_t *cluster, uint32_t *threads,
                            uint32_t *kmax, uint32_t *systems, uint32_t *ctas) {
    if (!p) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (i < p->classes.size()) {
        const PlanClass &pc = p->classes[i];
        if (cluster) *cluster = pc.sh.C;
        if (threads) *threads = pc.sh.threads;
        if (kmax) *kmax = pc.kmax;
        if (systems) *systems = (uint32_t)pc.items.size();
        if (ctas) *ctas = pc.grid_clusters * pc.sh.C;
        return GBDPCG_SUCCESS;
    }
    i -= (uint32_t)p->classes.size();
    if (i >= p->plain_items.size()) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "launch index");
    const SysDesc &d = p->descs[p->plain_items[i]];
    if (cluster) *cluster = 0;
    if (threads) *threads = 64;
    if (kmax) *kmax = 1;
    if (systems) *systems = 1;
    if (ctas) *ctas = d.N;
    return GBDPCG_SUCCESS;
}

int gbdpcg_plan_launch_kernel(gbdpcg_plan_t p, uint32_t i, uint32_t *storage, uint32_t *rows_per_thread,
                              uint32_t *algorithm) {
    if (!p) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (i < p->classes.size()) {
        const KernelVariant &v = p->classes[i].sh.vi->v;
        if (storage) *storage = (uint32_t)v.st;
        if (rows_per_thread) *rows_per_thread = (uint32_t)v.rpt;
        if (algorithm)
            *algorithm = v.alg == 1 ? GBDPCG_ALGO_SINGLE_REDUCTION
                         : v.alg == 3 ? GBDPCG_ALGO_RECURRENCE
                         : v.alg == 0 ? GBDPCG_ALGO_CLUSTER
                                      : 0u;
        return GBDPCG_SUCCESS;
    }
    if (i - p->classes.size() >= p->plain_items.size()) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "launch index");
    if (storage) *storage = 2;
    if (rows_per_thread) *rows_per_thread = 1;
    if (algorithm) *algorithm = GBDPCG_ALGO_PLAIN;
    return GBDPCG_SUCCESS;
}

int gbdpcg_plan_timeline(gbdpcg_plan_t p, int enable) {
    if (!p) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (enable != 0 && enable != 1) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "enable must be 0 or 1");
    HandleScope scope(p->h->device);
    if ((bool)enable == p->timeline) return GBDPCG_SUCCESS;
    p->timeline = enable != 0;
    if (p->timeline) {
        int rc = timeline_buffers(p);
        if (rc) {
            p->timeline = false;
            return rc;
        }
    }
    // the launches carry the timeline pointers: capture them again
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    if (p->graph) cudaGraphDestroy(p->graph);
    p->gexec = nullptr;
    p->graph = nullptr;
    return GBDPCG_SUCCESS;
}

int gbdpcg_plan_timeline_read(gbdpcg_plan_t p, gbdpcg_stamp *stamps, uint32_t capacity, uint32_t *count,
                              uint32_t *cta_sm, uint32_t sm_capacity, uint32_t *sm_count,
                              gbdpcg_stream_t stream) {
    static_assert(sizeof(gbdpcg_stamp) == sizeof(StampRec), "gbdpcg_stamp mirrors StampRec");
    if (!p || !count || !sm_count) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    if (!p->timeline) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "the plan's timeline is off");
    HandleScope scope(p->h->device);
    size_t items = 0;
    for (const auto &pc : p->classes) items += pc.items.size();
    const uint32_t ctas = p->cta_off.empty() ? 0 : p->cta_off.back();
    *count = (uint32_t)items;
    *sm_count = ctas;
    GB_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    if (stamps && capacity)
        GB_CUDA(cudaMemcpy(stamps, p->d_stamps.p, sizeof(StampRec) * std::min<size_t>(capacity, items),
                           cudaMemcpyDeviceToHost));
    if (cta_sm && sm_capacity && ctas)
        GB_CUDA(cudaMemcpy(cta_sm, p->d_ctasm.p, sizeof(uint32_t) * std::min<uint32_t>(sm_capacity, ctas),
                           cudaMemcpyDeviceToHost));
    return GBDPCG_SUCCESS;
}

int gbdpcg_plan_destroy(gbdpcg_plan_t p) {
    if (!p) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "plan is NULL");
    HandleScope scope(p->h->device);
    delete p;
    return GBDPCG_SUCCESS;
}

}  // extern "C"

// ------------------------------------------------------------------ autotuner
namespace {

struct Candidate {
    Shape sh;
    uint32_t kmax = 0, grid = 0;
};

// Launch shapes that hold every system of `items` with the variant family of
// `base` (precision, NP, Phi^-1 layout), honouring the config's storage,
// cluster-size and CTA-size requests.
std::vector<Candidate> tune_candidates(gbdpcg_plan_s *p, const PlanClass &base,
                                       const std::vector<uint32_t> &items, uint32_t flags) {
    std::vector<Candidate> out;
    Registry *reg = p->h->reg;
    const KernelVariant &bv = base.sh.vi->v;
    std::vector<int> algs = {bv.alg};
    if ((flags & GBDPCG_TUNE_RECURRENCE) && p->cfg.algorithm == GBDPCG_ALGO_AUTO && bv.alg == 0)
        algs.push_back(3);
    if ((flags & GBDPCG_TUNE_SINGLE_REDUCTION) && p->cfg.algorithm == GBDPCG_ALGO_AUTO && bv.alg == 0 && !bv.ptri)
        algs.push_back(1);
    const int want_st = p->cfg.storage == GBDPCG_STORAGE_REGISTERS ? 0
                        : p->cfg.storage == GBDPCG_STORAGE_SHARED  ? 2
                        : p->cfg.storage == GBDPCG_STORAGE_SPLIT   ? 1
                        : p->cfg.storage == GBDPCG_STORAGE_HYBRID  ? 3
                        : p->cfg.storage == GBDPCG_STORAGE_TMEM    ? 4
                        : p->cfg.storage == GBDPCG_STORAGE_STREAM  ? 5
                                                                   : -1;
    static const uint32_t kC[] = {1, 2, 3, 4, 5, 6, 7, 8, 16};
    // what the plan's systems need of a kernel: the single-reduction kernel has
    // no adjoint epilogue, the streamed one no forward + adjoint pair (a kernel
    // that rejects a system finishes at once and would look fastest)
    const bool adjoint = (p->descs[items[0]].flags & SYS_ADJOINT) != 0;
    for (auto &vi : reg->list) {
        const KernelVariant &v = vi.v;
        if (v.f64 != bv.f64 || v.acc != bv.acc || v.np != bv.np || v.ptri != bv.ptri) continue;
        if (std::find(algs.begin(), algs.end(), v.alg) == algs.end()) continue;
        if ((v.alg == 1 && (adjoint || p->fused)) || (streamed(v.st) && p->fused)) continue;
        if (v.fa != (int)p->fused) continue;  // pairs run on the variants built for them
        if (want_st >= 0 && v.st != want_st) continue;
        bool rows_ok = true;
        for (uint32_t i : items) rows_ok &= p->descs[i].n % v.rpt == 0;
        if (!rows_ok) continue;
        uint32_t cap = std::min<uint32_t>((uint32_t)vi.max_threads,
                                          p->cfg.max_threads ? p->cfg.max_threads : 1024u);
        for (uint32_t C : kC) {
            if (p->cfg.cluster_size && C != p->cfg.cluster_size) continue;
            uint32_t kmax = 0, thr = 0;
            bool ok = true;
            for (uint32_t i : items) {
                const uint32_t n = p->descs[i].n, N = p->descs[i].N;
                const uint32_t K = (N + C - 1) / C;
                ok &= N > (C - 1) * K;  // every CTA of the cluster owns a knot
                kmax = std::max(kmax, K);
                thr = std::max(thr, (K * n + v.rpt - 1) / v.rpt);
            }
            uint32_t threads = (thr + 31) / 32 * 32;
            if (streamed(v.st)) threads = std::min(threads, cap / 32 * 32);  // row groups beyond the cap
            if (!ok || threads > cap) continue;
            if (v.smem_bytes(kmax, C, threads / 32) > (size_t)reg->max_smem_optin) continue;
            Candidate cd;
            cd.sh.vi = &vi;
            cd.sh.C = C;
            cd.sh.K = kmax;
            cd.sh.threads = threads;
            cd.kmax = kmax;
            int active = 0;
            if (max_active_clusters(cd.sh, v.smem_bytes(kmax, C, threads / 32), &active) != GBDPCG_SUCCESS) {
                cudaGetLastError();
                continue;
            }
            if (active <= 0) continue;
            cd.grid = std::min<uint32_t>((uint32_t)items.size(), (uint32_t)active);
            out.push_back(cd);
        }
    }
    return out;
}

// The whole-plan pass of the autotuner (GBDPCG_TUNE_WHOLE_PLAN).  Each class
// was tuned alone, with the whole GPU to itself; in the plan the classes run
// side by side on several streams, where what counts is how many SM-seconds a
// class takes rather than how soon it finishes alone (a shape that finishes
// first by spreading thin clusters over every SM can lose to one that packs
// its systems densely).  So the plan is timed as it will run, every class
// launched on the plan's streams with its systems solving from zero into
// scratch, and each class in turn (the longest alone first) tries its other
// shapes that came within 30% of its best alone; a change is kept when the
// whole plan gets faster by more than 1%.  The plan's own lambda and results
// are not written.
int tune_whole_plan(gbdpcg_plan_s *p, const std::vector<std::vector<std::pair<float, Candidate>>> &timed,
                    uint32_t reps, cudaStream_t st, cudaEvent_t e0, cudaEvent_t e1, bool log) {
    const size_t sv = (p->f64 || p->refine) ? 8 : 4;
    size_t need = 0;
    for (const auto &d : p->descs) need += round_up((size_t)d.n * d.N * sv, 256);
    DevBuf scratch, d_wd, d_ord, d_q, d_res;
    int rc;
    if ((rc = scratch.ensure(std::max<size_t>(need, 256)))) return rc;
    if ((rc = d_wd.ensure(sizeof(SysDesc) * p->count))) return rc;
    if ((rc = d_ord.ensure(sizeof(uint32_t) * p->count))) return rc;
    if ((rc = d_q.ensure(sizeof(uint32_t) * p->classes.size()))) return rc;
    if ((rc = d_res.ensure(sizeof(SysResult) * p->nresults))) return rc;
    std::vector<SysDesc> wd = p->descs;
    size_t off = 0;
    for (auto &d : wd) {
        d.lambda = scratch.as<char>() + off;
        d.lambda0 = nullptr;
        d.flags |= SYS_LAMBDA0_ZERO;
        off += round_up((size_t)d.n * d.N * sv, 256);
    }
    GB_CUDA(cudaMemcpyAsync(d_wd.p, wd.data(), sizeof(SysDesc) * p->count, cudaMemcpyHostToDevice, st));
    const uint32_t ns = (uint32_t)p->streams.size();
    const uint32_t treps = std::max<uint32_t>(reps, 4);  // the fastest of several runs: steps differ by ~1%
    auto time_plan = [&](std::vector<PlanClass> cls, float *ms) -> int {
        std::vector<uint32_t> order;
        int lrc = layout_classes(p->descs, cls, order);
        if (lrc) return lrc;
        GB_CUDA(cudaMemcpyAsync(d_ord.p, order.data(), sizeof(uint32_t) * order.size(), cudaMemcpyHostToDevice,
                                st));
        const uint32_t nc = (uint32_t)cls.size();
        float best = 1e30f;
        for (uint32_t r = 0; r <= treps; ++r) {
            GB_CUDA(cudaMemsetAsync(d_q.p, 0, sizeof(uint32_t) * nc, st));
            GB_CUDA(cudaEventRecord(e0, st));
            GB_CUDA(cudaEventRecord(p->events[0], st));
            for (uint32_t c = 0; c < nc; ++c) {
                cudaStream_t s = p->streams[c % ns];
                if (c < ns) GB_CUDA(cudaStreamWaitEvent(s, p->events[0], 0));
                const PlanClass &pc = cls[c];
                LaunchParams lp;
                memset(&lp, 0, sizeof(lp));
                lp.descs = d_wd.as<SysDesc>();
                lp.order = d_ord.as<uint32_t>() + pc.order_off;
                lp.count = (uint32_t)pc.items.size();
                lp.kmax = pc.kmax;
                lp.queue = d_q.as<uint32_t>() + c;
                lp.results = d_res.as<SysResult>();
                lp.launch_id = c;
                if ((lrc = launch_cluster(pc.sh, lp, pc.grid_clusters, s))) return lrc;
            }
            for (uint32_t s = 0; s < std::min(ns, nc); ++s) {
                GB_CUDA(cudaEventRecord(p->events[1 + s], p->streams[s]));
                GB_CUDA(cudaStreamWaitEvent(st, p->events[1 + s], 0));
            }
            GB_CUDA(cudaEventRecord(e1, st));
            GB_CUDA(cudaEventSynchronize(e1));
            float t = 0;
            GB_CUDA(cudaEventElapsedTime(&t, e0, e1));
            if (r > 0) best = std::min(best, t);
        }
        *ms = best;
        return GBDPCG_SUCCESS;
    };
    std::vector<PlanClass> cur = p->classes;
    float t_best = 0;
    if ((rc = time_plan(cur, &t_best))) return rc;
    if (log) fprintf(stderr, "gbdpcg tune: whole plan %.4f ms (classes tuned alone)\n", t_best);
    // the longest classes alone first
    std::vector<size_t> idx(cur.size());
    for (size_t i = 0; i < idx.size(); ++i) idx[i] = i;
    auto alone = [&](size_t i) {
        float b = 1e30f;
        for (auto &t : timed[i]) b = std::min(b, t.first);
        return b;
    };
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return alone(a) > alone(b); });
    for (size_t i : idx) {
        const float best_alone = alone(i);
        std::vector<std::pair<float, Candidate>> alts = timed[i];
        std::stable_sort(alts.begin(), alts.end(),
                         [](const std::pair<float, Candidate> &a, const std::pair<float, Candidate> &b) {
                             return a.first < b.first;
                         });
        int tried = 0;
        for (const auto &a : alts) {
            if (a.first > 1.3f * best_alone || tried >= 4) break;
            const Candidate &cd = a.second;
            if (cd.sh.vi == cur[i].sh.vi && cd.sh.C == cur[i].sh.C && cd.sh.threads == cur[i].sh.threads) continue;
            ++tried;
            std::vector<PlanClass> trial = cur;
            trial[i].sh = cd.sh;
            trial[i].kmax = cd.kmax;
            float t = 0;
            if (time_plan(trial, &t) != GBDPCG_SUCCESS) {
                cudaGetLastError();
                GB_CUDA(cudaStreamSynchronize(st));
                continue;
            }
            if (log) {
                const KernelVariant &v = cd.sh.vi->v;
                fprintf(stderr, "gbdpcg tune: whole plan %.4f ms with class %zu (%zu systems) at st=%d rpt=%d alg=%d C=%u threads=%u%s\n",
                        t, i, cur[i].items.size(), v.st, v.rpt, v.alg, cd.sh.C, cd.sh.threads, t < 0.99f * t_best ? " (kept)" : "");
            }
            if (t < 0.99f * t_best) {
                t_best = t;
                cur[i] = trial[i];
            }
        }
    }
    GB_CUDA(cudaStreamSynchronize(st));
    p->classes = cur;
    return GBDPCG_SUCCESS;
}

}  // namespace

extern "C" {

int gbdpcg_plan_autotune(gbdpcg_plan_t p, uint32_t flags, uint32_t reps, gbdpcg_stream_t stream_) {
    if (!p) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (flags & ~(uint32_t)(GBDPCG_TUNE_RECURRENCE | GBDPCG_TUNE_SINGLE_REDUCTION | GBDPCG_TUNE_WHOLE_PLAN))
        return fail(GBDPCG_ERR_INVALID_ARGUMENT, "unknown tune flag");
    if (p->classes.empty()) return GBDPCG_SUCCESS;
    HandleScope scope(p->h->device);
    cudaStream_t st = (cudaStream_t)stream_;
    if (reps == 0) reps = 2;
    const bool adjoint = (p->descs[0].flags & (SYS_ADJOINT | SYS_FWD_ADJ)) != 0;
    const bool fused = p->fused;  // also a mu output per system
    const size_t sv = (p->f64 || p->refine) ? 8 : 4;  // lambda element (refinement: double)
    const size_t sS = p->f64 ? 8 : 4;                 // dS element (adjoint: the plan's type)
    // scratch for the largest class: lambda (and dS) of each of its systems
    size_t need = 0;
    for (auto &pc : p->classes) {
        size_t b = 0;
        for (uint32_t i : pc.items) {
            const size_t n = p->descs[i].n, N = p->descs[i].N;
            b += round_up(n * N * sv, 256) * (fused ? 2 : 1) + (adjoint ? round_up(3 * n * n * N * sS, 256) : 0);
        }
        need = std::max(need, b);
    }
    DevBuf scratch, d_td, d_ord, d_q, d_res;
    int rc;
    if ((rc = scratch.ensure(std::max<size_t>(need, 256)))) return rc;
    if ((rc = d_td.ensure(sizeof(SysDesc) * p->count))) return rc;
    if ((rc = d_ord.ensure(sizeof(uint32_t) * p->count))) return rc;
    if ((rc = d_q.ensure(sizeof(uint32_t)))) return rc;
    if ((rc = d_res.ensure(sizeof(SysResult) * p->nresults))) return rc;
    cudaEvent_t e0, e1;
    GB_CUDA(cudaEventCreate(&e0));
    cudaError_t ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        cudaEventDestroy(e0);
        GB_CUDA(ce);
    }
    struct Events {
        cudaEvent_t a, b;
        ~Events() {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
        }
    } ev{e0, e1};

    std::vector<SysDesc> td = p->descs;
    std::vector<std::pair<TuneKey, TuneChoice>> learned;
    // GBDPCG_TUNE_LOG=1: one line per timed shape on stderr (diagnostics)
    const char *log_env = getenv("GBDPCG_TUNE_LOG");
    const bool log = log_env && log_env[0] == '1';
    auto log_shape = [&](const PlanClass &pc, const Shape &sh, uint32_t grid, float ms, const char *tag) {
        if (!log) return;
        const KernelVariant &v = sh.vi->v;
        uint32_t nmin = 1u << 30, nmax = 0, Nmin = 1u << 30, Nmax = 0;
        for (uint32_t i : pc.items) {
            nmin = std::min(nmin, p->descs[i].n);
            nmax = std::max(nmax, p->descs[i].n);
            Nmin = std::min(Nmin, p->descs[i].N);
            Nmax = std::max(Nmax, p->descs[i].N);
        }
        fprintf(stderr, "gbdpcg tune: systems=%zu n=%u-%u N=%u-%u | np=%d st=%d rpt=%d alg=%d acc=%d C=%u threads=%u grid=%u | %.4f ms%s\n",
                pc.items.size(), nmin, nmax, Nmin, Nmax, v.np, v.st, v.rpt, v.alg, v.acc, sh.C, sh.threads, grid, ms, tag);
    };
    // every timed shape of each class, for the whole-plan pass
    std::vector<std::vector<std::pair<float, Candidate>>> timed(p->classes.size());
    for (size_t ci = 0; ci < p->classes.size(); ++ci) {
        PlanClass &pc = p->classes[ci];
        // this class's systems solve from zero into the scratch buffers
        size_t off = 0;
        char *base = scratch.as<char>();
        for (uint32_t i : pc.items) {
            SysDesc &d = td[i];
            const size_t n = d.n, N = d.N;
            d.lambda = base + off;
            d.lambda0 = nullptr;
            d.flags |= SYS_LAMBDA0_ZERO;
            off += round_up(n * N * sv, 256);
            if (adjoint) {
                d.dS = base + off;
                off += round_up(3 * n * n * N * sS, 256);
            }
            if (fused) {
                d.lam_fwd = d.lambda;
                d.mu = base + off;
                off += round_up(n * N * sv, 256);
            }
        }
        GB_CUDA(cudaMemcpyAsync(d_td.p, td.data(), sizeof(SysDesc) * p->count, cudaMemcpyHostToDevice, st));
        GB_CUDA(cudaMemcpyAsync(d_ord.p, pc.items.data(), sizeof(uint32_t) * pc.items.size(),
                                cudaMemcpyHostToDevice, st));
        auto time_shape = [&](const Shape &sh, uint32_t kmax, uint32_t grid, float *ms) -> int {
            LaunchParams lp;
            memset(&lp, 0, sizeof(lp));
            lp.descs = d_td.as<SysDesc>();
            lp.order = d_ord.as<uint32_t>();
            lp.count = (uint32_t)pc.items.size();
            lp.kmax = kmax;
            lp.queue = d_q.as<uint32_t>();
            lp.results = d_res.as<SysResult>();
            float best = 1e30f;
            for (uint32_t r = 0; r <= reps; ++r) {
                GB_CUDA(cudaMemsetAsync(d_q.p, 0, sizeof(uint32_t), st));
                GB_CUDA(cudaEventRecord(e0, st));
                int lrc = launch_cluster(sh, lp, grid, st);
                if (lrc) return lrc;
                GB_CUDA(cudaEventRecord(e1, st));
                GB_CUDA(cudaEventSynchronize(e1));
                float t = 0;
                GB_CUDA(cudaEventElapsedTime(&t, e0, e1));
                if (r > 0) best = std::min(best, t);
            }
            *ms = best;
            return GBDPCG_SUCCESS;
        };
        float best_ms = 0;
        if ((rc = time_shape(pc.sh, pc.kmax, pc.grid_clusters, &best_ms))) return rc;
        log_shape(pc, pc.sh, pc.grid_clusters, best_ms, " (planned)");
        Candidate best;
        best.sh = pc.sh;
        best.kmax = pc.kmax;
        best.grid = pc.grid_clusters;
        timed[ci].emplace_back(best_ms, best);
        for (const Candidate &cd : tune_candidates(p, pc, pc.items, flags)) {
            if (cd.sh.vi == pc.sh.vi && cd.sh.C == pc.sh.C && cd.sh.threads == pc.sh.threads) continue;
            float ms = 0;
            if (time_shape(cd.sh, cd.kmax, cd.grid, &ms) != GBDPCG_SUCCESS) {
                // a shape the launch rejects is skipped (launch errors are not
                // sticky); anything that leaves the stream failing ends tuning
                cudaGetLastError();
                GB_CUDA(cudaStreamSynchronize(st));
                continue;
            }
            log_shape(pc, cd.sh, cd.grid, ms, "");
            timed[ci].emplace_back(ms, cd);
            if (ms < best_ms * 0.98f) {
                best_ms = ms;
                best = cd;
            }
        }
        pc.sh = best.sh;
        pc.kmax = best.kmax;
        for (uint32_t i : pc.items) td[i] = p->descs[i];
    }
    GB_CUDA(cudaStreamSynchronize(st));
    if ((flags & GBDPCG_TUNE_WHOLE_PLAN) && !adjoint && !fused && p->classes.size() > 1 &&
        (rc = tune_whole_plan(p, timed, reps, st, e0, e1, log))) return rc;
    for (auto &pc : p->classes) {
        const Shape &sh = pc.sh;
        TuneChoice ch{sh.vi->v.st, sh.vi->v.rpt, sh.vi->v.alg, sh.C, sh.threads};
        for (uint32_t i : pc.items)
            learned.emplace_back(tune_key(p, fused ? 2 : (adjoint ? 1 : 0), p->descs[i].n, p->descs[i].N), ch);
    }
    {
        std::lock_guard<std::mutex> lk(p->h->tune_mu);
        for (auto &kv : learned) p->h->tune[kv.first] = kv.second;
    }
    drop_pieces(p);
    return plan_layout(p);
}

int gbdpcg_tune_export(gbdpcg_handle_t h, char *buffer, size_t capacity, size_t *length) {
    if (!h || !length || (capacity && !buffer)) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    std::string s;
    {
        std::lock_guard<std::mutex> lk(h->tune_mu);
        char line[160];
        for (auto &kv : h->tune) {
            const TuneKey &k = kv.first;
            const TuneChoice &c = kv.second;
            snprintf(line, sizeof(line), "%u %u %u %u %u %u %u %u %u : %d %d %d %u %u\n", k.f64, k.refine,
                     k.acc, k.ptri, k.adjoint, k.alg_req, k.storage_req, k.n, k.N, c.st, c.rpt, c.alg, c.C,
                     c.threads);
            s += line;
        }
    }
    *length = s.size();
    if (capacity) {
        const size_t m = std::min(capacity - 1, s.size());
        memcpy(buffer, s.data(), m);
        buffer[m] = 0;
    }
    return GBDPCG_SUCCESS;
}

int gbdpcg_tune_import(gbdpcg_handle_t h, const char *text) {
    if (!h || !text) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "NULL pointer");
    std::vector<std::pair<TuneKey, TuneChoice>> add;
    const char *p = text;
    uint32_t lineno = 0;
    while (*p) {
        const char *e = strchr(p, '\n');
        std::string line = e ? std::string(p, e - p) : std::string(p);
        p = e ? e + 1 : p + line.size();
        ++lineno;
        if (line.find_first_not_of(" \t\r") == std::string::npos) continue;
        unsigned f[9];
        int st, rpt, alg;
        unsigned C, thr;
        char colon = 0;
        if (sscanf(line.c_str(), "%u %u %u %u %u %u %u %u %u %c %d %d %d %u %u", &f[0], &f[1], &f[2], &f[3],
                   &f[4], &f[5], &f[6], &f[7], &f[8], &colon, &st, &rpt, &alg, &C, &thr) != 15 ||
            colon != ':')
            return fail(GBDPCG_ERR_INVALID_ARGUMENT, "tuning table line " + std::to_string(lineno) + " is malformed");
        for (int i = 0; i < 5; ++i)
            if (f[i] > (i == 2 ? 2u : 1u))
                return fail(GBDPCG_ERR_INVALID_ARGUMENT, "tuning table line " + std::to_string(lineno));
        if (f[5] > GBDPCG_ALGO_RECURRENCE || f[6] > GBDPCG_STORAGE_TMEM || f[7] == 0 || f[8] == 0 || C == 0 ||
            C > 16 || thr == 0 || thr > 1024 || thr % 32)
            return fail(GBDPCG_ERR_INVALID_ARGUMENT, "tuning table line " + std::to_string(lineno));
        const int np = np_for(f[7]);
        const bool f64v = f[0] && !f[1];
        if (!np || !find_variant(h->reg, f64v, (int)f[2], np, f[3] != 0, st, rpt, alg))
            return fail(GBDPCG_ERR_UNSUPPORTED, "tuning table line " + std::to_string(lineno) +
                                                    " names a kernel variant this library does not contain");
        TuneKey k;
        memset(&k, 0, sizeof(k));
        k.f64 = (uint8_t)f[0];
        k.refine = (uint8_t)f[1];
        k.acc = (uint8_t)f[2];
        k.ptri = (uint8_t)f[3];
        k.adjoint = (uint8_t)f[4];
        k.alg_req = (uint8_t)f[5];
        k.storage_req = (uint8_t)f[6];
        k.n = f[7];
        k.N = f[8];
        add.emplace_back(k, TuneChoice{st, rpt, alg, C, thr});
    }
    std::lock_guard<std::mutex> lk(h->tune_mu);
    for (auto &kv : add) h->tune[kv.first] = kv.second;
    return GBDPCG_SUCCESS;
}

int gbdpcg_tune_clear(gbdpcg_handle_t h) {
    if (!h) return fail(GBDPCG_ERR_INVALID_ARGUMENT, "handle is NULL");
    std::lock_guard<std::mutex> lk(h->tune_mu);
    h->tune.clear();
    return GBDPCG_SUCCESS;
}

}  // extern "C"
