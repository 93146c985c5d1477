"""Benchmark: batched PCG solves/s at relative residual 1e-6 on GB300.

Workload (one "step"): 4096 independent block-tridiagonal Schur-complement
systems, n drawn from {6, 12, 14, 24} (m = n/2), N uniform in [16, 128],
per-system seeds 0..4095 (a multi-GPU run of W ranks solves seeds 0..4096 W - 1,
split over the ranks by estimated cost with the library's partitioner),
gamma ~ N(0, 1), lambda0 = 0, FP32, block-Jacobi Phi^-1 (built on the GPU),
exit on the relative recursive residual ||r|| <= 1e-6 ||gamma||.  All systems
are solved by one CUDA-graph replay of the persistent cluster launches.

Printed JSON line (rank 0):
  value      solves/s with inputs resident in HBM (inputs, 1.1 GB, exceed L2)
  e2e        solves/s through gbdpcg_plan_solve_host (the batched pcg_solve:
             S and gamma in, Phi^-1 built on the GPU, lambda out) from pinned
             host buffers, host<->device copies inside the timed region
  roofline   bytes model: sizeof(T)*[(3N-2)n^2 + N n^2 + 6nN] per PCG
             iteration per system (S and Phi^-1 block rows once, vectors
             p, r, lambda read and written), summed over the iterations each
             system took, per step, divided by the step's device time;
             against the measured HBM copy bandwidth (the matrices stay on
             chip across iterations, so this streaming-equivalent rate can
             exceed it).  `compulsory` gives the once-per-solve bytes.
  cpu_baseline  the oracle's C port of the same PCG on the host cores
  plain_pcg  one system per launch with the plain (reference-scheme) kernel
  single_system  one system alone (n = 14, N = 32 and 128): us per iteration
             of each form, and the host-array solvePCG / pcg_solve calls
  single_system_n128  n = 14, N = 128, seeds 0-9, FP32 and FP64: the reference
             kernel rebuilt for sm_103a beside the plain kernel and the
             cluster solver (seed means)
  adjoint, precision  the forward + adjoint and FP32 + FP64 refinement configs
  around_solve  Schur formation (alone and with the fused Phi^-1), KKT
             back-substitution and CSR -> cbtd on one long horizon
  block_jacobi  the Phi^-1 build over the batch
  timeline   one execution's per-system timeline (staging share, us per
             iteration and idle tails per launch class, busy SMs over the
             step) and the latency floor of the dominant class and of one
             n = 14, N = 32 system; roofline.latency repeats the floors
--impl reference: times the reference's CPU path on the host cores — the
reference ships none, so the oracle's C port of its PCG (all host threads).
--only around-solve | block-jacobi | single-system | single-system-n128 | timeline |
adjoint: that section alone.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "gbd-pcg_gb300"))
sys.path.insert(0, ROOT)

METRIC = "batched solves/s @rel-res 1e-6 (4096 mixed systems)"
WORKLOAD = "mixed-batch-4096: n in {6,12,14,24}, N~U[16,128], fp32, block-Jacobi, relres 1e-6"
TOL, MAX_ITER = 1e-6, 500


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--systems", type=int, default=4096)
    ap.add_argument("--no-extras", action="store_true", help="skip the baselines and the other configurations")
    ap.add_argument("--only", default=None, choices=["around-solve", "block-jacobi", "single-system",
                                                     "single-system-n128", "timeline", "adjoint"],
                    help="time one section alone and print its JSON (profiling): the kernels either side of "
                         "the solve, the block-Jacobi build over the batch, or the n = 14, N = 128 seeds "
                         "beside the rebuilt reference kernel")
    ap.add_argument("--knots", type=int, default=65536, help="knots of the --only around-solve horizon")
    ap.add_argument("--algorithm", default="auto", choices=["auto", "standard", "recurrence", "single-reduction"])
    ap.add_argument("--storage", default="auto", choices=["auto", "registers", "shared", "split", "hybrid", "tmem"],
                    help="pin where the cluster solver keeps the matrix rows (profiling; default: the tuner's choice)")
    ap.add_argument("--cluster-size", type=int, default=0, help="pin the CTAs per system (profiling; 0: chosen)")
    ap.add_argument("--host-pieces", type=int, default=0,
                    help="pieces the end-to-end path pipelines copies and solves in (0: automatic)")
    ap.add_argument("--tune", default="shapes+recurrence+plan",
                    choices=["off", "shapes", "shapes+recurrence", "shapes+recurrence+plan", "shapes+algorithms"],
                    help="autotune the plan before timing (untimed set-up, like building the plan)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def rank_seeds(rank, count, world=1):
    """Seeds of the systems rank `rank` solves.  The job's batch is the
    world*count systems of seeds 0 .. world*count-1 (weak scaling: `count` per
    GPU); it is split over the ranks by estimated cost n^2 N with the
    library's partitioner (gbdpcg_partition), each rank solving its own part
    with no exchange of data.  One rank: seeds 0 .. count-1."""
    if world <= 1:
        return list(range(count))
    from gbdpcg import distributed as D
    from gbdpcg.workload import mixed_size
    sizes = np.array([mixed_size(s) for s in range(world * count)], np.uint32)
    part_of, _ = D.partition(sizes[:, 0], sizes[:, 1], world)
    return D.rank_items(part_of, rank).tolist()


def build_batch(rank, count, workers, world=1):
    from gbdpcg.workload import packed_batch
    return packed_batch(rank_seeds(rank, count, world), np.float32, workers=workers, pinv_layout=1)


def max_over_ranks(x, world, dev=None):
    """The largest of the ranks' values of x (each rank's own elapsed time);
    x itself on one rank."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(job_systems, steps, seconds):
    """Systems solved by all ranks per second of the slowest rank's time."""
    return job_systems * steps / seconds


def algorithmic_bytes(descs, iters, s=4):
    it = np.asarray(iters, np.float64)
    n = np.array([d[0] for d in descs], np.float64)
    N = np.array([d[1] for d in descs], np.float64)
    per_iter = s * ((3 * N - 2) * n * n + N * n * n + 6 * n * N)
    compulsory = s * (3 * n * n * N + n * n * N + 2 * n * N)
    flops = (2 * (3 * N - 2) * n * n + 2 * N * n * n + 10 * n * N)
    return float((per_iter * it).sum()), float(compulsory.sum()), float((flops * it).sum())


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.out = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        self.out.flush()
        rows = []
        with open(self.out.name) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        os.unlink(self.out.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({nm for r in rows for nm, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def relres64(S, g, lam, n, N):
    """||gamma - S lambda|| / ||gamma|| in FP64 for one cbtd system (host numpy)."""
    Sd = np.asarray(S, np.float64).reshape(N, 3 * n, n).transpose(0, 2, 1)
    x = np.asarray(lam, np.float64).reshape(N, n)
    y = np.einsum("kij,kj->ki", Sd[:, :, n:2 * n], x)
    if N > 1:
        y[1:] += np.einsum("kij,kj->ki", Sd[1:, :, 0:n], x[:-1])
        y[:-1] += np.einsum("kij,kj->ki", Sd[:-1, :, 2 * n:], x[1:])
    g = np.asarray(g, np.float64)
    return float(np.linalg.norm(g - y.reshape(-1)) / np.linalg.norm(g))


def cpu_port_baseline(Sa, Pa, ga, descs, sample, threads, passes=1):
    """The oracle's C port of the PCG on the first `sample` systems, `passes`
    times over, with `threads` host threads.  Returns (systems/s, seconds,
    threads used, iterations, status)."""
    from oracle import oracle as O
    O.lib()
    systems = []
    for (n, N, oS, oP, oV) in descs[:sample]:
        systems.append({"S": Sa[oS:oS + 3 * n * n * N], "Pinv": Pa[oP:oP + n * n * N],
                        "gamma": ga[oV:oV + n * N], "lambda": np.zeros(n * N, np.float32), "n": n, "N": N})
    t0 = time.perf_counter()
    for _ in range(passes):
        for sy in systems:  # every pass solves from lambda0 = 0, like the GPU path
            sy["lambda"][:] = 0.0
        iters, status, used = O.pcg_batch(systems, flags=O.PINV_BLOCKDIAG | O.EXIT_RELRES, nthreads=threads,
                                          max_iter=MAX_ITER, tol=TOL)
    dt = time.perf_counter() - t0
    return sample * passes / dt, dt, used, iters, status


def cpu_sample_size(rate, count, seconds=10.0):
    """(systems, passes) giving about `seconds` of host work at `rate` systems/s:
    the first systems of the batch, or the whole batch several times over."""
    want = max(64, int(rate * seconds))
    if want <= count:
        return want, 1
    return count, max(1, int(round(want / count)))


def single_system_latency(gbdpcg, h, dev):
    """us per PCG iteration of one system solved alone (n=14; N=32 and N=128;
    FP32 tol 1e-6 and FP64 tol 1e-12, reference exit test, seed 0), for the
    cluster solver (standard and recurrence forms) and the plain kernel."""
    import torch
    from gbdpcg.workload import generate
    out = []
    for N, dts in ((32, "f32"), (128, "f32"), (128, "f64")):
        n = 14
        tdt = torch.float64 if dts == "f64" else torch.float32
        npdt = np.float64 if dts == "f64" else np.float32
        sy = generate(n, N, 0)
        S = torch.from_numpy(sy.cbtd(npdt)).to(dev)
        g = torch.from_numpy(sy.gamma.astype(npdt)).to(dev)
        P = torch.empty(n * n * N, dtype=tdt, device=dev)
        h.block_jacobi(S, P, n, N, gbdpcg.PINV_BLOCKDIAG)
        Pt = torch.zeros(N, 3 * n, n, dtype=tdt, device=dev)
        Pt[:, n:2 * n, :] = P.view(N, n, n)
        Pt = Pt.view(-1)
        lam = torch.zeros(n * N, dtype=tdt, device=dev)
        tol = 1e-12 if dts == "f64" else 1e-6
        row = {"n": n, "N": N, "dtype": dts}
        for name, algo, PP, lay in (("cluster", gbdpcg.ALGO_CLUSTER, P, gbdpcg.PINV_BLOCKDIAG),
                                    ("recurrence", gbdpcg.ALGO_RECURRENCE, P, gbdpcg.PINV_BLOCKDIAG),
                                    ("plain", gbdpcg.ALGO_PLAIN, Pt, gbdpcg.PINV_CBTD)):
            cfg = gbdpcg.config(max_iter=500, exit_tol=tol, algorithm=algo, zero_guess=1)
            best = None
            for C in ((0,) if algo == gbdpcg.ALGO_PLAIN else (0, 1, 2, 4, 8, 16)):
                cfg.cluster_size = C
                try:
                    r = h.solve(S, PP, g, lam, n, N, lay, cfg)
                except gbdpcg.GbdpcgError:
                    continue
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                for _ in range(20):
                    h.solve(S, PP, g, lam, n, N, lay, cfg, sync=False)
                b.record()
                b.synchronize()
                us = 1e3 * a.elapsed_time(b) / 20
                if best is None or us < best[0]:
                    best = (us, r.iters, C)
            if best:
                row[name] = {"us_per_solve": best[0], "iters": best[1], "us_per_iteration": best[0] / best[1],
                             "cluster_size": best[2]}
        # the reference's own call, one system from pageable host arrays:
        # solvePCG (S, Pinv, gamma, lambda in; lambda out) and pcg_solve (Phi^-1
        # built on the GPU); median wall time per call, copies included
        Snp, gnp, Pnp = sy.cbtd(npdt), sy.gamma.astype(npdt), Pt.cpu().numpy()
        cfgh = gbdpcg.config(max_iter=500, exit_tol=tol)
        for name, PP in (("host_solvePCG", Pnp), ("host_pcg_solve", None)):
            lamh = np.zeros(n * N, npdt)
            gbdpcg.solve(Snp, PP, gnp, lamh, n, N, cfgh)  # warm
            ts = []
            for _ in range(30):
                lamh[:] = 0
                t0 = time.perf_counter()
                rh = gbdpcg.solve(Snp, PP, gnp, lamh, n, N, cfgh)
                ts.append(time.perf_counter() - t0)
            row[name] = {"us_per_call": 1e6 * float(np.median(ts)), "iters": int(rh.iters),
                         "path": "gbdpcg_solve from pageable numpy arrays, copies and sync included"}
        out.append(row)
    return out


def n128_seed_sweep(gbdpcg, h, dev, reps=20, seeds=range(10)):
    """The larger single system, n = 14, N = 128, seeds 0-9, FP32 to 1e-6 and
    FP64 to 1e-12 (the reference's exit test |r.z| < tol, max_iter 200):

      reference_kernel  the reference's own kernel pcg<T, 14, 128>
                        (include/pcg.cuh:54-218) rebuilt for sm_103a and
                        launched as its device-pointer solvePCG launches it
                        (include/interface.cuh:94-146: cooperative, N CTAs of
                        64 threads), cbtd Phi^-1 — a baseline, never the product
      plain             this library's plain kernel (the same scheme, runtime
                        sizes), cbtd Phi^-1
      cluster, recurrence  the cluster solver and its recurrence form, compact
                        Phi^-1, at the cluster size fastest on seed 0

    Every form: `reps` launches from the same inputs, CUDA events around each
    launch (the reference launcher's own method), mean per launch; reported as
    the mean over the seeds, with the per-seed passes."""
    import torch
    from gbdpcg.workload import generate
    from oracle import oracle as O  # the rebuilt reference kernel's launcher (baseline only)
    n, N = 14, 128
    stream = torch.cuda.current_stream()

    def per_launch(fn):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b))
        return 1e3 * float(np.mean(ts))

    out = {"n": n, "N": N, "seeds": list(seeds), "reps_per_seed": reps,
           "timing": "CUDA events around each launch, mean of the launches, then mean over seeds"}
    for dts, tdt, npdt, tol in (("f32", torch.float32, np.float32, 1e-6), ("f64", torch.float64, np.float64, 1e-12)):
        forms = {k: {"us": [], "iters": []} for k in ("reference_kernel", "plain", "cluster", "recurrence")}
        csize = {}
        for seed in seeds:
            sy = generate(n, N, seed)
            S = torch.from_numpy(sy.cbtd(npdt)).to(dev)
            g = torch.from_numpy(sy.gamma.astype(npdt)).to(dev)
            P = torch.empty(n * n * N, dtype=tdt, device=dev)
            h.block_jacobi(S, P, n, N, gbdpcg.PINV_BLOCKDIAG)
            Pt = torch.zeros(N, 3 * n, n, dtype=tdt, device=dev)
            Pt[:, n:2 * n, :] = P.view(N, n, n)
            Pt = Pt.view(-1)
            lam = torch.zeros(n * N, dtype=tdt, device=dev)
            if O.have_ref_kernel(dts, n, N):
                _, it, mie, ms = O.ref_kernel_solve(S.cpu().numpy(), Pt.cpu().numpy(), g.cpu().numpy(),
                                                    np.zeros(n * N, npdt), n, N, 200, tol, reps=reps + 1)
                forms["reference_kernel"]["us"].append(1e3 * float(np.mean(ms[1:])))
                forms["reference_kernel"]["iters"].append(it)
            for name, algo, PP, lay in (("plain", gbdpcg.ALGO_PLAIN, Pt, gbdpcg.PINV_CBTD),
                                        ("cluster", gbdpcg.ALGO_CLUSTER, P, gbdpcg.PINV_BLOCKDIAG),
                                        ("recurrence", gbdpcg.ALGO_RECURRENCE, P, gbdpcg.PINV_BLOCKDIAG)):
                cfg = gbdpcg.config(max_iter=200, exit_tol=tol, algorithm=algo, zero_guess=1)
                if name not in csize:  # cluster size: fastest on the first seed
                    best = None
                    for C in ((0,) if algo == gbdpcg.ALGO_PLAIN else (1, 2, 4, 8, 16)):
                        cfg.cluster_size = C
                        try:
                            us = per_launch(lambda: h.solve(S, PP, g, lam, n, N, lay, cfg, sync=False))
                        except gbdpcg.GbdpcgError:
                            continue
                        if best is None or us < best[0]:
                            best = (us, C)
                    csize[name] = best[1]
                cfg.cluster_size = csize[name]
                forms[name]["us"].append(per_launch(lambda: h.solve(S, PP, g, lam, n, N, lay, cfg, sync=False)))
                forms[name]["iters"].append(int(h.last_result().iters))
        row = {}
        for name, f in forms.items():
            if not f["us"]:
                row[name] = {"unavailable": "reference kernel not built"}
                continue
            us, it = float(np.mean(f["us"])), float(np.mean(f["iters"]))
            row[name] = {"us_per_solve_mean": us, "iters_mean": it, "us_per_iteration": us / it,
                         "iters_per_seed": f["iters"], "us_per_solve_per_seed": f["us"]}
            if name in csize and name != "plain":
                row[name]["cluster_size"] = csize[name]
        if "us_per_solve_mean" in row["reference_kernel"]:
            ref = row["reference_kernel"]["us_per_solve_mean"]
            row["speedup_vs_reference_kernel"] = {k: ref / row[k]["us_per_solve_mean"]
                                                  for k in ("plain", "cluster", "recurrence")}
        out[dts] = row
    return out


def timeline_summary(stamps, cta_sm, launches, sm_count):
    """Reads one execution's timeline (gbdpcg_plan_timeline_read): per launch
    class, the share of each system's time spent staging its rows, the us per
    PCG iteration, the mean time between two systems of one cluster (taking
    the next from the queue), and how long the class's clusters sat idle
    after the class's last system started; over the step, the fraction of SM-time with
    no CTA of the solver resident and busy, and the step's tail (from the last
    moment 90% of the SMs were busy to the end)."""
    ok = stamps["iters"] > 0
    st = stamps[ok]
    t0 = int(st["t_pop"].min())
    t_end = int(st["t_done"].max())
    T = t_end - t0
    cta_base = np.concatenate([[0], np.cumsum([l["ctas"] for l in launches if l["cluster"] > 0])])
    classes = []
    all_gaps = []
    for c, l in enumerate(launches):
        if l["cluster"] == 0:
            continue
        m = st["launch"] == c
        if not m.any():
            continue
        s = st[m]
        busy = (s["t_done"] - s["t_pop"]).astype(np.float64)
        stage = (s["t_staged"] - s["t_pop"]).astype(np.float64)
        per_iter = (s["t_solved"] - s["t_staged"]).astype(np.float64) / s["iters"]
        c_end = int(s["t_done"].max())
        last_done = {}
        for rec in s:
            last_done[int(rec["cluster"])] = max(last_done.get(int(rec["cluster"]), 0), int(rec["t_done"]))
        # between two systems of one cluster: from the first's results written
        # to the second taken from the queue (the pop and its cluster barrier)
        gaps = []
        for cl in np.unique(s["cluster"]):
            r = np.sort(s[s["cluster"] == cl], order="t_pop")
            gaps.extend((r["t_pop"][1:].astype(np.int64) - r["t_done"][:-1].astype(np.int64)).tolist())
        all_gaps.extend(gaps)
        idle_cta_ns = sum(c_end - v for v in last_done.values()) * l["cluster"]
        classes.append({"launch": c, "cluster": l["cluster"], "threads": l["threads"], "storage": l["storage"],
                        "rows_per_thread": l["rows_per_thread"], "algorithm": l["algorithm"],
                        "systems": int(m.sum()), "cta_busy_ms": float(busy.sum() * l["cluster"] / 1e6),
                        "staging_share": float(stage.sum() / busy.sum()),
                        "us_per_iteration_median": float(np.median(per_iter) / 1e3),
                        "start_ms": (int(s["t_pop"].min()) - t0) / 1e6, "end_ms": (c_end - t0) / 1e6,
                        "tail_idle_cta_ms": idle_cta_ns / 1e6,
                        "between_systems_us_mean": float(np.mean(gaps) / 1e3) if gaps else 0.0})
    # busy SMs over the step: an SM is busy while a CTA of a cluster is solving a system
    ev = []
    for rec in st:
        base = int(cta_base[rec["launch"]]) + int(rec["cluster"]) * launches[rec["launch"]]["cluster"]
        sms = set(int(x) for x in cta_sm[base:base + launches[rec["launch"]]["cluster"]])
        ev.append((int(rec["t_pop"]), 1, sms))
        ev.append((int(rec["t_done"]), -1, sms))
    ev.sort(key=lambda e: (e[0], e[1]))
    act = np.zeros(max(sm_count, int(cta_sm.max()) + 1 if cta_sm.size else sm_count), np.int64)
    busy_sm_ns, nbusy, last_t = 0.0, 0, t0
    last_full = t0
    for t, d, sms in ev:
        busy_sm_ns += nbusy * (t - last_t)
        if nbusy >= 0.9 * sm_count:
            last_full = t
        last_t = t
        for x in sms:
            if d > 0:
                act[x] += 1
                if act[x] == 1:
                    nbusy += 1
            else:
                act[x] -= 1
                if act[x] == 0:
                    nbusy -= 1
    classes.sort(key=lambda r: -r["cta_busy_ms"])
    return {"step_ms": T / 1e6, "sm_busy_frac": busy_sm_ns / (sm_count * T), "tail_ms": (t_end - last_full) / 1e6,
            "tail_share": (t_end - last_full) / T,
            "staging_share": float(((st["t_staged"] - st["t_pop"]).sum()) / (st["t_done"] - st["t_pop"]).sum()),
            "between_systems_share": float(sum(all_gaps) / (st["t_done"] - st["t_pop"]).sum()),
            "classes": classes}


def latency_floor(gbdpcg, cls, grid_clusters, dev_index=0, reps=100000):
    """The floor that the synchronisation primitives put under one PCG
    iteration of a launch shape: two cluster-wide reductions (1 and 2 values,
    in the form the kernel uses at that cluster size) and two CTA barriers
    (standard form) or one (recurrence form), each measured by
    gbdpcg_probe_primitives on the shape (cluster size, CTA size) with all the
    shape's clusters running at once; frac = floor / achieved."""
    C, thr = cls["cluster"], cls["threads"]
    under_load = gbdpcg.probe_primitives(dev_index, C, thr, grid_clusters, reps)
    alone = gbdpcg.probe_primitives(dev_index, C, thr, 1, reps)
    rec = cls["algorithm"] == gbdpcg.ALGO_RECURRENCE
    barriers = 1 if rec else 2
    # the cluster kernels reduce with transaction-counted stores for C >= 2,
    # with the CTA-barrier form for C = 1
    red = under_load["allreduce_tx_ns"] if C > 1 else under_load["allreduce_ns"]
    floor = red[0] + red[1] + barriers * under_load["syncthreads_ns"]
    ach = cls["us_per_iteration_median"] * 1e3
    return {"shape": {"cluster": C, "threads": thr, "storage": cls["storage"], "algorithm": cls["algorithm"],
                      "clusters_at_once": grid_clusters},
            "model": f"reduction(1 value) + reduction(2 values) + {barriers} x __syncthreads per iteration "
                     f"({'transaction-counted' if C > 1 else 'CTA-barrier'} reductions)",
            "floor_us_per_iter": floor / 1e3, "achieved_us_per_iter": ach / 1e3, "frac": floor / ach,
            "primitives_under_load_ns": under_load, "primitives_alone_ns": alone}


def timeline_and_floor(gbdpcg, h, plan, launches, dev, sm_count):
    """Timeline of one execution of the benchmark plan, and the latency floor
    of its dominant class and of one n = 14, N = 32 system (its own plan)."""
    import torch
    from gbdpcg.workload import generate
    plan.timeline(True)
    plan.execute()
    plan.execute()
    stamps, sms = plan.timeline_read()
    plan.timeline(False)
    summ = timeline_summary(stamps, sms, launches, sm_count)
    dom = summ["classes"][0]
    out = {"timeline": summ,
           "latency": {"dominant_class": latency_floor(gbdpcg, dom, launches[dom["launch"]]["ctas"] // dom["cluster"])}}
    # one n = 14, N = 32 system alone (FP32, tol 1e-6, reference exit test, seed 0)
    n, N = 14, 32
    sy = generate(n, N, 0)
    S = torch.from_numpy(sy.cbtd(np.float32)).to(dev)
    g = torch.from_numpy(sy.gamma.astype(np.float32)).to(dev)
    P = torch.empty(n * n * N, device=dev)
    h.block_jacobi(S, P, n, N, gbdpcg.PINV_BLOCKDIAG)
    lam = torch.zeros(n * N, device=dev)
    for algo, key in ((gbdpcg.ALGO_CLUSTER, "n14_N32_standard"), (gbdpcg.ALGO_RECURRENCE, "n14_N32_recurrence")):
        cfg = gbdpcg.config(max_iter=200, exit_tol=1e-6, algorithm=algo, zero_guess=1, cluster_size=1)
        p1 = gbdpcg.Plan(h, [{"S": S, "Pinv": P, "gamma": g, "lambda": lam, "n": n, "N": N}],
                         gbdpcg.PINV_BLOCKDIAG, cfg)
        l1 = p1.launches()
        p1.timeline(True)
        times = []
        for _ in range(5):
            p1.execute()
            s1, m1 = p1.timeline_read()
            times.append(s1)
        s1 = min(times, key=lambda x: int(x["t_solved"][0] - x["t_staged"][0]))
        cls = dict(l1[0], launch=0, us_per_iteration_median=float(s1["t_solved"][0] - s1["t_staged"][0]) / 1e3
                   / int(s1["iters"][0]))
        out["latency"][key] = latency_floor(gbdpcg, cls, 1)
        p1.close()
    return out


def adjoint_config(gbdpcg, h, dev, tune_flags=None, count=1024, n=14, N=64):
    """Forward + adjoint cost: batch 1024, n=14, N=64, FP32, L = 1/2 ||lambda - lambda*||^2.
    With tune_flags, both plans are autotuned alike (None: neither)."""
    import torch
    from gbdpcg.workload import generate
    fwd, adj = [], []
    rng = np.random.default_rng(12345)
    for b in range(count):
        sy = generate(n, N, 100000 + b)
        S = torch.from_numpy(sy.cbtd(np.float32)).to(dev)
        g = torch.from_numpy(sy.gamma.astype(np.float32)).to(dev)
        P = torch.empty(n * n * N, device=dev)
        fwd.append({"S": S, "Pinv": P, "gamma": g, "lambda": torch.zeros(n * N, device=dev), "n": n, "N": N})
        adj.append({"star": torch.from_numpy(rng.standard_normal(n * N).astype(np.float32)).to(dev)})
    cfg = gbdpcg.config(max_iter=500, exit_tol=1e-6, exit_mode=gbdpcg.EXIT_RELRES, zero_guess=1)
    pf = gbdpcg.Plan(h, fwd, gbdpcg.PINV_BLOCKDIAG, cfg)
    pf.build_block_jacobi()
    if tune_flags is not None:
        pf.autotune(flags=tune_flags)
    pf.execute()
    torch.cuda.synchronize()
    systems = []
    for f, a in zip(fwd, adj):
        a["gl"] = f["lambda"] - a["star"]
        systems.append({"S": f["S"], "Pinv": f["Pinv"], "gamma": a["gl"], "lambda": torch.empty_like(a["gl"]),
                        "lambda_fwd": f["lambda"], "dS": torch.empty_like(f["S"]), "n": n, "N": N})
    pa = gbdpcg.Plan(h, systems, gbdpcg.PINV_BLOCKDIAG, cfg)
    if tune_flags is not None:
        pa.autotune(flags=tune_flags)

    def timeit(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    t_f = timeit(pf.execute)
    t_a = timeit(pa.execute)
    res_a = pa.results()
    # forward + adjoint in one launch per class (gbdpcg_plan_create_fwd_adj):
    # the rows are staged once for both solves
    pairs = [{"S": f["S"], "Pinv": f["Pinv"], "gamma": f["gamma"], "lambda": torch.zeros_like(f["lambda"]),
              "lambda_target": a["star"], "grad_gamma": torch.empty_like(f["lambda"]),
              "grad_S": torch.empty_like(f["S"]), "n": n, "N": N} for f, a in zip(fwd, adj)]
    pj = gbdpcg.Plan.forward_adjoint(h, pairs, gbdpcg.PINV_BLOCKDIAG, cfg)
    if tune_flags is not None:
        pj.autotune(flags=tune_flags)
    t_j = timeit(pj.execute)
    res_j = pj.results()
    out = {"systems": count, "n": n, "N": N, "forward_ms": t_f, "adjoint_ms": t_a,
           "forward_plus_adjoint_over_forward": (t_f + t_a) / t_f,
           "adjoint_all_converged": all(r.status == 0 for r in res_a),
           "fused_ms": t_j, "fused_over_forward": t_j / t_f,
           "shapes": {k: [[l["cluster"], l["threads"], l["storage"], l["rows_per_thread"], l["algorithm"],
                           l["systems"]] for l in pl.launches()] for k, pl in (("forward", pf), ("fused", pj))},
           "fused_all_converged": all(r.status == 0 for r in res_j),
           "autotuned": tune_flags is not None,
           "note": "adjoint = PCG solve of S mu = lambda - lambda* plus the dS, dgamma epilogue; fused = "
                   "forward and adjoint solves and the epilogue in one launch (gbdpcg_plan_create_fwd_adj)"}
    pf.close()
    pa.close()
    pj.close()
    return out


def precision_config(gbdpcg, h, dev, count=256, n=24, N=256, workers=8):
    """FP32 PCG + FP64 refinement vs FP64 PCG, all to relative residual 1e-10,
    on ill-conditioned systems (Q log-U[1e-2,1e4], R log-U[1e-3,1]): FP64 PCG
    as one batched plan over the whole batch, and as the plain kernel one
    system per launch (a sample, extrapolated)."""
    import torch
    from gbdpcg.workload import generate
    import multiprocessing as mp
    seeds = list(range(200000, 200000 + count))
    with mp.get_context("spawn").Pool(workers) as pool:
        syss = pool.starmap(_gen_ill, [(n, N, sd) for sd in seeds], chunksize=4)
    S64 = [torch.from_numpy(S).to(dev) for S, g in syss]
    g64 = [torch.from_numpy(g).to(dev) for S, g in syss]
    out = {"systems": count, "n": n, "N": N, "target_relres": 1e-10}
    # FP32 + FP64 refinement: one plan, dtype 2; inner dots in FP64, then in float-float
    for key, dot in (("refined", gbdpcg.DOT_FP64), ("refined_float2", gbdpcg.DOT_FLOAT2)):
        systems = [{"S": S64[i], "Pinv": torch.empty(n * n * N, dtype=torch.float32, device=dev),
                    "gamma": g64[i], "lambda": torch.zeros(n * N, dtype=torch.float64, device=dev),
                    "n": n, "N": N} for i in range(count)]
        cfg = gbdpcg.config(exit_mode=gbdpcg.EXIT_RELRES, exit_tol=1e-10, max_iter=40000, max_outer=60,
                            zero_guess=1, dot_precision=dot)
        pr = gbdpcg.Plan(h, systems, gbdpcg.PINV_BLOCKDIAG, cfg, dtype=2)
        pr.build_block_jacobi()
        pr.execute()  # warm (the graph is captured on the first execution)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        pr.execute()
        e1.record()
        e1.synchronize()
        rr = pr.results()
        out[key] = {"ms": e0.elapsed_time(e1), "converged": sum(r.status == 0 for r in rr),
                    "inner_dots": "fp64" if dot == gbdpcg.DOT_FP64 else "float-float",
                    "inner_iters_mean": float(np.mean([r.iters for r in rr])),
                    "outer_mean": float(np.mean([r.outer for r in rr])),
                    "relres_max": float(max(r.relres for r in rr))}
        lam = [s["lambda"] for s in systems]
        # true FP64 relative residual of the refined solutions, recomputed on the host
        out[key]["true_relres_fp64_max_sample"] = max(
            relres64(syss[i][0], syss[i][1], lam[i].cpu().numpy(), n, N)
            for i in range(0, count, max(1, count // 16)))
        pr.close()
    # FP64 PCG over the whole batch: one plan, FP64 rows streamed from L2/HBM
    # (no on-chip FP64 shape holds n = 24, N = 256), compact block-Jacobi Phi^-1
    systems = [{"S": S64[i], "Pinv": torch.empty(n * n * N, dtype=torch.float64, device=dev),
                "gamma": g64[i], "lambda": torch.zeros(n * N, dtype=torch.float64, device=dev),
                "n": n, "N": N} for i in range(count)]
    cfg64 = gbdpcg.config(exit_mode=gbdpcg.EXIT_RELRES, exit_tol=1e-10, max_iter=40000, zero_guess=1)
    pb = gbdpcg.Plan(h, systems, gbdpcg.PINV_BLOCKDIAG, cfg64, dtype=1)
    pb.build_block_jacobi()
    pb.execute()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    pb.execute()
    e1.record()
    e1.synchronize()
    rb = pb.results()
    out["fp64_pcg"] = {"ms": e0.elapsed_time(e1), "converged": sum(r.status == 0 for r in rb),
                       "iters_mean": float(np.mean([r.iters for r in rb])),
                       "relres_max": float(max(r.relres for r in rb)),
                       "true_relres_fp64_max_sample": max(
                           relres64(syss[i][0], syss[i][1], systems[i]["lambda"].cpu().numpy(), n, N)
                           for i in range(0, count, max(1, count // 16))),
                       "launches": [[l["cluster"], l["threads"], l["storage"], l["rows_per_thread"], l["systems"]]
                                    for l in pb.launches()],
                       "how": "one batched FP64 plan over all systems (streamed rows, compact Phi^-1)"}
    pb.close()
    # plain FP64 PCG (the reference's scheme: cbtd Phi^-1, one cooperative launch per system)
    t64, it64, conv64 = 0.0, [], 0
    nsamp = min(count, 32)
    for i in range(nsamp):
        P64 = torch.empty(3 * n * n * N, dtype=torch.float64, device=dev)
        h.block_jacobi(S64[i], P64, n, N, gbdpcg.PINV_CBTD)
        lam = torch.zeros(n * N, dtype=torch.float64, device=dev)
        cfgp = gbdpcg.config(exit_mode=gbdpcg.EXIT_RELRES, exit_tol=1e-10, max_iter=40000, zero_guess=1,
                             algorithm=gbdpcg.ALGO_PLAIN)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        r = h.solve(S64[i], P64, g64[i], lam, n, N, gbdpcg.PINV_CBTD, cfgp, sync=False)
        b.record()
        b.synchronize()
        r = h.last_result()
        t64 += a.elapsed_time(b)
        it64.append(r.iters)
        conv64 += r.status == 0
    out["fp64_plain_pcg"] = {"ms_for_batch_extrapolated": t64 / nsamp * count, "sample": nsamp,
                             "converged": conv64, "iters_mean": float(np.mean(it64)),
                             "how": "the plain kernel, one cooperative launch per system"}
    for key in ("refined", "refined_float2"):
        out["speedup_" + key + "_vs_fp64_batched"] = out["fp64_pcg"]["ms"] / out[key]["ms"]
        out["speedup_" + key + "_vs_fp64_plain"] = out["fp64_plain_pcg"]["ms_for_batch_extrapolated"] / out[key]["ms"]
    return out


def around_solve_kernels(gbdpcg, dev, hbm_gbs, n=24, N=65536, reps=5):
    """The steps either side of the solve on one long horizon (n = 24, m = 12,
    N = 65536 knots, FP32, random data): Schur-complement formation (alone and
    with the fused block-Jacobi Phi^-1), KKT back-substitution and the
    CSR -> cbtd adapter.  HBM-bound kernels: GB/s of
    their compulsory bytes (each input read once, each output written once)
    against the measured copy bandwidth."""
    import torch
    m = n // 2
    f = dict(dtype=torch.float32, device=dev)
    A = torch.randn(N * n * n, **f) / n ** 0.5
    B = torch.randn(N * n * m, **f)
    Qd = torch.rand((N + 1) * n, **f) + 1.0
    Rd = torch.rand(N * m, **f) + 0.1
    q = torch.randn((N + 1) * n, **f)
    r = torch.randn(N * m, **f)
    c = torch.randn(N * n, **f)
    S = torch.empty(3 * n * n * N, **f)
    g = torch.empty(n * N, **f)
    x = torch.empty((N + 1) * n, **f)
    u = torch.empty(N * m, **f)
    lam = torch.randn(N * n, **f)
    # CSR of a full block-tridiagonal band: row r of knot k holds columns of knots k-1..k+1
    rows = n * N
    k = torch.arange(rows, device=dev) // n
    lo = torch.clamp(k - 1, min=0) * n
    hi = torch.clamp(k + 2, max=N) * n
    cnt = (hi - lo).to(torch.int64)
    rp = torch.zeros(rows + 1, dtype=torch.int64, device=dev)
    rp[1:] = torch.cumsum(cnt, 0)
    nnz = int(rp[-1].item())
    rid = torch.repeat_interleave(torch.arange(rows, device=dev), cnt)
    ci = (lo[rid] + torch.arange(nnz, device=dev) - rp[:-1][rid]).to(torch.int32)
    rp32 = rp.to(torch.int32)
    val = torch.randn(nnz, **f)
    err = torch.zeros(1, dtype=torch.int32, device=dev)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        b.synchronize()
        return a.elapsed_time(b) / reps

    s = 4
    out = {"n": n, "m": m, "N": N, "dtype": "f32"}
    Pi = torch.empty(n * n * N, **f)
    form_bytes = s * (N * n * n + N * n * m + 2 * (N + 1) * n + N * m + N * n + 3 * n * n * N + n * N)
    rows_b = [("form_schur", lambda: gbdpcg.form_schur(A, B, Qd, Rd, q, r, c, n, m, N, S, g), form_bytes),
              ("form_schur_pinv", lambda: gbdpcg.form_schur(A, B, Qd, Rd, q, r, c, n, m, N, S, g, Pinv_out=Pi),
               form_bytes + s * n * n * N),
              ("kkt_backsub", lambda: gbdpcg.kkt_backsub(A, B, Qd, Rd, q, r, lam, n, m, N, x, u),
               s * (N * n * n + N * n * m + 2 * (N + 1) * n + 2 * N * m + N * n + (N + 1) * n)),
              ("csr_to_cbtd", lambda: gbdpcg.csr_to_cbtd(rp32, ci, val, n, N, S, err),
               4 * (rows + 1) + 4 * nnz + s * nnz + s * 3 * n * n * N)]
    for name, fn, nbytes in rows_b:
        ms = timed(fn)
        out[name] = {"ms": ms, "bytes": nbytes, "gbs": nbytes / (ms / 1e3) / 1e9,
                     "frac_of_hbm": nbytes / (ms / 1e3) / 1e9 / hbm_gbs}
    out["note"] = "csr_to_cbtd is synchronous (it reads back its error word)"
    return out


def block_jacobi_build(plan, descs, hbm_gbs, reps=5):
    """The block-Jacobi Phi^-1 build over the plan's systems (device-resident):
    S_kk read and its inverse written once per knot."""
    import torch
    plan.build_block_jacobi()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        plan.build_block_jacobi()
    b.record()
    b.synchronize()
    ms = a.elapsed_time(b) / reps
    knots = sum(N for (n, N, _, _, _) in descs)
    nbytes = sum(2 * 4 * n * n * N for (n, N, _, _, _) in descs)
    return {"ms": ms, "knots": knots, "bytes": nbytes, "gbs": nbytes / (ms / 1e3) / 1e9,
            "frac_of_hbm": nbytes / (ms / 1e3) / 1e9 / hbm_gbs,
            "note": "one warp per knot, rotating Gauss-Jordan in registers: issue-bound, not HBM-bound"}


def _gen_ill(n, N, seed):
    from gbdpcg.workload import generate
    sy = generate(n, N, seed, ill=True)
    return sy.cbtd(), sy.gamma


def run_reference(args):
    """--impl reference: the reference has no CPU implementation of its PCG; the
    oracle's C port of it runs on all host threads over the same workload."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, ROOT)
    from oracle import build_oracle
    build_oracle.build()
    from oracle import oracle as O
    descs, Sa, ga, nP = build_batch(0, args.systems, os.cpu_count() or 1)
    # block-Jacobi Phi^-1 (compact) on the host in FP64, like the GPU builder
    Pa = np.zeros(nP, np.float32)
    for (n, N, oS, oP, oV) in descs:
        lo, di, up = O.unpack_cbtd(Sa[oS:oS + 3 * n * n * N], n, N)
        Pa[oP:oP + n * n * N] = O.block_jacobi(di, "compact").astype(np.float32)
    threads = os.cpu_count() or 1
    # each step: about 5 s of host work (the whole batch once, or its first systems);
    # calibrated on 256 systems
    rate, _, _, _, _ = cpu_port_baseline(Sa, Pa, ga, descs, min(256, len(descs)), threads)
    sample = int(min(len(descs), max(64, rate * 5.0)))
    for _ in range(args.warmup):
        cpu_port_baseline(Sa, Pa, ga, descs, min(sample, 64), threads)
    times, used = [], threads
    for _ in range(args.steps):
        r, dt, used, _, _ = cpu_port_baseline(Sa, Pa, ga, descs, sample, threads)
        times.append(dt)
    total = sum(times)
    value = sample * args.steps / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "systems_per_step": sample, "l2": "host run"},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": used, "kind": "port",
                             "sample": f"first {sample} of the {len(descs)} systems per step (the reference ships "
                                       f"no CPU path; oracle/pcg_oracle.c restates its PCG)"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    import gbdpcg
    if not os.path.exists(gbdpcg.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    gbdpcg.lib()
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    if args.only == "around-solve":
        print(json.dumps({"around_solve": around_solve_kernels(gbdpcg, dev, hbm, N=args.knots)}), flush=True)
        return
    if args.only == "adjoint":
        h1 = gbdpcg.Handle(local)
        print(json.dumps({"adjoint": adjoint_config(gbdpcg, h1, dev, gbdpcg.TUNE_RECURRENCE)}), flush=True)
        h1.close()
        return
    if args.only == "single-system":
        h1 = gbdpcg.Handle(local)
        print(json.dumps({"single_system": single_system_latency(gbdpcg, h1, dev)}), flush=True)
        h1.close()
        return
    if args.only == "single-system-n128":
        h1 = gbdpcg.Handle(local)
        print(json.dumps({"single_system_n128": n128_seed_sweep(gbdpcg, h1, dev)}), flush=True)
        h1.close()
        return

    descs, Sa, ga, nP = build_batch(rank, args.systems, max(1, (os.cpu_count() or 1) // max(1, world)), world)
    count = len(descs)              # this rank's part of the job's batch
    job_systems = world * args.systems
    dS = torch.from_numpy(Sa).to(dev)
    dg = torch.from_numpy(ga).to(dev)
    dP = torch.empty(nP, dtype=torch.float32, device=dev)
    dl = torch.zeros(ga.size, dtype=torch.float32, device=dev)
    h = gbdpcg.Handle(local)
    algo = {"auto": gbdpcg.ALGO_AUTO, "standard": gbdpcg.ALGO_CLUSTER, "recurrence": gbdpcg.ALGO_RECURRENCE,
            "single-reduction": gbdpcg.ALGO_SINGLE_REDUCTION}[args.algorithm]
    storage = {"auto": gbdpcg.STORAGE_AUTO, "registers": gbdpcg.STORAGE_REGISTERS, "shared": gbdpcg.STORAGE_SHARED,
               "split": gbdpcg.STORAGE_SPLIT, "hybrid": gbdpcg.STORAGE_HYBRID, "tmem": gbdpcg.STORAGE_TMEM}[args.storage]
    cfg = gbdpcg.config(max_iter=MAX_ITER, exit_tol=TOL, exit_mode=gbdpcg.EXIT_RELRES, zero_guess=1, algorithm=algo,
                        host_pieces=args.host_pieces, storage=storage, cluster_size=args.cluster_size)
    plan = gbdpcg.Plan(h, layout=gbdpcg.PINV_BLOCKDIAG, cfg=cfg, packed=(descs, dS, dP, dg, dl))
    plan.build_block_jacobi()
    torch.cuda.synchronize()
    if args.only == "block-jacobi":
        print(json.dumps({"block_jacobi": block_jacobi_build(plan, descs, hbm)}), flush=True)
        return
    tune_s = 0.0
    tune_flags = {"off": None, "shapes": 0, "shapes+recurrence": gbdpcg.TUNE_RECURRENCE,
                  "shapes+recurrence+plan": gbdpcg.TUNE_RECURRENCE | gbdpcg.TUNE_WHOLE_PLAN,
                  "shapes+algorithms": gbdpcg.TUNE_RECURRENCE | gbdpcg.TUNE_SINGLE_REDUCTION}[args.tune]
    if tune_flags is not None:
        t0 = time.perf_counter()
        plan.autotune(flags=tune_flags)
        tune_s = time.perf_counter() - t0
    launches = plan.launches()
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    stream = torch.cuda.current_stream()
    if args.only == "timeline":
        for _ in range(3):
            plan.execute()
        print(json.dumps({"timeline": timeline_and_floor(gbdpcg, h, plan, launches, dev, sm_count)}), flush=True)
        return
    for _ in range(max(3, args.warmup)):
        plan.execute()
    res = plan.results()
    iters = [r.iters for r in res]
    status = [r.status for r in res]
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident timing
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("timed")  # profilers can select the timed launches by this range
        e0.record(stream)
        for _ in range(args.steps):
            plan.execute()
        e1.record(stream)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        barrier()
    clocks = clk.summary()
    ms = max_over_ranks(e0.elapsed_time(e1), world, dev)
    ms_step = ms / args.steps
    value = whole_job_rate(job_systems, args.steps, ms / 1e3)

    # ---- end to end from pinned host buffers through the C ABI: the batched
    # pcg_solve (S and gamma in, Phi^-1 built on the device, lambda and the
    # results out), every copy inside the timed region
    hS = torch.from_numpy(Sa).pin_memory()
    hP = dP.cpu().pin_memory()
    hg = torch.from_numpy(ga).pin_memory()
    hl = torch.zeros(ga.size, dtype=torch.float32).pin_memory()
    # The host link is shared with the box's other jobs: each step is timed on
    # its own (every call waits for its results) and the rate is taken from
    # the median step, with the mean-step rate reported beside it.
    e2e_steps = max(5, args.steps // 2)

    def host_steps(fn):
        fn()  # warm
        barrier()
        ts = []
        gc.collect()
        gc.disable()  # as timeit does: no cyclic collection inside a timed step
        try:
            for _ in range(e2e_steps):
                t0 = time.perf_counter()
                fn()
                ts.append(time.perf_counter() - t0)
        finally:
            gc.enable()
        return (max_over_ranks(statistics.median(ts), world, dev), max_over_ranks(sum(ts), world, dev))

    e2e_med, e2e_s = host_steps(lambda: plan.solve_host(hS, hg, hl, with_results=True))
    h2d = (hS.numel() + hg.numel()) * 4
    d2h = hl.numel() * 4 + count * 24
    # the same with a host-built Phi^-1 copied in as well (solvePCG with Pinv)
    e2e_p_med, e2e_p_s = host_steps(lambda: plan.execute_host(hS, hP, hg, hl, with_results=True))

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    # ---- accuracy in FP64 (sample) and the bytes model
    algo_bytes, compulsory, flops = algorithmic_bytes(descs, iters)
    lam = dl.cpu().numpy()
    worst = max(relres64(Sa[oS:oS + 3 * n * n * N], ga[oV:oV + n * N], lam[oV:oV + n * N], n, N)
                for (n, N, oS, oP, oV) in descs[:: max(1, count // 64)])

    achieved = algo_bytes / (ms_step / 1e3) / 1e9
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            tj = json.load(f).get(WORKLOAD)
        if tj and tj.get("systems") == count:
            traffic = tj["dram_bytes_per_step"]
    except (OSError, ValueError):
        pass

    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator, see config)",
        "config": {"workload": WORKLOAD, "algorithm": args.algorithm, "storage": args.storage,
                   "cluster_size": args.cluster_size, "systems_per_gpu": args.systems,
                   "global_batch": job_systems,
                   "seeds": (f"[0, {job_systems})" + ("" if world == 1 else
                             ", split over the ranks by estimated cost (gbdpcg_partition)")),
                   "l2": "inputs (1.1 GB/GPU) larger than L2",
                   "parallelism": f"replicas{world} (independent systems per GPU)",
                   "launches_per_step": len(launches), "autotune": args.tune,
                   "autotune_s": round(tune_s, 2),
                   "launch_shapes": [[l["cluster"], l["threads"], l["storage"], l["rows_per_thread"],
                                      l["algorithm"], l["systems"]] for l in launches]},
        "iterations": {"mean": float(np.mean(iters)), "max": int(np.max(iters)), "min": int(np.min(iters)),
                       "all_converged": bool(all(s == 0 for s in status))},
        "true_relres_max_sample": worst,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic,
                     "basis": "streaming-equivalent bytes sizeof(T)[(3N-2)n^2+Nn^2+6nN] per PCG iteration "
                              "per system, summed over iterations, per step; peak = measured HBM copy",
                     "compulsory": {"bytes_per_step": compulsory,
                                    "achieved": compulsory / (ms_step / 1e3) / 1e9,
                                    "frac": compulsory / (ms_step / 1e3) / 1e9 / hbm},
                     "fp32_flops_per_step": flops, "fp32_tflops": flops / (ms_step / 1e3) / 1e12},
        "e2e": {"value": whole_job_rate(job_systems, 1, e2e_med), "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": e2e_steps, "statistic": "median step",
                "mean_step_value": whole_job_rate(job_systems, e2e_steps, e2e_s),
                "path": "gbdpcg_plan_solve_host (batched pcg_solve): S, gamma in; Phi^-1 built on the GPU; "
                        "lambda and results out; pinned host memory",
                "with_pinv_copied": {"value": whole_job_rate(job_systems, 1, e2e_p_med), "unit": "solves/s",
                                     "mean_step_value": whole_job_rate(job_systems, e2e_steps, e2e_p_s),
                                     "h2d_bytes_per_step": h2d + hP.numel() * 4,
                                     "path": "gbdpcg_plan_execute_host (solvePCG with Pinv)"}},
        "gpu_launches": len(launches) * args.steps,
        "clocks": clocks,
    }

    if not args.no_extras and world == 1:
        # ---- plain PCG: one system per launch (reference scheme, cbtd Phi^-1), on a sample
        sample = descs[:: max(1, count // 128)][:128]
        Pc = dP.cpu().numpy()
        t_plain, t_single, n_ok = 0.0, 0.0, 0
        for (n, N, oS, oP, oV) in sample:
            Pt = np.zeros((N, 3 * n, n), np.float32)
            Pt[:, n:2 * n, :] = Pc[oP:oP + n * n * N].reshape(N, n, n)
            tPt = torch.from_numpy(Pt.reshape(-1)).to(dev)
            tS = dS[oS:oS + 3 * n * n * N]
            tg = dg[oV:oV + n * N]
            lamt = torch.zeros(n * N, device=dev)
            cp = gbdpcg.config(max_iter=MAX_ITER, exit_tol=TOL, exit_mode=gbdpcg.EXIT_RELRES,
                               algorithm=gbdpcg.ALGO_PLAIN, zero_guess=1)
            cc = gbdpcg.config(max_iter=MAX_ITER, exit_tol=TOL, exit_mode=gbdpcg.EXIT_RELRES, zero_guess=1)
            h.solve(tS, tPt, tg, lamt, n, N, gbdpcg.PINV_CBTD, cp)  # warm
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            h.solve(tS, tPt, tg, lamt, n, N, gbdpcg.PINV_CBTD, cp, sync=False)
            b.record(stream)
            b.synchronize()
            t_plain += a.elapsed_time(b)
            a.record(stream)
            h.solve(tS, dP[oP:oP + n * n * N], tg, lamt, n, N, gbdpcg.PINV_BLOCKDIAG, cc, sync=False)
            b.record(stream)
            b.synchronize()
            t_single += a.elapsed_time(b)
            n_ok += 1
        plain_rate = n_ok / (t_plain / 1e3)
        line["plain_pcg"] = {"value": plain_rate, "unit": "solves/s",
                             "sample": f"{n_ok} systems of the batch, one cooperative launch each "
                                       "(plain kernel, cbtd Phi^-1)",
                             "batched_speedup": value / plain_rate,
                             "single_cluster_solve_value": n_ok / (t_single / 1e3)}
        # ---- host-core port of the same PCG (the CPU baseline)
        threads = os.cpu_count() or 1
        Pn = dP.cpu().numpy()
        rate, _, _, _, _ = cpu_port_baseline(Sa, Pn, ga, descs, min(256, count), threads)
        csample, cpasses = cpu_sample_size(rate, count)
        rate, dt, used, _, _ = cpu_port_baseline(Sa, Pn, ga, descs, csample, threads, cpasses)
        line["cpu_baseline"] = {"value": rate, "unit": "solves/s", "cores": used, "kind": "port",
                                "sample": f"first {csample} of the {count} systems x {cpasses} passes, "
                                          f"oracle/pcg_oracle.c, {dt:.1f} s"}
    if not args.no_extras and world == 1:
        for key, fn in (("single_system", lambda: single_system_latency(gbdpcg, h, dev)),
                        ("single_system_n128", lambda: n128_seed_sweep(gbdpcg, h, dev)),
                        ("adjoint", lambda: adjoint_config(gbdpcg, h, dev, tune_flags)),
                        ("precision", lambda: precision_config(gbdpcg, h, dev)),
                        ("around_solve", lambda: around_solve_kernels(gbdpcg, dev, hbm)),
                        ("block_jacobi", lambda: block_jacobi_build(plan, descs, hbm)),
                        ("timeline", lambda: timeline_and_floor(gbdpcg, h, plan, launches, dev, sm_count))):
            try:
                line[key] = fn()
            except Exception as e:  # report, do not lose the headline line
                line[key] = {"error": repr(e)}
        lat = line.get("timeline", {}).get("latency")
        if lat:
            # the bound that binds: per-iteration latency against the floor the
            # synchronisation primitives put under an iteration
            line["roofline"]["latency"] = {
                k: {"floor_us_per_iter": v["floor_us_per_iter"], "achieved_us_per_iter": v["achieved_us_per_iter"],
                    "frac": v["frac"], "shape": v["shape"]} for k, v in lat.items()}
    print(json.dumps(line), flush=True)
    plan.close()
    h.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
