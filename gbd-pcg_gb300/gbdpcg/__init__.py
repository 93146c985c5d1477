"""Python binding of the GB300 PCG solver's C ABI (include/gbdpcg.h).

The compute runs in libgbdpcg.so (hand-written sm_103a CUDA); this module only
marshals arguments.  There is no fallback: if the library is missing, every
call raises.

Mirrors the reference's interface (Sdevaud/GBD-PCG include/interface.cuh,
include/types.cuh): `pcg_config` defaults (tol 1e-6, 25 iterations),
`solvePCG(S, Pinv, gamma, lambda, stateSize, knotPoints, config)` with lambda
in/out, `pcg_solve(S, gamma, lambda, ...)` with the preconditioner built on the
GPU.  Unlike the reference, the host form returns the iteration count (the
reference returns 1, include/interface.cuh:90) and reports errors by raising
instead of exiting the process.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "_build", "libgbdpcg.so")

SUCCESS, ERR_INVALID_ARGUMENT, ERR_UNSUPPORTED, ERR_CUDA, ERR_NO_MEMORY = 0, 1, 2, 3, 4
CONVERGED, MAX_ITER, BREAKDOWN, TIMEOUT, REJECTED = 0, 1, 2, 3, -1
EXIT_REFERENCE, EXIT_RELRES = 0, 1
PINV_CBTD, PINV_BLOCKDIAG = 0, 1
ALGO_AUTO, ALGO_CLUSTER, ALGO_PLAIN, ALGO_SINGLE_REDUCTION, ALGO_RECURRENCE = 0, 1, 2, 3, 4
TUNE_RECURRENCE, TUNE_SINGLE_REDUCTION, TUNE_WHOLE_PLAN = 1, 2, 4
DOT_NATIVE, DOT_FP64, DOT_FLOAT2 = 0, 1, 2
STORAGE_AUTO, STORAGE_REGISTERS, STORAGE_SHARED, STORAGE_SPLIT, STORAGE_HYBRID, STORAGE_TMEM = 0, 1, 2, 3, 4, 5
STORAGE_STREAM = 6


class GbdpcgError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what}: {status_string(code)} ({code}): {last_error()}")
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [("exit_tol", ctypes.c_double), ("max_iter", ctypes.c_uint32),
                ("exit_mode", ctypes.c_uint32), ("dot_precision", ctypes.c_uint32),
                ("algorithm", ctypes.c_uint32), ("cluster_size", ctypes.c_uint32),
                ("max_threads", ctypes.c_uint32), ("storage", ctypes.c_uint32),
                ("use_graph", ctypes.c_uint32), ("zero_guess", ctypes.c_uint32),
                ("max_outer", ctypes.c_uint32), ("streams", ctypes.c_uint32), ("host_pieces", ctypes.c_uint32),
                ("inner_tol", ctypes.c_double)]


class Result(ctypes.Structure):
    _fields_ = [("iters", ctypes.c_uint32), ("status", ctypes.c_int32), ("eta", ctypes.c_double),
                ("relres", ctypes.c_double), ("outer", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]

    def __repr__(self):
        return (f"Result(iters={self.iters}, status={self.status}, eta={self.eta:.3g}, "
                f"relres={self.relres:.3g}, outer={self.outer})")


class PackedSystem(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("N", ctypes.c_uint32), ("S_off", ctypes.c_uint64),
                ("Pinv_off", ctypes.c_uint64), ("vec_off", ctypes.c_uint64)]


class FwdAdjSystem(ctypes.Structure):
    """gbdpcg_fwd_adj_system: a forward solve and the adjoint of L = 1/2 ||lambda - lambda*||^2."""
    _fields_ = [("S", ctypes.c_void_p), ("Pinv", ctypes.c_void_p), ("gamma", ctypes.c_void_p),
                ("lambda_", ctypes.c_void_p), ("lambda_target", ctypes.c_void_p), ("grad_gamma", ctypes.c_void_p),
                ("grad_S", ctypes.c_void_p), ("n", ctypes.c_uint32), ("N", ctypes.c_uint32)]


class Stamp(ctypes.Structure):
    """gbdpcg_stamp: one system's timeline (GPU global clock, ns)."""
    _fields_ = [("t_pop", ctypes.c_uint64), ("t_staged", ctypes.c_uint64), ("t_solved", ctypes.c_uint64),
                ("t_done", ctypes.c_uint64), ("system", ctypes.c_uint32), ("launch", ctypes.c_uint32),
                ("cluster", ctypes.c_uint32), ("iters", ctypes.c_uint32)]


class Probe(ctypes.Structure):
    """gbdpcg_probe: ns per repetition of each synchronisation primitive."""
    _fields_ = [("loop_ns", ctypes.c_double), ("syncthreads_ns", ctypes.c_double),
                ("cluster_barrier_ns", ctypes.c_double), ("dsmem_store_barrier_ns", ctypes.c_double),
                ("allreduce_ns", ctypes.c_double * 3), ("allreduce_tx_ns", ctypes.c_double * 3)]


def probe_primitives(device=0, cluster=1, threads=128, clusters=1, reps=100000) -> dict:
    """Latency of the solver's synchronisation primitives (gbdpcg_probe_primitives)."""
    p = Probe()
    _check(lib().gbdpcg_probe_primitives(device, cluster, threads, clusters, reps, ctypes.byref(p)),
           "gbdpcg_probe_primitives")
    return {"loop_ns": p.loop_ns, "syncthreads_ns": p.syncthreads_ns, "cluster_barrier_ns": p.cluster_barrier_ns,
            "dsmem_store_barrier_ns": p.dsmem_store_barrier_ns, "allreduce_ns": list(p.allreduce_ns),
            "allreduce_tx_ns": list(p.allreduce_tx_ns)}


def probe_timeout(device=0, cluster=2) -> tuple:
    """A wait that nothing completes, through the solver's bounded wait
    (gbdpcg_probe_timeout): (status, ms waited)."""
    st, ms = ctypes.c_int(0), ctypes.c_double(0)
    _check(lib().gbdpcg_probe_timeout(device, cluster, ctypes.byref(st), ctypes.byref(ms)), "gbdpcg_probe_timeout")
    return st.value, ms.value


class System(ctypes.Structure):
    _fields_ = [("S", ctypes.c_void_p), ("Pinv", ctypes.c_void_p), ("gamma", ctypes.c_void_p),
                ("lambda_", ctypes.c_void_p), ("lambda_fwd", ctypes.c_void_p), ("dS", ctypes.c_void_p),
                ("n", ctypes.c_uint32), ("N", ctypes.c_uint32)]


# Every symbol of include/gbdpcg.h with its ctypes signature.
_P, _U, _I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
_SIGS = {
    "gbdpcg_version": ([], _I),
    "gbdpcg_status_string": ([_I], ctypes.c_char_p),
    "gbdpcg_last_error": ([], ctypes.c_char_p),
    "gbdpcg_config_init": ([_P], None),
    "gbdpcg_create": ([_P, _I], _I),
    "gbdpcg_destroy": ([_P], _I),
    "gbdpcg_solve_f32": ([_P, _P, _P, _P, _U, _U, _P, _P], _I),
    "gbdpcg_solve_f64": ([_P, _P, _P, _P, _U, _U, _P, _P], _I),
    "gbdpcg_solve_dev_f32": ([_P, _P, _P, _U, _P, _P, _U, _U, _P, _P, _P], _I),
    "gbdpcg_solve_dev_f64": ([_P, _P, _P, _U, _P, _P, _U, _U, _P, _P, _P], _I),
    "gbdpcg_last_result": ([_P, _P], _I),
    "gbdpcg_block_jacobi_f32": ([_P, _P, _P, _U, _U, _U, _P], _I),
    "gbdpcg_block_jacobi_f64": ([_P, _P, _P, _U, _U, _U, _P], _I),
    "gbdpcg_block_jacobi_f64to32": ([_P, _P, _P, _U, _U, _P], _I),
    "gbdpcg_refine_solve_dev": ([_P, _P, _P, _P, _P, _U, _U, _P, _P, _P], _I),
    "gbdpcg_solve_plain_noalloc_f32": ([_P, _P, _P, _P, _U, _U, _P, _P, _P], _I),
    "gbdpcg_adjoint_dev_f32": ([_P, _P, _P, _U, _P, _P, _P, _P, _U, _U, _P, _P, _P], _I),
    "gbdpcg_plan_create": ([_P, _I, _P, _U, _U, _P, _P], _I),
    "gbdpcg_plan_create_fwd_adj": ([_P, _I, _P, _U, _U, _P, _P], _I),
    "gbdpcg_plan_execute": ([_P, _P], _I),
    "gbdpcg_plan_create_packed": ([_P, _I, _P, _U, _P, _P, _P, _P, _U, _P, _P], _I),
    "gbdpcg_plan_execute_host": ([_P, _P, _P, _P, _P, _P, _P], _I),
    "gbdpcg_plan_solve_host": ([_P, _P, _P, _P, _P, _P], _I),
    "gbdpcg_plan_build_block_jacobi": ([_P, _P], _I),
    "gbdpcg_plan_results": ([_P, _P, _P], _I),
    "gbdpcg_plan_launch_count": ([_P, _P], _I),
    "gbdpcg_plan_launch_info": ([_P, _U, _P, _P, _P, _P, _P], _I),
    "gbdpcg_plan_launch_kernel": ([_P, _U, _P, _P, _P], _I),
    "gbdpcg_plan_destroy": ([_P], _I),
    "gbdpcg_plan_timeline": ([_P, _I], _I),
    "gbdpcg_plan_timeline_read": ([_P, _P, _U, _P, _P, _U, _P, _P], _I),
    "gbdpcg_probe_primitives": ([_I, _U, _U, _U, _U, _P], _I),
    "gbdpcg_probe_timeout": ([_I, _U, _P, _P], _I),
    "gbdpcg_partition": ([_P, _P, _P, _U, _U, _P, _P], _I),
    "gbdpcg_form_schur_f32": ([_P] * 7 + [_U, _U, _U, _P, _P, _P], _I),
    "gbdpcg_form_schur_f64": ([_P] * 7 + [_U, _U, _U, _P, _P, _P], _I),
    "gbdpcg_form_schur_pinv_f32": ([_P] * 7 + [_U, _U, _U, _P, _P, _P, _P], _I),
    "gbdpcg_form_schur_pinv_f64": ([_P] * 7 + [_U, _U, _U, _P, _P, _P, _P], _I),
    "gbdpcg_kkt_backsub_f32": ([_P] * 7 + [_U, _U, _U, _P, _P, _P], _I),
    "gbdpcg_kkt_backsub_f64": ([_P] * 7 + [_U, _U, _U, _P, _P, _P], _I),
    "gbdpcg_csr_to_cbtd_f32": ([_P, _P, _P, _U, _U, _P, _P, _P], _I),
    "gbdpcg_csr_to_cbtd_f64": ([_P, _P, _P, _U, _U, _P, _P, _P], _I),
    "gbdpcg_dense_to_cbtd_f32": ([_P, ctypes.c_uint64, _I, _U, _U, _P, _P, _P], _I),
    "gbdpcg_dense_to_cbtd_f64": ([_P, ctypes.c_uint64, _I, _U, _U, _P, _P, _P], _I),
    "gbdpcg_plan_autotune": ([_P, _U, _U, _P], _I),
    "gbdpcg_tune_export": ([_P, _P, ctypes.c_size_t, _P], _I),
    "gbdpcg_tune_import": ([_P, ctypes.c_char_p], _I),
    "gbdpcg_tune_clear": ([_P], _I),
}

_lib = None


def lib():
    """Load libgbdpcg.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libgbdpcg.so not built ({LIB_PATH}); run gbd-pcg_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def status_string(code: int) -> str:
    return lib().gbdpcg_status_string(code).decode()


def last_error() -> str:
    return lib().gbdpcg_last_error().decode()


def _check(code: int, what: str):
    if code != SUCCESS:
        raise GbdpcgError(code, what)


def config(**kw) -> Config:
    """pcg_config defaults (include/types.cuh:18-34) with overrides."""
    c = Config()
    lib().gbdpcg_config_init(ctypes.byref(c))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise AttributeError(k)
        setattr(c, k, v)
    return c


def _np_ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


# ------------------------------------------------------------------- host pointers
def solve(S: np.ndarray, Pinv: Optional[np.ndarray], gamma: np.ndarray, lam: np.ndarray,
          n: int, N: int, cfg: Optional[Config] = None) -> Result:
    """Host-array solve (solvePCG host overload; Pinv None = pcg_solve with the
    block-Jacobi preconditioner built on the GPU).  `lam` is updated in place."""
    dt = lam.dtype
    if dt not in (np.float32, np.float64):
        raise TypeError("float32 or float64 arrays")
    for a in (S, gamma, lam) + ((Pinv,) if Pinv is not None else ()):
        if a.dtype != dt or not a.flags.c_contiguous:
            raise TypeError("all arrays must be C-contiguous and of one dtype")
    if S.size != 3 * n * n * N or gamma.size != n * N or lam.size != n * N:
        raise ValueError("array sizes do not match n, N")
    if Pinv is not None and Pinv.size != 3 * n * n * N:
        raise ValueError("Pinv must be cbtd (3 n^2 N)")
    r = Result()
    fn = lib().gbdpcg_solve_f64 if dt == np.float64 else lib().gbdpcg_solve_f32
    _check(fn(_np_ptr(S), _np_ptr(Pinv) if Pinv is not None else None, _np_ptr(gamma), _np_ptr(lam),
              n, N, ctypes.byref(cfg) if cfg is not None else None, ctypes.byref(r)), "gbdpcg_solve")
    return r


def solvePCG(h_S, h_Pinv, h_gamma, h_lambda, stateSize, knotPoints, config_=None) -> int:
    """The reference's host solvePCG (include/interface.cuh:24-32); returns the
    iteration count."""
    return solve(h_S, h_Pinv, h_gamma, h_lambda, stateSize, knotPoints, config_).iters


def pcg_solve(h_S, h_gamma, h_lambda, stateSize, knotPoints, config_=None) -> int:
    """The reference's documented pcg_solve (README.md:42): block-Jacobi Phi^-1
    built on the GPU; returns the iteration count."""
    return solve(h_S, None, h_gamma, h_lambda, stateSize, knotPoints, config_).iters


# ------------------------------------------------------------------- device pointers (torch)
def _tp(t) -> Optional[int]:
    return None if t is None else t.data_ptr()


def _stream(stream) -> Optional[int]:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return stream if isinstance(stream, int) else stream.cuda_stream


class Handle:
    def __init__(self, device: int = 0):
        self.h = ctypes.c_void_p()
        _check(lib().gbdpcg_create(ctypes.byref(self.h), device), "gbdpcg_create")

    def close(self):
        if self.h:
            lib().gbdpcg_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, S, Pinv, gamma, lam, n, N, layout=PINV_CBTD, cfg=None, stream=None, sync=True):
        """Device solve; torch CUDA tensors; `lam` in/out.  Returns Result if sync."""
        cfg = cfg or config()
        fn = lib().gbdpcg_solve_dev_f64 if lam.dtype.itemsize == 8 else lib().gbdpcg_solve_dev_f32
        r = Result()
        _check(fn(self.h, _tp(S), _tp(Pinv), layout, _tp(gamma), _tp(lam), n, N, ctypes.byref(cfg),
                  ctypes.byref(r) if sync else None, _stream(stream)), "gbdpcg_solve_dev")
        return r if sync else None

    def last_result(self) -> Result:
        r = Result()
        _check(lib().gbdpcg_last_result(self.h, ctypes.byref(r)), "gbdpcg_last_result")
        return r

    def block_jacobi(self, S, Pinv_out, n, N, layout=PINV_BLOCKDIAG, stream=None):
        fn = lib().gbdpcg_block_jacobi_f64 if S.dtype.itemsize == 8 else lib().gbdpcg_block_jacobi_f32
        _check(fn(self.h, _tp(S), _tp(Pinv_out), layout, n, N, _stream(stream)), "gbdpcg_block_jacobi")

    def block_jacobi_f64to32(self, S64, Pinv32_out, n, N, stream=None):
        _check(lib().gbdpcg_block_jacobi_f64to32(self.h, _tp(S64), _tp(Pinv32_out), n, N, _stream(stream)),
               "gbdpcg_block_jacobi_f64to32")

    def refine_solve(self, S64, Pinv32, gamma64, lam64, n, N, cfg=None, stream=None, sync=True):
        """FP64 system by FP32 PCG + FP64 refinement (cfg.exit_mode must be EXIT_RELRES)."""
        cfg = cfg or config(exit_mode=EXIT_RELRES, exit_tol=1e-10, max_iter=20000)
        r = Result()
        _check(lib().gbdpcg_refine_solve_dev(self.h, _tp(S64), _tp(Pinv32), _tp(gamma64), _tp(lam64), n, N,
                                             ctypes.byref(cfg), ctypes.byref(r) if sync else None,
                                             _stream(stream)), "gbdpcg_refine_solve_dev")
        return r if sync else None

    def tune_export(self) -> str:
        """The handle's tuning table as text."""
        n = ctypes.c_size_t()
        _check(lib().gbdpcg_tune_export(self.h, None, 0, ctypes.byref(n)), "gbdpcg_tune_export")
        buf = ctypes.create_string_buffer(n.value + 1)
        _check(lib().gbdpcg_tune_export(self.h, buf, n.value + 1, ctypes.byref(n)), "gbdpcg_tune_export")
        return buf.value.decode()

    def tune_import(self, text: str):
        _check(lib().gbdpcg_tune_import(self.h, text.encode()), "gbdpcg_tune_import")

    def tune_clear(self):
        _check(lib().gbdpcg_tune_clear(self.h), "gbdpcg_tune_clear")

    def adjoint(self, S, Pinv, lam, grad_lam, grad_gamma, grad_S, n, N, layout=PINV_CBTD, cfg=None,
                stream=None, sync=True):
        cfg = cfg or config()
        r = Result()
        _check(lib().gbdpcg_adjoint_dev_f32(self.h, _tp(S), _tp(Pinv), layout, _tp(lam), _tp(grad_lam),
                                            _tp(grad_gamma), _tp(grad_S), n, N, ctypes.byref(cfg),
                                            ctypes.byref(r) if sync else None, _stream(stream)),
               "gbdpcg_adjoint_dev_f32")
        return r if sync else None


class Plan:
    """Batched solve of many systems (device tensors).  `systems` is a list of
    dicts with keys S, Pinv, gamma, lambda (and lambda_fwd, dS for an adjoint
    plan), n, N.  The tensors must stay alive as long as the plan."""

    def __init__(self, handle: Handle, systems=None, layout=PINV_BLOCKDIAG, cfg=None, dtype=None,
                 packed=None):
        cfg = cfg or config()
        self.handle = handle
        self.p = ctypes.c_void_p()
        if packed is not None:
            # packed = (list of (n, N, S_off, Pinv_off, vec_off), S, Pinv, gamma, lambda) tensors
            descs, S, P, g, l = packed
            arr = (PackedSystem * len(descs))(*[PackedSystem(*d) for d in descs])
            self.count = len(descs)
            dt = dtype if dtype is not None else (1 if S.dtype.itemsize == 8 else 0)
            _check(lib().gbdpcg_plan_create_packed(handle.h, dt, ctypes.cast(arr, ctypes.c_void_p), len(descs),
                                                   _tp(S), _tp(P), _tp(g), _tp(l), layout, ctypes.byref(cfg),
                                                   ctypes.byref(self.p)), "gbdpcg_plan_create_packed")
            return
        if dtype is None:
            dtype = 1 if systems[0]["S"].dtype.itemsize == 8 else 0
        arr = (System * len(systems))()
        for i, s in enumerate(systems):
            arr[i] = System(_tp(s["S"]), _tp(s["Pinv"]), _tp(s["gamma"]), _tp(s["lambda"]),
                            _tp(s.get("lambda_fwd")), _tp(s.get("dS")), s["n"], s["N"])
        self.count = len(systems)
        self.handle = handle
        self.p = ctypes.c_void_p()
        _check(lib().gbdpcg_plan_create(handle.h, dtype, ctypes.cast(arr, ctypes.c_void_p), len(systems),
                                        layout, ctypes.byref(cfg), ctypes.byref(self.p)), "gbdpcg_plan_create")

    @classmethod
    def forward_adjoint(cls, handle, systems, layout=PINV_BLOCKDIAG, cfg=None, dtype=None):
        """A plan of forward + adjoint pairs (gbdpcg_plan_create_fwd_adj): dicts
        with S, Pinv, gamma, lambda, lambda_target, grad_gamma, grad_S, n, N.
        results() returns 2 count results: the forward solves', then the
        adjoint solves'."""
        cfg = cfg or config()
        self = cls.__new__(cls)
        self.handle = handle
        self.p = ctypes.c_void_p()
        if dtype is None:
            dtype = 1 if systems[0]["S"].dtype.itemsize == 8 else 0
        arr = (FwdAdjSystem * len(systems))()
        for i, s in enumerate(systems):
            arr[i] = FwdAdjSystem(_tp(s["S"]), _tp(s["Pinv"]), _tp(s["gamma"]), _tp(s["lambda"]),
                                  _tp(s["lambda_target"]), _tp(s["grad_gamma"]), _tp(s["grad_S"]), s["n"], s["N"])
        self.count = 2 * len(systems)
        _check(lib().gbdpcg_plan_create_fwd_adj(handle.h, dtype, ctypes.cast(arr, ctypes.c_void_p), len(systems),
                                                layout, ctypes.byref(cfg), ctypes.byref(self.p)),
               "gbdpcg_plan_create_fwd_adj")
        return self

    def execute(self, stream=None):
        _check(lib().gbdpcg_plan_execute(self.p, _stream(stream)), "gbdpcg_plan_execute")

    def execute_host(self, h_S, h_P, h_g, h_l, with_results=False, stream=None):
        """End-to-end from host arrays (numpy or pinned CPU tensors).  With
        with_results, returns the per-system results as a ctypes array of
        Result (a sequence, filled in place by the library)."""
        def ptr(a):
            if a is None:
                return None
            return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data_as(ctypes.c_void_p)
        res = (Result * self.count)() if with_results else None
        _check(lib().gbdpcg_plan_execute_host(self.p, ptr(h_S), ptr(h_P), ptr(h_g), ptr(h_l),
                                              ctypes.cast(res, ctypes.c_void_p) if res is not None else None,
                                              _stream(stream)), "gbdpcg_plan_execute_host")
        return res

    def solve_host(self, h_S, h_g, h_l, with_results=False, stream=None):
        """pcg_solve over the batch from host arrays: S and gamma in, Phi^-1 built
        on the device, lambda out (results as in execute_host)."""
        def ptr(a):
            return a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data_as(ctypes.c_void_p)
        res = (Result * self.count)() if with_results else None
        _check(lib().gbdpcg_plan_solve_host(self.p, ptr(h_S), ptr(h_g), ptr(h_l),
                                            ctypes.cast(res, ctypes.c_void_p) if res is not None else None,
                                            _stream(stream)), "gbdpcg_plan_solve_host")
        return res

    def build_block_jacobi(self, stream=None):
        _check(lib().gbdpcg_plan_build_block_jacobi(self.p, _stream(stream)), "gbdpcg_plan_build_block_jacobi")

    def results(self, stream=None):
        arr = (Result * self.count)()
        _check(lib().gbdpcg_plan_results(self.p, ctypes.cast(arr, ctypes.c_void_p), _stream(stream)),
               "gbdpcg_plan_results")
        return arr  # ctypes array of Result: a sequence, no per-element conversion

    def launches(self):
        c = ctypes.c_uint32()
        _check(lib().gbdpcg_plan_launch_count(self.p, ctypes.byref(c)), "gbdpcg_plan_launch_count")
        out = []
        for i in range(c.value):
            v = [ctypes.c_uint32() for _ in range(5)]
            _check(lib().gbdpcg_plan_launch_info(self.p, i, *[ctypes.byref(x) for x in v]),
                   "gbdpcg_plan_launch_info")
            d = dict(zip(("cluster", "threads", "kmax", "systems", "ctas"), [x.value for x in v]))
            k = [ctypes.c_uint32() for _ in range(3)]
            _check(lib().gbdpcg_plan_launch_kernel(self.p, i, *[ctypes.byref(x) for x in k]),
                   "gbdpcg_plan_launch_kernel")
            d.update(zip(("storage", "rows_per_thread", "algorithm"), [x.value for x in k]))
            out.append(d)
        return out

    def timeline(self, enable=True):
        """Switch the per-system timeline of the executions on or off."""
        _check(lib().gbdpcg_plan_timeline(self.p, 1 if enable else 0), "gbdpcg_plan_timeline")

    def timeline_read(self, stream=None):
        """The last execution's timeline: (structured numpy array of the
        records, numpy array of the SM of every CTA of every launch)."""
        import numpy as np
        n, m = ctypes.c_uint32(), ctypes.c_uint32()
        _check(lib().gbdpcg_plan_timeline_read(self.p, None, 0, ctypes.byref(n), None, 0, ctypes.byref(m),
                                               _stream(stream)), "gbdpcg_plan_timeline_read")
        recs = (Stamp * max(1, n.value))()
        sms = (ctypes.c_uint32 * max(1, m.value))()
        _check(lib().gbdpcg_plan_timeline_read(self.p, ctypes.cast(recs, ctypes.c_void_p), n.value, ctypes.byref(n),
                                               ctypes.cast(sms, ctypes.c_void_p), m.value, ctypes.byref(m),
                                               _stream(stream)), "gbdpcg_plan_timeline_read")
        dt = np.dtype([("t_pop", "<u8"), ("t_staged", "<u8"), ("t_solved", "<u8"), ("t_done", "<u8"),
                       ("system", "<u4"), ("launch", "<u4"), ("cluster", "<u4"), ("iters", "<u4")])
        return (np.frombuffer(bytes(recs), dtype=dt)[:n.value].copy(),
                np.frombuffer(bytes(sms), dtype=np.uint32)[:m.value].copy())

    def autotune(self, flags=0, reps=0, stream=None):
        """Times each launch class's candidate shapes on the plan's systems and
        keeps the fastest (see gbdpcg_plan_autotune); returns launches()."""
        _check(lib().gbdpcg_plan_autotune(self.p, flags, reps, _stream(stream)), "gbdpcg_plan_autotune")
        return self.launches()

    def close(self):
        if self.p:
            lib().gbdpcg_plan_destroy(self.p)
            self.p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------- autograd
_default_handles = {}


def default_handle(device: int = 0) -> Handle:
    h = _default_handles.get(device)
    if h is None:
        h = _default_handles[device] = Handle(device)
    return h


def _make_fn():
    import torch

    class PCGSolve(torch.autograd.Function):
        """lambda = S^-1 gamma by PCG; backward by the adjoint PCG solve
        (S symmetric): dgamma = mu with S mu = dL/dlambda, and dS on the
        block-tridiagonal pattern = -1/2 (mu lambda^T + lambda mu^T)."""

        @staticmethod
        def forward(ctx, S, Pinv, gamma, n, N, layout, cfg_kw):
            h = default_handle(S.device.index or 0)
            lam = torch.zeros_like(gamma)
            r = h.solve(S, Pinv, gamma, lam, n, N, layout, config(**cfg_kw))
            ctx.save_for_backward(S, Pinv, lam)
            ctx.meta = (n, N, layout, cfg_kw)
            ctx.result = r
            return lam

        @staticmethod
        def backward(ctx, grad_lam):
            S, Pinv, lam = ctx.saved_tensors
            n, N, layout, cfg_kw = ctx.meta
            h = default_handle(S.device.index or 0)
            g_gamma = torch.empty_like(lam)
            g_S = torch.empty_like(S)
            h.adjoint(S, Pinv, lam, grad_lam.contiguous(), g_gamma, g_S, n, N, layout, config(**cfg_kw))
            return g_S, None, g_gamma, None, None, None, None

    return PCGSolve


_fn = None


def pcg_solve_autograd(S, Pinv, gamma, n, N, layout=PINV_BLOCKDIAG, **cfg_kw):
    """Differentiable solve of one float32 system (torch CUDA tensors)."""
    global _fn
    if _fn is None:
        _fn = _make_fn()
    return _fn.apply(S, Pinv, gamma, n, N, layout, cfg_kw)


def csr_to_cbtd(row_ptr, col_ind, val, n, N, out, err, stream=None):
    """CSR (device tensors: uint32-compatible int32 row_ptr / col_ind, values)
    -> cbtd `out` (3 n^2 N); `err` is a one-element int32 device tensor."""
    fn = lib().gbdpcg_csr_to_cbtd_f64 if val.dtype.itemsize == 8 else lib().gbdpcg_csr_to_cbtd_f32
    _check(fn(_tp(row_ptr), _tp(col_ind), _tp(val), n, N, _tp(out), _tp(err), _stream(stream)), "gbdpcg_csr_to_cbtd")


def dense_to_cbtd(D, n, N, out, row_major=False, ld=None, err=None, stream=None):
    """The three diagonal blocks per block row of a dense n N x n N device
    matrix (leading dimension ld, default n N) -> cbtd `out`; with `err` (a
    one-element int32 device tensor) entries outside the band are checked."""
    fn = lib().gbdpcg_dense_to_cbtd_f64 if D.dtype.itemsize == 8 else lib().gbdpcg_dense_to_cbtd_f32
    _check(fn(_tp(D), ld if ld is not None else n * N, 1 if row_major else 0, n, N, _tp(out), _tp(err),
              _stream(stream)), "gbdpcg_dense_to_cbtd")


def form_schur(A, B, Qd, Rd, q, r, c, n, m, N, S_out, gamma_out, Pinv_out=None, stream=None):
    """S = C Theta^-1 C^T (cbtd) and gamma = -(c + C Theta^-1 g) from the
    trajectory-optimisation data (device tensors; A_k, B_k column-major); with
    Pinv_out, also the compact block-Jacobi Phi^-1 from the same pass."""
    f64 = A.dtype.itemsize == 8
    if Pinv_out is None:
        fn = lib().gbdpcg_form_schur_f64 if f64 else lib().gbdpcg_form_schur_f32
        _check(fn(*[_tp(t) for t in (A, B, Qd, Rd, q, r, c)], n, m, N, _tp(S_out), _tp(gamma_out),
                  _stream(stream)), "gbdpcg_form_schur")
        return
    fn = lib().gbdpcg_form_schur_pinv_f64 if f64 else lib().gbdpcg_form_schur_pinv_f32
    _check(fn(*[_tp(t) for t in (A, B, Qd, Rd, q, r, c)], n, m, N, _tp(S_out), _tp(gamma_out), _tp(Pinv_out),
              _stream(stream)), "gbdpcg_form_schur_pinv")


def kkt_backsub(A, B, Qd, Rd, q, r, lam, n, m, N, x_out, u_out, stream=None):
    """z = -Theta^-1 (g + C^T lambda): states x (n (N+1)) and controls u (m N)."""
    fn = lib().gbdpcg_kkt_backsub_f64 if A.dtype.itemsize == 8 else lib().gbdpcg_kkt_backsub_f32
    _check(fn(*[_tp(t) for t in (A, B, Qd, Rd, q, r, lam)], n, m, N, _tp(x_out), _tp(u_out), _stream(stream)),
           "gbdpcg_kkt_backsub")
