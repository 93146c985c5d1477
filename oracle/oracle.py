"""ORACLE — test infrastructure only.

CPU-side oracle for the GB300 PCG solver.  Only tests/, __graft_entry__.smoke()
and bench.py's host-core baseline may import this module; the product never does.

Contents
  * synthetic Schur-complement systems S = C Theta^-1 C^T of optimal control
    (one block row [A_k  B_k  -I] of C per knot), packed in the reference's
    compressed block-tridiagonal ("cbtd") layout: per knot one n x 3n
    column-major block row [S_{k,k-1} | S_{k,k} | S_{k,k+1}], element (r, c) at
    k*3n^2 + c*n + r (include/utils.cuh:62,71,80; include/pcg.cuh:108), with the
    missing blocks of knots 0 and N-1 stored as zeros
    (examples/pcg_solve.cu:14,22);
  * the block-Jacobi preconditioner Phi^-1 = blockdiag(S_kk^-1) in FP64, in the
    cbtd layout (the reference's Pinv argument, include/interface.cuh:24-32) or
    compact (n^2 per knot);
  * the FP64 block-tridiagonal Cholesky solve, the accuracy oracle;
  * ctypes bindings to oracle/pcg_oracle.c (the CPU restatement of
    include/pcg.cuh:54-218) and to oracle/ref_launcher.cu (the reference
    kernel rebuilt for sm_103a, loaded from oracle/_ref/).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")

PINV_BLOCKDIAG, EXIT_RELRES, ACC64 = 1, 2, 4
CONVERGED, MAX_ITER, BREAKDOWN = 0, 1, 2

# Sizes the reference kernel is rebuilt at (oracle/ref_kernels.cu).
REF_SIZES = {
    "f32": [(2, 3), (3, 5), (5, 2), (14, 32), (14, 64), (14, 128), (6, 64), (12, 64), (24, 128)],
    "f64": [(2, 3), (3, 5), (14, 32), (14, 128)],
}


# --------------------------------------------------------------------------- generator
# The synthetic systems come from the package's workload module (pure numpy).
import sys as _sys
_PKG = os.path.join(os.path.dirname(HERE), "gbd-pcg_gb300")
if _PKG not in _sys.path:
    _sys.path.insert(0, _PKG)
from gbdpcg.workload import System, generate, generate_mixed, pack_cbtd  # noqa: E402,F401


def quantize(a: np.ndarray, bits: int = 20) -> np.ndarray:
    """Round to the grid 2^-bits.  LAPACK/BLAS differ between platforms in the
    last bits; rounding the generated inputs to a coarse grid makes the golden
    cases bit-identical on every machine (values below 2^3 then fit FP32)."""
    return np.round(np.asarray(a, np.float64) * 2.0 ** bits) / 2.0 ** bits


def golden_case(n: int, N: int, seed: int, dtype):
    """Platform-independent inputs of a golden case: (S, Pinv cbtd, gamma)."""
    sy = generate(n, N, seed)
    S = quantize(sy.cbtd()).astype(dtype)
    P = quantize(block_jacobi(sy.D)).astype(dtype)
    g = quantize(sy.gamma).astype(dtype)
    return S, P, g


def digest(*arrays) -> str:
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


def unpack_cbtd(S: np.ndarray, n: int, N: int):
    """flat cbtd -> (lower, diag, upper) blocks, each (N, n, n) row-major."""
    M = np.asarray(S, dtype=np.float64).reshape(N, 3 * n, n).transpose(0, 2, 1)
    return M[:, :, 0:n], M[:, :, n:2 * n], M[:, :, 2 * n:3 * n]


def dense_from_cbtd(S: np.ndarray, n: int, N: int) -> np.ndarray:
    lo, di, up = unpack_cbtd(S, n, N)
    A = np.zeros((n * N, n * N))
    for k in range(N):
        A[k * n:(k + 1) * n, k * n:(k + 1) * n] = di[k]
        if k > 0:
            A[k * n:(k + 1) * n, (k - 1) * n:k * n] = lo[k]
        if k + 1 < N:
            A[k * n:(k + 1) * n, (k + 1) * n:(k + 2) * n] = up[k]
    return A


def block_jacobi(D: np.ndarray, layout: str = "cbtd") -> np.ndarray:
    """Phi^-1 = blockdiag(S_kk^-1) in FP64 (via Cholesky), packed as cbtd
    (zero off-diagonal blocks) or compact (n^2 per knot, column-major)."""
    N, n, _ = D.shape
    L = np.linalg.cholesky(D)
    Li = np.linalg.inv(L)
    Pk = np.einsum("kji,kjl->kil", Li, Li)           # L^-T L^-1
    Pk = 0.5 * (Pk + Pk.transpose(0, 2, 1))
    if layout == "compact":
        return Pk.transpose(0, 2, 1).reshape(-1).copy()
    return pack_cbtd(Pk, np.zeros((max(N - 1, 0), n, n)))


def block_cholesky_solve(S: np.ndarray, n: int, N: int, rhs: np.ndarray) -> np.ndarray:
    """FP64 solve of S x = rhs for a symmetric positive definite block-tridiagonal S
    given in cbtd layout: S = L L^T with L block lower bidiagonal."""
    lo, di, _ = unpack_cbtd(S, n, N)
    g = np.asarray(rhs, dtype=np.float64).reshape(N, n)
    Lkk = [None] * N
    Lsub = [None] * N
    y = np.zeros((N, n))
    for k in range(N):
        Dk = di[k].copy()
        if k > 0:
            Lsub[k] = np.linalg.solve(Lkk[k - 1], lo[k].T).T   # L_{k,k-1} = S_{k,k-1} L_{k-1}^-T
            Dk -= Lsub[k] @ Lsub[k].T
        Lkk[k] = np.linalg.cholesky(0.5 * (Dk + Dk.T))
        b = g[k] - (Lsub[k] @ y[k - 1] if k > 0 else 0.0)
        y[k] = np.linalg.solve(Lkk[k], b)
    x = np.zeros((N, n))
    for k in range(N - 1, -1, -1):
        b = y[k] - (Lsub[k + 1].T @ x[k + 1] if k + 1 < N else 0.0)
        x[k] = np.linalg.solve(Lkk[k].T, b)
    return x.reshape(-1)


def matvec64(S: np.ndarray, x: np.ndarray, n: int, N: int) -> np.ndarray:
    """S x in FP64 for cbtd S (numpy, vectorised over knots)."""
    lo, di, up = unpack_cbtd(S, n, N)
    X = np.asarray(x, dtype=np.float64).reshape(N, n)
    y = np.einsum("kij,kj->ki", di, X)
    if N > 1:
        y[1:] += np.einsum("kij,kj->ki", lo[1:], X[:-1])
        y[:-1] += np.einsum("kij,kj->ki", up[:-1], X[1:])
    return y.reshape(-1)


def relres(S, lam, gamma, n, N) -> float:
    g = np.asarray(gamma, dtype=np.float64)
    return float(np.linalg.norm(g - matvec64(S, lam, n, N)) / max(np.linalg.norm(g), 1e-300))


# ------------------------------------------------------------------ reference example data
# ---- trajectory-optimisation problem around the solve (FP64 numpy references
# of csrc/kkt.cu's formation and back-substitution)

def generate_problem(n: int, N: int, seed: int, ill: bool = False):
    """The data behind generate(n, N, seed): A, B, Q, R drawn exactly as there
    (same generator, same order), plus cost gradients q, r and constraint
    right-hand side c from a second stream.  Blocks as (N, rows, cols) arrays."""
    rng = np.random.default_rng(seed)
    m = max(1, n // 2)
    A = rng.standard_normal((N, n, n)) / np.sqrt(n)
    rho = np.max(np.abs(np.linalg.eigvals(A)), axis=1)
    A *= (0.98 / rho)[:, None, None]
    B = rng.standard_normal((N, n, m))
    if ill:
        Qd = np.exp(rng.uniform(np.log(1e-2), np.log(1e4), (N + 1, n)))
        Rd = np.exp(rng.uniform(np.log(1e-3), 0.0, (N, m)))
    else:
        Qd = rng.uniform(1.0, 10.0, (N + 1, n))
        Rd = rng.uniform(0.1, 1.0, (N, m))
    r2 = np.random.default_rng(seed + 1_000_003)
    return {"n": n, "m": m, "N": N, "A": A, "B": B, "Qd": Qd, "Rd": Rd,
            "q": r2.standard_normal((N + 1, n)), "r": r2.standard_normal((N, m)), "c": r2.standard_normal((N, n))}


def problem_device_layout(P, dtype=np.float64):
    """Flat arrays in the layout gbdpcg_form_schur / gbdpcg_kkt_backsub read
    (A_k, B_k column-major, knot-major)."""
    col = lambda M: np.ascontiguousarray(M.transpose(0, 2, 1)).reshape(-1).astype(dtype)
    return {"A": col(P["A"]), "B": col(P["B"]), "Qd": P["Qd"].reshape(-1).astype(dtype),
            "Rd": P["Rd"].reshape(-1).astype(dtype), "q": P["q"].reshape(-1).astype(dtype),
            "r": P["r"].reshape(-1).astype(dtype), "c": P["c"].reshape(-1).astype(dtype)}


def form_schur(P):
    """S = C Theta^-1 C^T (flat cbtd) and gamma = -(c + C Theta^-1 g), FP64."""
    A, B, n, N = P["A"], P["B"], P["n"], P["N"]
    Qi, Ri = 1.0 / P["Qd"], 1.0 / P["Rd"]
    D = np.einsum("kij,kj,klj->kil", A, Qi[:N], A) + np.einsum("kij,kj,klj->kil", B, Ri, B)
    D[:, np.arange(n), np.arange(n)] += Qi[1:]
    D = 0.5 * (D + D.transpose(0, 2, 1))
    O = -(Qi[1:N][:, :, None] * A[1:].transpose(0, 2, 1))
    gamma = -(P["c"] + np.einsum("kij,kj->ki", A, Qi[:N] * P["q"][:N])
              + np.einsum("kij,kj->ki", B, Ri * P["r"]) - Qi[1:] * P["q"][1:])
    return pack_cbtd(D, O), gamma.reshape(-1)


def kkt_backsub(P, lam):
    """z = -Theta^-1 (g + C^T lambda): x (N+1, n), u (N, m), FP64."""
    A, B, N = P["A"], P["B"], P["N"]
    L = np.asarray(lam, np.float64).reshape(N, -1)
    sx = P["q"].copy()
    sx[:N] += np.einsum("kji,kj->ki", A, L)
    sx[1:] -= L
    su = P["r"] + np.einsum("kji,kj->ki", B, L)
    return -sx / P["Qd"], -su / P["Rd"]


def kkt_dense(P):
    """The full KKT matrix [Theta C^T; C 0] and right-hand side [-g; c] (dense,
    FP64), variables ordered (x_0..x_N, u_0..u_{N-1}, lambda_0..lambda_{N-1})."""
    n, m, N = P["n"], P["m"], P["N"]
    nz = n * (N + 1) + m * N
    C = np.zeros((n * N, nz))
    for k in range(N):
        C[k * n:(k + 1) * n, k * n:(k + 1) * n] = P["A"][k]
        C[k * n:(k + 1) * n, n * (N + 1) + k * m:n * (N + 1) + (k + 1) * m] = P["B"][k]
        C[k * n:(k + 1) * n, (k + 1) * n:(k + 2) * n] = -np.eye(n)
    Th = np.diag(np.concatenate([P["Qd"].reshape(-1), P["Rd"].reshape(-1)]))
    K = np.block([[Th, C.T], [C, np.zeros((n * N, n * N))]])
    g = np.concatenate([P["q"].reshape(-1), P["r"].reshape(-1)])
    return K, np.concatenate([-g, P["c"].reshape(-1)])


def example_system(path: str | None = None):
    """The reference example's n=2, N=3 data (examples/pcg_solve.cu:14-31), read from
    the committed fixture tests/golden/example_n2_N3.json."""
    import json
    if path is None:
        path = os.path.join(os.path.dirname(HERE), "tests", "golden", "example_n2_N3.json")
    with open(path) as f:
        d = json.load(f)
    S = np.asarray(d["S"], dtype=np.float32)
    # examples/pcg_solve.cu:24-28: elementwise reciprocal of the non-zeros of S
    Pinv = np.where(S == 0, np.float32(0), np.float32(1) / np.where(S == 0, 1, S)).astype(np.float32)
    return dict(n=2, N=3, S=S, Pinv=Pinv, gamma=np.asarray(d["gamma"], dtype=np.float32),
                lambda0=np.zeros(6, dtype=np.float32))


# ---------------------------------------------------------------------------- C oracle
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(BUILD_DIR, "libpcg_oracle.so")
        if not os.path.exists(path):
            raise RuntimeError(f"oracle library missing: {path} (run oracle/build_oracle.py)")
        L = ctypes.CDLL(path)
        P, u32, f32, f64, ip = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_float, ctypes.c_double, ctypes.c_void_p
        L.oracle_ref_pcg_f32.argtypes = [P, P, P, P, u32, u32, u32, f32, ip]
        L.oracle_ref_pcg_f32.restype = u32
        L.oracle_ref_pcg_f64.argtypes = [P, P, P, P, u32, u32, u32, f64, ip]
        L.oracle_ref_pcg_f64.restype = u32
        for nm in ("oracle_pcg_f32", "oracle_pcg_f64", "oracle_pcg_cg1_f32", "oracle_pcg_cg1_f64"):
            getattr(L, nm).argtypes = [P, P, P, P, u32, u32, u32, f64, u32, ip, ip, ip]
            getattr(L, nm).restype = ctypes.c_int
        for nm in ("oracle_matvec_f32", "oracle_matvec_f64"):
            getattr(L, nm).argtypes = [P, P, P, u32, u32]
        L.oracle_pcg_batch.argtypes = [P, u32, ctypes.c_int, u32, ctypes.c_int]
        L.oracle_pcg_batch.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _dt(a):
    return np.float64 if np.asarray(a).dtype == np.float64 else np.float32


def ref_pcg(S, Pinv, gamma, lambda0, n, N, max_iter=25, tol=1e-6):
    """Restatement of the reference kernel (include/pcg.cuh:54-218), exact order.
    Returns (lambda, iters, max_iter_exit)."""
    dt = _dt(S)
    S, Pinv, gamma = (np.ascontiguousarray(a, dtype=dt) for a in (S, Pinv, gamma))
    lam = np.array(lambda0, dtype=dt, copy=True)
    mie = ctypes.c_int(0)
    fn = lib().oracle_ref_pcg_f64 if dt == np.float64 else lib().oracle_ref_pcg_f32
    it = fn(_ptr(S), _ptr(Pinv), _ptr(gamma), _ptr(lam), n, N, max_iter, tol, ctypes.byref(mie))
    return lam, int(it), int(mie.value)


def pcg(S, Pinv, gamma, lambda0, n, N, max_iter=200, tol=1e-6, flags=0):
    """Product-semantics PCG on the host (sequential dots).  Returns
    (lambda, iters, status, eta, rr) with rr = ||r||^2 of the recursive residual."""
    dt = _dt(S)
    S, Pinv, gamma = (np.ascontiguousarray(a, dtype=dt) for a in (S, Pinv, gamma))
    lam = np.array(lambda0, dtype=dt, copy=True)
    it, eta, rr = ctypes.c_uint32(0), ctypes.c_double(0), ctypes.c_double(0)
    fn = lib().oracle_pcg_f64 if dt == np.float64 else lib().oracle_pcg_f32
    st = fn(_ptr(S), _ptr(Pinv), _ptr(gamma), _ptr(lam), n, N, max_iter, tol, flags,
            ctypes.byref(it), ctypes.byref(eta), ctypes.byref(rr))
    return lam, int(it.value), int(st), float(eta.value), float(rr.value)


def pcg_single_reduction(S, Pinv, gamma, lambda0, n, N, max_iter=200, tol=1e-6, flags=0):
    """Single-reduction (Chronopoulos-Gear) PCG with compact block-diagonal Phi^-1.
    Returns (lambda, iters, status, eta, rr)."""
    dt = _dt(S)
    S, Pinv, gamma = (np.ascontiguousarray(a, dtype=dt) for a in (S, Pinv, gamma))
    lam = np.array(lambda0, dtype=dt, copy=True)
    it, eta, rr = ctypes.c_uint32(0), ctypes.c_double(0), ctypes.c_double(0)
    fn = lib().oracle_pcg_cg1_f64 if dt == np.float64 else lib().oracle_pcg_cg1_f32
    st = fn(_ptr(S), _ptr(Pinv), _ptr(gamma), _ptr(lam), n, N, max_iter, tol, flags,
            ctypes.byref(it), ctypes.byref(eta), ctypes.byref(rr))
    return lam, int(it.value), int(st), float(eta.value), float(rr.value)


class _OracleSystem(ctypes.Structure):
    _fields_ = [("S", ctypes.c_void_p), ("Pinv", ctypes.c_void_p), ("gamma", ctypes.c_void_p),
                ("lambda_", ctypes.c_void_p), ("n", ctypes.c_uint32), ("N", ctypes.c_uint32),
                ("max_iter", ctypes.c_uint32), ("tol", ctypes.c_double),
                ("iters", ctypes.c_uint32), ("status", ctypes.c_int)]


def pcg_batch(systems, flags=0, nthreads=None, max_iter=200, tol=1e-6, is_f64=False):
    """Host-core batched PCG over a worker pool.  `systems` is a list of dicts with
    S, Pinv, gamma, lambda (arrays of one dtype, lambda updated in place), n, N.
    Returns (iters, status) arrays and the number of threads used."""
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    arr = (_OracleSystem * len(systems))()
    for i, s in enumerate(systems):
        arr[i] = _OracleSystem(_ptr(s["S"]).value, _ptr(s["Pinv"]).value, _ptr(s["gamma"]).value,
                               _ptr(s["lambda"]).value, s["n"], s["N"], max_iter, tol, 0, 0)
    used = lib().oracle_pcg_batch(ctypes.cast(arr, ctypes.c_void_p), len(systems), int(is_f64),
                                  flags, nthreads)
    return (np.array([a.iters for a in arr]), np.array([a.status for a in arr]), used)


# --------------------------------------------------------------- rebuilt reference kernel
def ref_kernel_name(dtype: str, n: int, N: int) -> str:
    """Itanium mangling of pcg<T, n, N>(T*, T*, T*, T*, T*, T*, T*, T*, uint32_t*, bool*,
    uint32_t, T) (include/pcg.cuh:54-68)."""
    t = "d" if dtype == "f64" else "f"
    return f"_Z3pcgI{t}Lj{n}ELj{N}EEvPT_S1_S1_S1_S1_S1_S1_S1_PjPbjS0_"


def ref_cubin(dtype: str) -> str:
    return os.path.join(REF_DIR, f"ref_pcg_{dtype}.cubin")


def have_ref_kernel(dtype="f32", n=None, N=None) -> bool:
    if not os.path.exists(ref_cubin(dtype)):
        return False
    if not os.path.exists(os.path.join(BUILD_DIR, "libref_launcher.so")):
        return False
    return n is None or (n, N) in REF_SIZES[dtype]


_reflib = None


def ref_kernel_solve(S, Pinv, gamma, lambda0, n, N, max_iter=25, tol=1e-6, reps=1):
    """Run the reference kernel rebuilt for sm_103a on the GPU.  Returns
    (lambda, iters, max_iter_exit, per-launch device ms)."""
    global _reflib
    if _reflib is None:
        L = ctypes.CDLL(os.path.join(BUILD_DIR, "libref_launcher.so"))
        P, u32 = ctypes.c_void_p, ctypes.c_uint32
        L.refpcg_solve.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, u32, u32, P, P, P,
                                   P, u32, ctypes.c_double, ctypes.c_int, P, P, P, ctypes.c_char_p,
                                   ctypes.c_int]
        L.refpcg_solve.restype = ctypes.c_int
        _reflib = L
    dt = _dt(S)
    dts = "f64" if dt == np.float64 else "f32"
    if (n, N) not in REF_SIZES[dts]:
        raise ValueError(f"reference kernel not instantiated at {dts} n={n} N={N}")
    S, Pinv, gamma = (np.ascontiguousarray(a, dtype=dt) for a in (S, Pinv, gamma))
    lam = np.array(lambda0, dtype=dt, copy=True)
    it, mie = ctypes.c_uint32(0), ctypes.c_int(0)
    ms = np.zeros(max(reps, 1), dtype=np.float32)
    err = ctypes.create_string_buffer(512)
    rc = _reflib.refpcg_solve(ref_cubin(dts).encode(), ref_kernel_name(dts, n, N).encode(),
                              int(dt == np.float64), n, N, _ptr(S), _ptr(Pinv), _ptr(gamma), _ptr(lam),
                              max_iter, tol, reps, ctypes.byref(it), ctypes.byref(mie), _ptr(ms), err, 512)
    if rc != 0:
        raise RuntimeError(f"reference kernel launch failed: {err.value.decode()}")
    return lam, int(it.value), int(mie.value), ms
