"""Synthetic optimal-control workloads in the reference's data layout.

S = C Theta^-1 C^T with one block row [A_k  B_k  -I] of C per knot, acting on
(x_k, u_k, x_{k+1}); Theta = blockdiag(Q_0..Q_N, R_0..R_{N-1}).  Packed in the
compressed block-tridiagonal (cbtd) layout of the reference
(include/pcg.cuh:104-110, include/utils.cuh:62,71,80): per knot one n x 3n
column-major block row [S_{k,k-1} | S_{k,k} | S_{k,k+1}], element (r, c) at
k*3n^2 + c*n + r; the blocks S_{0,-1} and S_{N-1,N} are zero padding
(examples/pcg_solve.cu:14,22).  Pure numpy; used by the benchmark, the tests
and the oracle.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class System:
    n: int
    N: int
    D: np.ndarray      # (N, n, n) diagonal blocks S_kk, FP64
    O: np.ndarray      # (N-1, n, n) super-diagonal blocks S_{k,k+1}, FP64
    gamma: np.ndarray  # (n*N,) FP64
    seed: int = 0

    def cbtd(self, dtype=np.float64) -> np.ndarray:
        return pack_cbtd(self.D, self.O).astype(dtype)


def generate(n: int, N: int, seed: int, ill: bool = False, rng=None) -> System:
    """A_k ~ N(0, 1/n) rescaled to spectral radius 0.98, B_k ~ N(0, 1) (n x m,
    m = n/2), Q_k = diag U[1, 10] (k = 0..N), R_k = diag U[0.1, 1]; when `ill`,
    Q_k log-uniform in [1e-2, 1e4] and R_k log-uniform in [1e-3, 1].
      S_kk      = A_k Q_k^-1 A_k^T + B_k R_k^-1 B_k^T + Q_{k+1}^-1
      S_{k,k+1} = -Q_{k+1}^-1 A_{k+1}^T
    gamma ~ N(0, 1).  Draw order: A, B, Q, R, gamma from default_rng(seed)."""
    if rng is None:
        rng = np.random.default_rng(seed)
    m = max(1, n // 2)
    A = rng.standard_normal((N, n, n)) / np.sqrt(n)
    rho = np.max(np.abs(np.linalg.eigvals(A)), axis=1)
    A *= (0.98 / rho)[:, None, None]
    B = rng.standard_normal((N, n, m))
    if ill:
        Q = np.exp(rng.uniform(np.log(1e-2), np.log(1e4), (N + 1, n)))
        R = np.exp(rng.uniform(np.log(1e-3), 0.0, (N, m)))
    else:
        Q = rng.uniform(1.0, 10.0, (N + 1, n))
        R = rng.uniform(0.1, 1.0, (N, m))
    gamma = rng.standard_normal(n * N)
    Qi, Ri = 1.0 / Q, 1.0 / R
    D = np.einsum("kij,kj,klj->kil", A, Qi[:N], A) + np.einsum("kij,kj,klj->kil", B, Ri, B)
    D[:, np.arange(n), np.arange(n)] += Qi[1:]
    D = 0.5 * (D + D.transpose(0, 2, 1))
    O = -(Qi[1:N][:, :, None] * A[1:].transpose(0, 2, 1))
    return System(n, N, D, O, gamma, seed)


def mixed_size(seed: int, sizes=(6, 12, 14, 24), nmin=16, nmax=128):
    """(n, N) of generate_mixed(seed) without building the system (the same
    first two draws)."""
    rng = np.random.default_rng(seed)
    n = int(rng.choice(np.asarray(sizes)))
    N = int(rng.integers(nmin, nmax + 1))
    return n, N


def generate_mixed(seed: int, sizes=(6, 12, 14, 24), nmin=16, nmax=128) -> System:
    """One system of the mixed batch: n from `sizes`, N uniform in [nmin, nmax],
    then the generator above, all from default_rng(seed)."""
    rng = np.random.default_rng(seed)
    n = int(rng.choice(np.asarray(sizes)))
    N = int(rng.integers(nmin, nmax + 1))
    return generate(n, N, seed, rng=rng)


def pack_cbtd(D: np.ndarray, O: np.ndarray) -> np.ndarray:
    """(N, n, n) diagonal + (N-1, n, n) super-diagonal blocks -> flat cbtd array."""
    N, n, _ = D.shape
    Sc = np.zeros((N, 3 * n, n), dtype=np.float64)   # Sc[k, c, r] = block row k, (r, c)
    Sc[:, n:2 * n, :] = D.transpose(0, 2, 1)
    if N > 1:
        Sc[1:, 0:n, :] = O                              # S_{k,k-1} = O_{k-1}^T
        Sc[:-1, 2 * n:3 * n, :] = O.transpose(0, 2, 1)  # S_{k,k+1} = O_k
    return Sc.reshape(-1)


def _gen_mixed_packed(seed: int, dtype):
    s = generate_mixed(seed)
    return s.n, s.N, s.cbtd(dtype), s.gamma.astype(dtype)


def packed_batch(seeds, dtype=np.float32, workers: int = 1, pinv_layout: int = 1):
    """Mixed systems packed into arenas.  Returns (descs, S, gamma, Pinv_elems)
    with descs = [(n, N, S_off, Pinv_off, vec_off)] in element offsets, each
    system's S offset rounded up to 16 bytes (so bulk copies stay aligned).
    pinv_layout 1 = compact block-diagonal (n^2 per knot), 0 = cbtd."""
    seeds = list(seeds)
    if workers > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(workers) as pool:
            parts = pool.starmap(_gen_mixed_packed, [(s, dtype) for s in seeds], chunksize=16)
    else:
        parts = [_gen_mixed_packed(s, dtype) for s in seeds]
    align = 16 // np.dtype(dtype).itemsize
    descs, offS, offP, offV = [], 0, 0, 0
    for n, N, S, g in parts:
        descs.append((n, N, offS, offP, offV))
        offS += -(-S.size // align) * align
        pm = n * n * N if pinv_layout == 1 else 3 * n * n * N
        offP += -(-pm // align) * align
        offV += -(-g.size // align) * align
    Sa = np.zeros(offS, dtype)
    ga = np.zeros(offV, dtype)
    for (n, N, oS, oP, oV), (_, _, S, g) in zip(descs, parts):
        Sa[oS:oS + S.size] = S
        ga[oV:oV + g.size] = g
    return descs, Sa, ga, offP
