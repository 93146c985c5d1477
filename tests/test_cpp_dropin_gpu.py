"""The reference's C++ interface (include/gpu_pcg.cuh: solvePCG, pcg_solve,
pcg_config) compiled with g++ against libgbdpcg.so and run on the GPU: a
caller written for the reference gets the reference's iteration count and
lambda within the FP32 tolerance of the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(gb, out, defines=()):
    cuda = os.path.dirname(os.path.dirname(shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"))
    libdir = os.path.dirname(gb.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", *defines, "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "cpp", "dropin_example.cpp"),
           "-o", out, "-L" + libdir, "-lgbdpcg", "-Wl,-rpath," + libdir, "-L" + os.path.join(cuda, "lib64"),
           "-lcudart", "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    subprocess.run(cmd, check=True, capture_output=True)
    return out


@pytest.fixture(scope="module")
def exe(gb, tmp_path_factory):
    return _compile(gb, str(tmp_path_factory.mktemp("cpp") / "dropin"))


@pytest.fixture(scope="module")
def exe_plain(gb, tmp_path_factory):
    return _compile(gb, str(tmp_path_factory.mktemp("cpp") / "dropin_plain"),
                    ["-DGBDPCG_DROPIN_ALGORITHM=GBDPCG_ALGO_PLAIN"])


def _run(exe, tmp_path, n, N, S, P, g, max_iter, tol, csr=False):
    dt = S.dtype
    path = str(tmp_path / "in.bin")
    with open(path, "wb") as f:
        f.write(np.array([n, N, dt.itemsize, 2 if csr else int(P is not None)], np.uint32).tobytes())
        for a in (S, P, g, np.zeros(n * N, dt)):
            if a is not None:
                f.write(np.ascontiguousarray(a, dt).tobytes())
    out = subprocess.run([exe, path, str(max_iter), repr(tol)], check=True, capture_output=True, text=True).stdout
    lines = out.split()
    return int(lines[1]), np.frombuffer(bytes.fromhex(lines[2]), dt)


@pytest.mark.gpu
def test_example_through_cpp_interface(exe, exe_plain, gb, oracle_mod, handle, tmp_path):
    """The reference's own example (examples/pcg_solve.cu).  Its S is indefinite
    and its Phi^-1 an elementwise reciprocal, so the iterates depend on the
    summation order: the plain algorithm (the reference's order) reproduces the
    reference bit for bit; the default cluster solver reproduces itself."""
    O = oracle_mod
    ex = O.example_system()
    lam_o, it_o, _ = O.ref_pcg(ex["S"], ex["Pinv"], ex["gamma"], ex["lambda0"], 2, 3)
    it, lam = _run(exe_plain, tmp_path, 2, 3, ex["S"], ex["Pinv"], ex["gamma"], 25, 1e-6)
    assert it == it_o == 10 and lam.tobytes() == lam_o.tobytes()
    it, lam = _run(exe, tmp_path, 2, 3, ex["S"], ex["Pinv"], ex["gamma"], 25, 1e-6)
    lam_c = ex["lambda0"].copy()
    r = gb.solve(ex["S"], ex["Pinv"], ex["gamma"], lam_c, 2, 3, gb.config())
    assert it == r.iters and lam.tobytes() == lam_c.tobytes()


@pytest.mark.gpu
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_generated_through_cpp_interface(exe, oracle_mod, handle, tmp_path, dt):
    O = oracle_mod
    n, N = 14, 32
    sy = O.generate(n, N, 0)
    S, P, g = sy.cbtd(dt), O.block_jacobi(sy.D).astype(dt), sy.gamma.astype(dt)
    tol = 1e-6 if dt == np.float32 else 1e-12
    it, lam = _run(exe, tmp_path, n, N, S, P, g, 200, tol)
    lam_o, it_o, _ = O.ref_pcg(S, P, g, np.zeros(n * N, dt), n, N, 200, tol)
    assert it == it_o
    assert np.linalg.norm(lam - lam_o) / np.linalg.norm(lam_o) < (1e-5 if dt == np.float32 else 1e-12)
    # pcg_solve: no Pinv, block-Jacobi built on the GPU
    it2, lam2 = _run(exe, tmp_path, n, N, S, None, g, 200, tol)
    assert abs(it2 - it_o) <= 1
    assert O.relres(sy.cbtd(), lam2, sy.gamma, n, N) < (1e-3 if dt == np.float32 else 1e-7)


@pytest.mark.gpu
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_csr_overload_through_cpp_interface(exe, oracle_mod, handle, tmp_path, dt):
    """The reference's CSR overload of solvePCG (a stub that exits in the
    reference): S and Phi^-1 as csr_t give the bits of the same matrices passed
    in the cbtd layout."""
    O = oracle_mod
    n, N = 12, 40
    sy = O.generate(n, N, 3)
    S, P, g = sy.cbtd(dt), O.block_jacobi(sy.D).astype(dt), sy.gamma.astype(dt)
    tol = 1e-6 if dt == np.float32 else 1e-12
    it_c, lam_c = _run(exe, tmp_path, n, N, S, P, g, 200, tol)
    it_r, lam_r = _run(exe, tmp_path, n, N, S, P, g, 200, tol, csr=True)
    assert it_r == it_c and lam_r.tobytes() == lam_c.tobytes()


@pytest.mark.gpu
def test_not_converged_is_an_error_when_asked(gb, oracle_mod, handle, tmp_path):
    """Built with GBDPCG_ERROR_ON_MAX_ITER, a drop-in solve that stops at
    pcg_max_iter is the error GBDPCG_ERR_NOT_CONVERGED (printed, exit code 5,
    like gpuErrchk); without it the iteration count is returned as the
    reference returns it."""
    O = oracle_mod
    strict = _compile(gb, str(tmp_path / "dropin_strict"), ["-DGBDPCG_ERROR_ON_MAX_ITER"])
    n, N = 14, 32
    sy = O.generate(n, N, 0)
    S, P, g = sy.cbtd(np.float32), O.block_jacobi(sy.D).astype(np.float32), sy.gamma.astype(np.float32)
    path = str(tmp_path / "in.bin")
    with open(path, "wb") as f:
        f.write(np.array([n, N, 4, 1], np.uint32).tobytes())
        for a in (S, P, g, np.zeros(n * N, np.float32)):
            f.write(a.tobytes())
    r = subprocess.run([strict, path, "2", "1e-6"], capture_output=True, text=True)
    assert r.returncode == 5 and "not converged" in r.stderr, (r.returncode, r.stderr)
    r = subprocess.run([strict, path, "200", "1e-6"], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("iters "), r.stderr
