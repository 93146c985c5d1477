"""CPU tests of the oracle (test infrastructure): generator, layout helpers,
block-Jacobi, block Cholesky, and the C restatement of the reference PCG
pinned to golden vectors."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_example_fixture_matches_reference_source(oracle_mod):
    ex = oracle_mod.example_system()
    assert ex["S"].size == 36 and ex["gamma"].size == 6
    # the padding blocks of the example are zero (examples/pcg_solve.cu:14,22)
    assert not ex["S"][:4].any() and not ex["S"][-4:].any()


def test_ref_oracle_example(oracle_mod):
    O = oracle_mod
    ex = O.example_system()
    lam, it, mie = O.ref_pcg(ex["S"], ex["Pinv"], ex["gamma"], ex["lambda0"], 2, 3)
    assert it == 10 and mie == 0


def _golden():
    path = os.path.join(HERE, "golden", "ref_outputs.json")
    if not os.path.exists(path):
        pytest.skip("golden reference outputs not generated")
    with open(path) as f:
        return json.load(f)


def test_ref_oracle_matches_rebuilt_reference_outputs(oracle_mod):
    """Outputs of the reference kernel rebuilt for sm_103a (committed golden
    vectors) equal the CPU restatement bit for bit."""
    O = oracle_mod
    for case in _golden():
        dt = np.float64 if case["dtype"] == "f64" else np.float32
        n, N = case["n"], case["N"]
        if case["case"] == "example":
            ex = O.example_system()
            S, P, g = ex["S"], ex["Pinv"], ex["gamma"]
        else:
            S, P, g = O.golden_case(n, N, case["seed"], dt)
            assert O.digest(S, P, g) == case["input_digest"], case["case"]
        lam, it, mie = O.ref_pcg(S, P, g, np.zeros(n * N, dt), n, N, case["max_iter"], case["tol"])
        assert it == case["iters"] and mie == case["max_iter_exit"], case["case"]
        assert lam.tobytes().hex() == case["lam_hex"], case["case"]


def test_generator_structure(oracle_mod):
    O = oracle_mod
    sy = O.generate(14, 32, 0)
    S = sy.cbtd()
    A = O.dense_from_cbtd(S, 14, 32)
    assert np.allclose(A, A.T, atol=1e-12)
    ev = np.linalg.eigvalsh(A)
    assert ev[0] > 0
    lo, di, up = O.unpack_cbtd(S, 14, 32)
    assert not lo[0].any() and not up[-1].any()
    assert np.array_equal(O.pack_cbtd(sy.D, sy.O), S)


def test_mixed_generator_sizes(oracle_mod):
    ns, Ns = set(), []
    for seed in range(200):
        s = oracle_mod.generate_mixed(seed)
        ns.add(s.n)
        Ns.append(s.N)
    assert ns == {6, 12, 14, 24}
    assert min(Ns) >= 16 and max(Ns) <= 128


def test_block_cholesky_vs_dense(oracle_mod):
    O = oracle_mod
    for n, N, ill in ((14, 32, False), (6, 9, False), (24, 20, True), (3, 1, False)):
        sy = O.generate(n, N, 1, ill=ill)
        S = sy.cbtd()
        x = O.block_cholesky_solve(S, n, N, sy.gamma)
        xd = np.linalg.solve(O.dense_from_cbtd(S, n, N), sy.gamma)
        assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < (1e-7 if ill else 1e-12)


def test_block_jacobi_inverts_diagonal_blocks(oracle_mod):
    O = oracle_mod
    sy = O.generate(12, 10, 2)
    Pc = O.block_jacobi(sy.D, "compact").reshape(10, 12, 12)   # column-major blocks
    for k in range(10):
        assert np.allclose(Pc[k].T @ sy.D[k], np.eye(12), atol=1e-10)
    Pt = O.block_jacobi(sy.D, "cbtd")
    lo, di, up = O.unpack_cbtd(Pt, 12, 10)
    assert not lo.any() and not up.any()
    assert np.allclose(di, Pc.transpose(0, 2, 1))


@pytest.mark.parametrize("n,N", [(14, 32), (6, 64), (24, 40)])
def test_product_oracle_agrees_with_ref_restatement(oracle_mod, n, N):
    """The product-semantics PCG (sequential dots, compact Phi^-1) and the exact
    restatement take the same number of passes and agree to FP32 accuracy."""
    O = oracle_mod
    sy = O.generate(n, N, 0)
    S = sy.cbtd(np.float32)
    g = sy.gamma.astype(np.float32)
    lam_r, it_r, _ = O.ref_pcg(S, O.block_jacobi(sy.D).astype(np.float32), g, np.zeros(n * N, np.float32),
                               n, N, 200, 1e-6)
    lam_p, it_p, st, _, _ = O.pcg(S, O.block_jacobi(sy.D, "compact").astype(np.float32), g,
                                  np.zeros(n * N, np.float32), n, N, 200, 1e-6, flags=O.PINV_BLOCKDIAG)
    assert it_r == it_p and st == O.CONVERGED
    assert np.linalg.norm(lam_p - lam_r) / np.linalg.norm(lam_r) < 1e-5


def test_relres_mode_reaches_tolerance_fp64(oracle_mod):
    O = oracle_mod
    n, N = 14, 64
    sy = O.generate(n, N, 3)
    S = sy.cbtd()
    lam, it, st, eta, rr = O.pcg(S, O.block_jacobi(sy.D, "compact"), sy.gamma, np.zeros(n * N), n, N,
                                 500, 1e-10, flags=O.PINV_BLOCKDIAG | O.EXIT_RELRES)
    assert st == O.CONVERGED
    assert O.relres(S, lam, sy.gamma, n, N) < 2e-10
    x = O.block_cholesky_solve(S, n, N, sy.gamma)
    assert np.linalg.norm(lam - x) / np.linalg.norm(x) < 1e-8


def test_batch_worker_pool_matches_serial(oracle_mod):
    O = oracle_mod
    systems, serial = [], []
    for seed in range(12):
        s = O.generate_mixed(seed)
        S = s.cbtd(np.float32)
        P = O.block_jacobi(s.D, "compact").astype(np.float32)
        g = s.gamma.astype(np.float32)
        systems.append(dict(S=S, Pinv=P, gamma=g, **{"lambda": np.zeros(s.n * s.N, np.float32)}, n=s.n, N=s.N))
        serial.append(O.pcg(S, P, g, np.zeros(s.n * s.N, np.float32), s.n, s.N, 200, 1e-6,
                            flags=O.PINV_BLOCKDIAG | O.EXIT_RELRES))
    iters, status, used = O.pcg_batch(systems, flags=O.PINV_BLOCKDIAG | O.EXIT_RELRES, nthreads=4)
    assert used == 4
    for s, it, st, ref in zip(systems, iters, status, serial):
        assert it == ref[1] and st == ref[2]
        assert s["lambda"].tobytes() == ref[0].tobytes()


def test_ref_kernel_mangled_names(oracle_mod):
    """The launcher looks the rebuilt kernel up by its Itanium-mangled name."""
    assert oracle_mod.ref_kernel_name("f32", 14, 32) == "_Z3pcgIfLj14ELj32EEvPT_S1_S1_S1_S1_S1_S1_S1_PjPbjS0_"
    assert oracle_mod.ref_kernel_name("f64", 2, 3) == "_Z3pcgIdLj2ELj3EEvPT_S1_S1_S1_S1_S1_S1_S1_PjPbjS0_"


@pytest.mark.parametrize("n,N", [(6, 5), (14, 8), (7, 1)])
def test_kkt_formation_and_backsub_solve_the_kkt_system(oracle_mod, n, N):
    """The FP64 references of the steps around the solve: the Schur complement
    equals the generator's S for the same seed, and form -> solve -> back-
    substitute satisfies the dense KKT system."""
    O = oracle_mod
    P = O.generate_problem(n, N, 4)
    S, gamma = O.form_schur(P)
    assert np.allclose(S, O.generate(n, N, 4).cbtd(), rtol=0, atol=1e-12)
    lam = np.linalg.solve(O.dense_from_cbtd(S, n, N), gamma)
    x, u = O.kkt_backsub(P, lam)
    K, rhs = O.kkt_dense(P)
    sol = np.concatenate([x.reshape(-1), u.reshape(-1), lam])
    assert np.linalg.norm(K @ sol - rhs) <= 1e-10 * np.linalg.norm(rhs)
