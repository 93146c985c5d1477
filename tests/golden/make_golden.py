"""Writes the golden fixtures under tests/golden/.

  example_n2_N3.json   the input data of the reference's only example
                       (examples/pcg_solve.cu:14-31: S, gamma; lambda0 = 0;
                       Pinv is the elementwise reciprocal of S's non-zeros,
                       :24-28), parsed from the reference checkout.
  ref_outputs.json     outputs of the reference kernel rebuilt for sm_103a
                       (oracle/_ref, run through oracle/ref_launcher.cu) on the
                       example and on seeded generator systems whose inputs are
                       quantized to a 2^-20 grid (oracle.golden_case), so that
                       every machine regenerates the same input bits (the
                       recorded input_digest checks it).  Needs a GPU:
                       `python tests/golden/make_golden.py --ref-outputs OUT.json`.

Usage: python tests/golden/make_golden.py [--example] [--ref-outputs PATH]
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
# the reference checkout: GBDPCG_REFERENCE_DIR, else a `reference` directory
# beside this repository's root
REFERENCE_DIR = os.environ.get("GBDPCG_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")
EXAMPLE = os.path.join(REFERENCE_DIR, "examples", "pcg_solve.cu")


def _array(src: str, name: str) -> list[float]:
    m = re.search(r"\b" + name + r"\s*\[\s*\d+\s*\]\s*=\s*\{([^}]*)\}", src)
    if not m:
        raise ValueError(f"{name} not found")
    return [float(t) for t in m.group(1).replace("\n", " ").split(",") if t.strip()]


def make_example() -> None:
    with open(EXAMPLE) as f:
        src = f.read()
    out = {"source": "examples/pcg_solve.cu:14-31", "n": 2, "N": 3,
           "S": _array(src, "h_S"), "gamma": _array(src, "h_gamma"),
           "lambda0": _array(src, "h_lambda")}
    with open(os.path.join(HERE, "example_n2_N3.json"), "w") as f:
        json.dump(out, f, indent=1)


# cases run through the rebuilt reference: (dtype, n, N, seed, max_iter, tol)
REF_CASES = [("f32", 14, 32, 0, 200, 1e-6), ("f32", 14, 128, 0, 200, 1e-6), ("f32", 14, 64, 8, 200, 1e-6),
             ("f64", 14, 128, 0, 200, 1e-12), ("f64", 14, 32, 1, 200, 1e-12),
             ("f32", 6, 64, 2, 200, 1e-6), ("f32", 12, 64, 3, 200, 1e-6),
             ("f32", 24, 128, 4, 200, 1e-6), ("f32", 3, 5, 5, 50, 1e-6),
             ("f32", 5, 2, 6, 50, 1e-6), ("f64", 3, 5, 7, 50, 1e-12)]
# the larger single system n = 14, N = 128 on seeds 1..9 (seed 0 is above),
# FP32 to 1e-6 and FP64 to 1e-12
REF_CASES += [(dts, 14, 128, seed, 200, tol) for dts, tol in (("f32", 1e-6), ("f64", 1e-12))
              for seed in range(1, 10)]


def make_ref_outputs(path: str) -> None:
    import numpy as np
    sys.path.insert(0, ROOT)
    from oracle import oracle as O

    res = []
    ex = O.example_system()
    lam, it, mie, _ = O.ref_kernel_solve(ex["S"], ex["Pinv"], ex["gamma"], ex["lambda0"], 2, 3, 25, 1e-6)
    res.append(dict(case="example", dtype="f32", n=2, N=3, max_iter=25, tol=1e-6, iters=it,
                    max_iter_exit=mie, lam_hex=lam.tobytes().hex()))
    for dts, n, N, seed, mi, tol in REF_CASES:
        dt = np.float64 if dts == "f64" else np.float32
        S, P, g = O.golden_case(n, N, seed, dt)
        lam, it, mie, _ = O.ref_kernel_solve(S, P, g, np.zeros(n * N, dt), n, N, mi, tol)
        res.append(dict(case=f"gen_seed{seed}", dtype=dts, n=n, N=N, seed=seed, max_iter=mi, tol=tol,
                        input_digest=O.digest(S, P, g), iters=it, max_iter_exit=mie,
                        lam_hex=lam.tobytes().hex()))
    with open(path, "w") as f:
        json.dump(res, f, indent=1)


if __name__ == "__main__":
    if "--example" in sys.argv or len(sys.argv) == 1:
        make_example()
    if "--ref-outputs" in sys.argv:
        make_ref_outputs(sys.argv[sys.argv.index("--ref-outputs") + 1])
