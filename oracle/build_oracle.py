"""ORACLE build recipe — test infrastructure only.

  oracle/_build/libpcg_oracle.so     gcc, from oracle/pcg_oracle.c
  oracle/_build/libref_launcher.so   nvcc, from oracle/ref_launcher.cu (host code)
  oracle/_ref/ref_pcg_{f32,f64}.cubin
      nvcc, device-only, from oracle/ref_kernels.cu, which includes the
      reference's include/pcg.cuh from the reference checkout (directory
      GBDPCG_REFERENCE_DIR, else `reference` beside this repository); built
      only where that checkout exists (the cubins are architecture-neutral on the host side
      and are carried to machines that have no checkout).

Usage: python oracle/build_oracle.py [--force]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# the reference checkout: GBDPCG_REFERENCE_DIR, else a `reference` directory
# beside this repository's root
REFERENCE_DIR = os.environ.get("GBDPCG_REFERENCE_DIR") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference")
REFERENCE_INCLUDE = os.path.join(REFERENCE_DIR, "include")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _stale(out: str, srcs: list[str], force: bool) -> bool:
    if force or not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, quiet: bool = True) -> None:
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    src = os.path.join(HERE, "pcg_oracle.c")
    out = os.path.join(BUILD, "libpcg_oracle.so")
    if _stale(out, [src, os.path.join(HERE, "pcg_oracle.h")], force):
        jobs.append(["gcc", "-O3", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", src,
                     "-o", out, "-lpthread", "-lm"])
    src = os.path.join(HERE, "ref_launcher.cu")
    out = os.path.join(BUILD, "libref_launcher.so")
    if _stale(out, [src], force):
        jobs.append([_nvcc(), "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", ARCH,
                     src, "-o", out])
    if os.path.exists(os.path.join(REFERENCE_INCLUDE, "pcg.cuh")):
        os.makedirs(REF_OUT, exist_ok=True)
        src = os.path.join(HERE, "ref_kernels.cu")
        deps = [src, os.path.join(HERE, "glass", "glass.cuh")]
        for dt, extra in (("f32", []), ("f64", ["-DREF_PCG_DOUBLE"])):
            out = os.path.join(REF_OUT, f"ref_pcg_{dt}.cubin")
            if _stale(out, deps, force):
                jobs.append([_nvcc(), "-cubin", ARCH, "-O3", "-lineinfo", *extra,
                             "-I" + os.path.join(HERE, "glass"), "-I" + REFERENCE_INCLUDE,
                             src, "-o", out])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    if not quiet:
        print(f"oracle: {len(jobs)} build step(s)")


if __name__ == "__main__":
    build(force="--force" in sys.argv, quiet=False)
