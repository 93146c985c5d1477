"""Build recipe of the GB300 PCG library: every translation unit of csrc/ is
compiled for sm_103a in parallel and linked into _build/libgbdpcg.so (CUDA
runtime linked statically; the library exports only the C ABI of
include/gbdpcg.h).

Usage: python gbd-pcg_gb300/build.py [--force] [-j N]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgbdpcg.so")
ARCH = ["-gencode=arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fvisibility=hidden",
         "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs + [os.path.join(ROOT, "include", "gbdpcg.h")]


def _run(cmd: list[str]) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    hdr_time = max(os.path.getmtime(h) for h in headers())
    cmds, objs = [], []
    for src in sources():
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(os.path.getmtime(src), hdr_time):
            cmds.append([nvcc(), *ARCH, *FLAGS, "-c", src, "-o", obj] + (["-Xptxas", "-v"] if verbose else []))
    jobs = jobs or max(1, min(len(cmds), os.cpu_count() or 1))
    logs = []
    if cmds:
        with ThreadPoolExecutor(max_workers=jobs) as ex:
            logs = list(ex.map(_run, cmds))
    if cmds or force or not os.path.exists(LIB):
        _run([nvcc(), *ARCH, "-shared", "-o", LIB, *objs])
    return "\n".join(logs)


if __name__ == "__main__":
    j = None
    if "-j" in sys.argv:
        j = int(sys.argv[sys.argv.index("-j") + 1])
    log = build(force="--force" in sys.argv, jobs=j, verbose="-v" in sys.argv)
    if log:
        print(log)
    print(LIB)
