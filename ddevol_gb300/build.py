"""Builds the sm_103a library ``ddevol_gb300/_native/libtpgp_gb300.so`` in-tree.

Translation units compiled in parallel with nvcc, then linked:

* ``csrc/branch_abi.cu`` -- the reference-compatible ``tpgp_cuda_*`` ABI;
* ``csrc/engine.cu``     -- the device-resident ``tpgp_gb_*`` ABI and kernels;
* ``csrc/serve.cu``      -- the serving loop;
* ``csrc/checkpoint.cu`` -- restart records in the reference's format;

then the CLI front end ``cli/tpgp_gb_cli.c`` (gcc) into ``_native/tpgp_gb_cli``.

Numerical flags follow the reference's contract for its CUDA backend
(DDevol engine/cuda/CMakeLists.txt:26-27): no FMA contraction, IEEE division
and square root, no flush-to-zero, host code without fast-math or FP
contraction.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_native")
LIB = os.path.join(OUT_DIR, "libtpgp_gb300.so")
UNITS = ["branch_abi.cu", "engine.cu", "serve.cu", "checkpoint.cu"]
CLI_SRC = os.path.join(HERE, "cli", "tpgp_gb_cli.c")
CLI = os.path.join(OUT_DIR, "tpgp_gb_cli")

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    "--fmad=false", "--ftz=false", "--prec-div=true", "--prec-sqrt=true",
    "-Xcompiler", "-fPIC,-fno-fast-math,-ffp-contract=off,-O2",
    "-Xptxas", "-warn-spills",
]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the GB300 library cannot be built")
    return path


def _sources():
    return [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(HERE), "include"))
    for d in deps:
        if os.path.isdir(d):
            if any(os.path.getmtime(os.path.join(d, f)) > t for f in os.listdir(d)):
                return True
        elif os.path.getmtime(d) > t:
            return True
    return False


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles the library (and the CLI) if any source is newer; returns the library."""
    if not force and not _stale():
        if not os.path.exists(CLI) or os.path.getmtime(CLI) < os.path.getmtime(CLI_SRC):
            build_cli()
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    compiler = nvcc()
    objs = []

    def compile_one(unit):
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OUT_DIR, unit.replace(".cu", ".o"))
        cmd = [compiler, *NVCC_FLAGS, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(_sources())) as pool:
        objs = list(pool.map(compile_one, _sources()))
    tmp = LIB + ".tmp"
    cmd = [compiler, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp, *objs,
           "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli()
    return LIB


def build_cli() -> str:
    """The CLI front end (C, links the library only through include/)."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the CLI")
    cmd = [cc, "-O2", "-std=c11", "-Wall", "-Wextra", "-fno-fast-math", "-ffp-contract=off",
           "-o", CLI, CLI_SRC, "-L" + OUT_DIR, "-ltpgp_gb300", "-Wl,-rpath,$ORIGIN", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{r.stdout}\n{r.stderr}")
    return CLI


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
