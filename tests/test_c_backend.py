"""The reference-facing branch backend driven from a C program.

``tests/c/branch_backend.c`` links ``libtpgp_gb300.so`` through
``include/tpgp_cuda_rev.h`` only, with the CPU oracle as the engine around it
(the oracle's branch hook calls ``tpgp_cuda_branches`` for every rotation, as
DDevol's engine calls its CUDA backend, engine/src/tpgp_rev.c:622-640).  The
program is compiled as strict C11 with every warning an error, the way the
reference compiles its own backend tests (engine/CMakeLists.txt:154-159).

* CPU: it compiles and links against the library, and with no device
  visible the library refuses to create a context, with a message, and the
  program exits 77 (the reference tests' skip code) -- no CPU substitute.
* GPU: the status contract, raw children bitwise equal to the oracle's for
  1-, 2-, 3- and 32-word keys, Strang trajectories with the GPU as branch
  backend bitwise equal (map and ledger) to the oracle's own, the same
  through the allocation-free entry point, and two threads on one context.
"""
import os
import subprocess

import pytest

from ddevol_gb300 import build as gbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SOURCE = os.path.join(ROOT, "tests", "c", "branch_backend.c")
ORACLE_DIR = os.path.join(ROOT, "oracle")


def compile_program(out_dir) -> str:
    lib = gbuild.build()
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    lib_dir, orc_dir = os.path.dirname(lib), os.path.join(ORACLE_DIR, "_build")
    exe = os.path.join(str(out_dir), "branch_backend")
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-Wpedantic", "-Werror",
           "-fno-fast-math", "-ffp-contract=off",
           "-I", os.path.join(ROOT, "include"), "-I", ORACLE_DIR,
           SOURCE, "-o", exe,
           "-L", lib_dir, "-ltpgp_gb300", "-L", orc_dir, "-lorc",
           f"-Wl,-rpath,{lib_dir}:{orc_dir}", "-lpthread", "-lm"]
    done = subprocess.run(cmd, capture_output=True, text=True)
    assert done.returncode == 0, done.stderr
    return exe


def test_compiles_and_refuses_without_a_device(tmp_path):
    exe = compile_program(tmp_path)
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    done = subprocess.run([exe], capture_output=True, text=True, env=env, timeout=120)
    assert done.returncode == 77, (done.returncode, done.stdout, done.stderr)
    assert "no CUDA device" in done.stdout and "no CPU substitute" in done.stdout
    forced = subprocess.run([exe, "--require-device"], capture_output=True, text=True, env=env,
                            timeout=120)
    assert forced.returncode == 1


@pytest.mark.gpu
def test_gpu_branch_backend_from_c(tmp_path):
    exe = compile_program(tmp_path)
    done = subprocess.run([exe, "--require-device"], capture_output=True, text=True, timeout=600)
    print(done.stdout)
    assert done.returncode == 0, (done.stdout, done.stderr)
    assert ", 0 failed" in done.stdout
