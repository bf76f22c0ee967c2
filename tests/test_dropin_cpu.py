"""The reference's own programs linked against libtpgp_gb300.so (CPU).

``make -C oracle dropin`` compiles, from the reference checkout's sources
unchanged, the reference CLI and its two CUDA-backend test programs
(engine/tests/test_cuda_rev.c, engine/tests/test_cuda_trajectory_rev.c) with
this library linked where the reference links engine/src/cuda_rev.cu.  That
they compile and link is the drop-in claim at the C level; here, without a
device, each must then refuse the GPU path loudly: the test programs exit 77
(their skip code) reporting a compiled backend, and the CLI's ``--backend
cuda`` fails instead of falling back to a CPU backend.  Needs the checkout
(DDEVOL_REFERENCE); the same checks with a device are made by
tests/c/branch_backend.c, which needs no reference sources.
"""
import os
import subprocess

import pytest

from ddevol_gb300 import build as gbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("DDEVOL_REFERENCE", "")
REF_DIR = os.path.join(ROOT, "oracle", "_ref")

pytestmark = pytest.mark.skipif(not (REF and os.path.isdir(os.path.join(REF, "engine"))),
                                reason="DDEVOL_REFERENCE does not name the reference checkout")


@pytest.fixture(scope="module")
def programs():
    gbuild.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin"], check=True,
                   capture_output=True)
    return {name: os.path.join(REF_DIR, name)
            for name in ("tpgp_rev_gb", "test_cuda_rev_gb", "test_cuda_trajectory_rev_gb",
                         "strang_backend_gb")}


def run(path, *args):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    return subprocess.run([path, *args], capture_output=True, text=True, env=env, timeout=120)


def test_reference_backend_tests_link_and_skip_without_device(programs):
    for name in ("test_cuda_rev_gb", "test_cuda_trajectory_rev_gb"):
        done = run(programs[name])
        assert done.returncode == 77, (name, done.stdout, done.stderr)
        assert "tpgp_cuda:" in done.stdout + done.stderr   # this library's message
    assert "compiled=1" in run(programs["test_cuda_rev_gb"]).stderr
    # with the device required, a missing device is a failure, not a skip
    assert run(programs["test_cuda_trajectory_rev_gb"], "--require-device").returncode == 1


def test_device_resident_backend_of_the_engine_map(programs, tmp_path):
    """tests/c/strang_backend.c: a Strang step of the reference engine's own
    tpgp_map through the device-resident ABI (the integration sketch, made
    real).  Linked against the library it refuses without a device; linked
    against tests/c/oracle_engine.cpp (the device calls restated on the
    oracle) it runs its 30-step comparison with the reference engine and
    finds map and ledger bitwise equal."""
    done = run(programs["strang_backend_gb"])
    assert done.returncode == 77 and "no CPU substitute" in done.stdout
    eng = os.path.join(REF, "engine")
    orc = os.path.join(ROOT, "oracle", "_build")
    objs = []
    for src in ("src/tpgp_rev.c", "src/metal_stub_rev.c", "cuda/stub_rev.c"):
        obj = str(tmp_path / (os.path.basename(src) + ".o"))
        subprocess.run(["gcc", "-O2", "-std=c17", "-fno-fast-math", "-ffp-contract=off",
                        "-fopenmp", "-I", os.path.join(eng, "include"), "-c",
                        os.path.join(eng, src), "-o", obj], check=True, capture_output=True)
        objs.append(obj)
    sb, oe = str(tmp_path / "sb.o"), str(tmp_path / "oe.o")
    subprocess.run(["gcc", "-O2", "-std=c17", "-Wall", "-Wextra", "-Werror", "-I",
                    os.path.join(eng, "include"), "-I", os.path.join(ROOT, "include"), "-c",
                    os.path.join(ROOT, "tests", "c", "strang_backend.c"), "-o", sb], check=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-c",
                    os.path.join(ROOT, "tests", "c", "oracle_engine.cpp"), "-o", oe], check=True)
    exe = str(tmp_path / "strang_backend_host")
    subprocess.run(["g++", "-fopenmp", "-o", exe, sb, oe, *objs, "-L", orc, "-lorc",
                    f"-Wl,-rpath,{orc}", "-lm", "-lpthread"], check=True)
    done = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert done.returncode == 0, done.stderr
    assert "bitwise the engine's" in done.stdout


def test_reference_cli_cuda_backend_has_no_cpu_fallback(programs):
    done = run(programs["tpgp_rev_gb"], "--model", "j1j2", "--n", "8", "--dt", "0.01", "--time",
               "0.02", "--threshold", "1e-6", "--cap", "100000", "--initial", "local",
               "--backend", "cuda")
    assert done.returncode != 0
    assert "tpgp_cuda:" in done.stderr + done.stdout
