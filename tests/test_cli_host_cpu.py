"""The CLI's host logic end to end on the CPU (no GPU).

The CLI front end (ddevol_gb300/cli/tpgp_gb_cli.c) is linked here against
tests/c/oracle_engine.cpp -- the device-resident calls it makes, restated on
the CPU oracle (test infrastructure; bitwise the device engine, which the GPU
suite checks) -- and the library's host-only record code.  The CLI's own
logic is then checked against the reference CLI's behaviour:

* the CSV of the 16-spin ring (tests/golden/cli_ring16.csv, the reference
  CLI's own run): every reference column within 1e-12, fid, active and the
  drop columns bitwise (engine/src/compare_tables.cpp semantics);
* a restart continues bitwise (engine/tests/test_cli_restart_rev.cmake);
* a walltime pause checkpoints and exits 75, and resuming completes the run
  as if uninterrupted;
* a cap stop exits 1 with a record, and a restart with a raised cap
  continues to the uninterrupted run's final row;
* an existing CSV is never overwritten.
"""
import csv
import io
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
ARGS = ["--model", "edges", "--edges", os.path.join(GOLDEN, "ring16.edges"), "--n", "16",
        "--initial", "local", "--dt", "0.01", "--threshold", "1e-6"]
COMPARED = ["fid", "active", "l2_norm", "drop_l1", "drop_l2_sum", "drop_l2_squared",
            "arithmetic_l2", "pf_observable_bound", "total_observable_bound"]
BITWISE = ["fid", "active", "drop_l1", "drop_l2_sum", "drop_l2_squared", "arithmetic_l2"]


@pytest.fixture(scope="module")
def cli(tmp_path_factory):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    out = tmp_path_factory.mktemp("cli_host")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_include = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
    orc = os.path.join(ROOT, "oracle", "_build")
    objs = []
    for src, lang in (("ddevol_gb300/csrc/checkpoint.cu", "c++"),
                      ("tests/c/oracle_engine.cpp", "c++")):
        obj = str(out / (os.path.basename(src) + ".o"))
        subprocess.run(["g++", "-O2", "-std=c++17", "-x", lang, "-I", cuda_include, "-c",
                        os.path.join(ROOT, src), "-o", obj], check=True)
        objs.append(obj)
    exe = str(out / "tpgp_gb_cli_host")
    subprocess.run(["g++", "-O2", "-x", "c", "-std=c11", "-fno-fast-math", "-ffp-contract=off",
                    "-c", os.path.join(ROOT, "ddevol_gb300/cli/tpgp_gb_cli.c"), "-o",
                    exe + ".o"], check=True)
    subprocess.run(["g++", "-o", exe, exe + ".o", *objs, "-L", orc, "-lorc",
                    f"-Wl,-rpath,{orc}", "-lm"], check=True)
    return exe


def run(cli, *args, code=0):
    done = subprocess.run([cli, *args], capture_output=True, text=True, timeout=300)
    assert done.returncode == code, done.stderr[-2000:]
    return done


def table(path):
    with open(path) as f:
        rows = [line for line in f if not line.startswith("#")]
    return list(csv.DictReader(io.StringIO("".join(rows))))


def test_csv_matches_the_reference_cli(cli, tmp_path):
    out = tmp_path / "host.csv"
    run(cli, *ARGS, "--time", "0.2", "--output", str(out))
    ours, ref = table(out), table(os.path.join(GOLDEN, "cli_ring16.csv"))
    assert len(ours) == len(ref) == 21
    for a, b in zip(ours, ref):
        for col in COMPARED:
            assert abs(float(a[col]) - float(b[col])) <= 1e-12, (a["time"], col)
        for col in BITWISE:
            assert np.float64(a[col]).view(np.uint64) == np.float64(b[col]).view(np.uint64)


def final_row(path):
    row = table(path)[-1]
    return [row[c] for c in ["time"] + COMPARED]


def test_restart_pause_and_cap_stop(cli, tmp_path):
    full = tmp_path / "full.csv"
    run(cli, *ARGS, "--time", "0.2", "--output", str(full))
    # restart from a checkpoint half way
    ck = str(tmp_path / "half.tpgpck")
    run(cli, *ARGS, "--time", "0.1", "--checkpoint", ck, "--output", str(tmp_path / "a.csv"))
    rest = tmp_path / "rest.csv"
    run(cli, *ARGS, "--restart", ck, "--time", "0.2", "--output", str(rest))
    assert [final_row(full)] == [final_row(rest)]
    assert [list(r.values())[:10] for r in table(full)[10:]] == \
        [list(r.values())[:10] for r in table(rest)]
    # a walltime pause after the first row: record, exit 75; resuming completes
    wk = str(tmp_path / "wall.tpgpck")
    run(cli, *ARGS, "--time", "0.2", "--walltime", "1e-9", "--checkpoint", wk,
        "--output", str(tmp_path / "w.csv"), code=75)
    assert len(table(tmp_path / "w.csv")) == 1
    resumed = tmp_path / "w2.csv"
    run(cli, *ARGS, "--restart", wk, "--output", str(resumed))
    assert final_row(resumed) == final_row(full)
    # a cap stop: exit 1 with a record; a raised cap continues
    cc = str(tmp_path / "cap.tpgpck")
    stopped = run(cli, *ARGS, "--time", "0.2", "--cap", "500", "--checkpoint", cc,
                  "--output", str(tmp_path / "c.csv"), code=1)
    assert "rejected" in stopped.stderr
    raised = tmp_path / "c2.csv"
    run(cli, "--restart", cc, "--cap", "5000", "--output", str(raised))
    assert final_row(raised) == final_row(full)
    # lowering the cap on a restart is refused
    run(cli, "--restart", cc, "--cap", "100", "--output", str(tmp_path / "c3.csv"), code=2)
    # an existing CSV is never overwritten
    kept = full.read_text()
    refused = run(cli, *ARGS, "--time", "0.02", "--output", str(full), code=2)
    assert "File exists" in refused.stderr and full.read_text() == kept
