"""The CLI front end on the device path (ddevol_gb300/cli/tpgp_gb_cli.c,
built by build()) against the reference CLI's own run, and its restart.

* CSV parity: the 16-spin J1-J2 ring (the benchmark's term list through the
  edges file), local X_0, dt = 0.01, 20 steps, threshold 1e-6, exact ledger:
  every column the reference computes without MPFR matches the reference
  CLI's CSV (tests/golden/cli_ring16.csv) within 1e-12 absolute, rows matched
  on time, as engine/src/compare_tables.cpp compares tables; fid, active and
  the drop columns are bitwise equal.
* Restart parity: 10 steps with a checkpoint, then --restart to 20 steps,
  gives bitwise the rows and the final map of an uninterrupted 20-step run
  (the reference's engine/tests/test_cli_restart_rev.cmake check).
"""
import csv
import io
import os
import subprocess

import numpy as np
import pytest

from ddevol_gb300 import build

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
ARGS = ["--model", "edges", "--edges", os.path.join(GOLDEN, "ring16.edges"), "--n", "16",
        "--initial", "local", "--dt", "0.01", "--threshold", "1e-6", "--cap", "1000000"]
COMPARED = ["fid", "active", "l2_norm", "drop_l1", "drop_l2_sum", "drop_l2_squared",
            "arithmetic_l2", "pf_observable_bound", "total_observable_bound"]
BITWISE = ["fid", "active", "drop_l1", "drop_l2_sum", "drop_l2_squared", "arithmetic_l2"]


def table(path):
    with open(path) as f:
        rows = [line for line in f if not line.startswith("#")]
    return list(csv.DictReader(io.StringIO("".join(rows))))


def run(*extra):
    cli = build.build_cli()
    r = subprocess.run([cli, *ARGS, *extra], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return r


def test_csv_matches_the_reference_cli(tmp_path):
    out = tmp_path / "gb.csv"
    run("--time", "0.2", "--output", str(out))
    ours, ref = table(out), table(os.path.join(GOLDEN, "cli_ring16.csv"))
    assert len(ours) == len(ref) == 21
    for a, b in zip(ours, ref):
        assert abs(float(a["time"]) - float(b["time"])) <= 1e-12
        for col in COMPARED:
            assert abs(float(a[col]) - float(b[col])) <= 1e-12, (a["time"], col, a[col], b[col])
        for col in BITWISE:
            assert np.float64(a[col]).view(np.uint64) == np.float64(b[col]).view(np.uint64), \
                (a["time"], col)


def test_restart_continues_bitwise(tmp_path):
    full, part, rest = tmp_path / "full.csv", tmp_path / "part.csv", tmp_path / "rest.csv"
    ck_full, ck = str(tmp_path / "full.tpgpck"), str(tmp_path / "run.tpgpck")
    run("--time", "0.2", "--output", str(full), "--checkpoint", ck_full)
    run("--time", "0.1", "--output", str(part), "--checkpoint", ck)
    run("--restart", ck, "--time", "0.2", "--output", str(rest))
    a, b = table(full), table(rest)
    assert len(b) == 11  # steps 10..20
    for ra, rb in zip(a[10:], b):
        for col in ["time"] + COMPARED:
            assert ra[col] == rb[col], (ra["time"], col)
    # the final records hold the same map and ledger
    import ctypes as C

    from ddevol_gb300 import native
    lib = native.load()
    recs = []
    for path in (ck_full, ck):
        rec = native.GbCheckpoint()
        err = C.create_string_buffer(256)
        assert lib.tpgp_gb_checkpoint_load(path.encode(), C.byref(rec), err, 256) == 0, err.value
        recs.append(rec)
    x, y = recs
    assert x.step == y.step == 20 and x.len == y.len
    assert np.array_equal(np.ctypeslib.as_array(x.keys, (x.len,)), np.ctypeslib.as_array(y.keys, (y.len,)))
    assert np.array_equal(np.ctypeslib.as_array(x.values, (x.len,)).view(np.uint64),
                          np.ctypeslib.as_array(y.values, (y.len,)).view(np.uint64))
    assert x.ledger.rotations == y.ledger.rotations and x.pf_bound == y.pf_bound
    for rec in recs:
        lib.tpgp_gb_checkpoint_free(C.byref(rec))
