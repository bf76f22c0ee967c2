"""The CLI front end without a device (ddevol_gb300/cli/tpgp_gb_cli.c).

Options are checked before the device is touched, as the reference CLI
checks them before it creates its CUDA context (engine/src/cli_rev.c:437-448,
then :476-485): usage, unknown options, an END that is not a whole number of
steps, a missing edges file and an unreadable restart record are reported
with exit status 2 on any machine.
Valid options, or a valid restart record (tests/golden/cli_ring16.tpgpck, the
reference CLI's own checkpoint), reach the device and then stop with the
library's message: there is no CPU path.
"""
import os
import subprocess

import pytest

from ddevol_gb300 import build as gbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CHECKPOINT = os.path.join(ROOT, "tests", "golden", "cli_ring16.tpgpck")


@pytest.fixture(scope="module")
def cli():
    gbuild.build()
    return gbuild.CLI


def run(cli, *args):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    return subprocess.run([cli, *args], capture_output=True, text=True, env=env, timeout=60)


def test_usage_and_option_errors(cli):
    done = run(cli, "--help")
    assert done.returncode == 0 and "Usage: tpgp_gb_cli" in done.stderr
    done = run(cli, "--bogus", "1")
    assert done.returncode == 2 and "Unknown option: --bogus" in done.stderr
    done = run(cli, "--dt")  # an option without its value
    assert done.returncode == 2 and "Usage" in done.stderr


def test_reference_cli_options(cli, tmp_path):
    """The reference CLI's other options: --backend cuda (its GPU backend's
    name) selects this device path and a CPU backend is refused; --threads is
    accepted; the MPFR-only modes are refused as a reference build without
    MPFR refuses them; a walltime stop needs a checkpoint path distinct from
    the CSV (cli_rev.c:426-431, 450-462)."""
    assert "No GB300 device" in run(cli, "--backend", "cuda", "--threads", "4").stderr
    for args, message in ((["--backend", "serial"], "device path only"),
                          (["--validated"], "needs MPFR"),
                          (["--residual-depth", "2"], "needs the MPFR"),
                          (["--max-fid-bound", "0.1"], "MPFR-enclosed"),
                          (["--walltime", "5"], "needs --checkpoint"),
                          (["--checkpoint", str(tmp_path / "a"), "--output", str(tmp_path / "a")],
                           "must differ from --output"),
                          (["--checkpoint-every", "0"], "Usage"),
                          (["--walltime", "-1"], "Usage")):
        done = run(cli, *args)
        assert done.returncode == 2 and message in done.stderr, (args, done.stderr)
    ok = run(cli, "--walltime", "5", "--checkpoint", str(tmp_path / "w.tpgpck"),
             "--checkpoint-seconds", "1")
    assert ok.returncode == 2 and "No GB300 device" in ok.stderr


def test_option_values_are_taken_whole(cli):
    """As the reference CLI parses them (cli_rev.c:133-149): a real must be a
    finite decimal with nothing after it, a count an unsigned decimal."""
    for args in (["--dt", "0.01x"], ["--dt", "nan"], ["--time", "inf"], ["--n", "-3"],
                 ["--n", "8.5"], ["--cap", ""], ["--threads", "0"], ["--exact-ledger", "2"],
                 ["--checkpoint-every", "ten"], ["--linear-size", "+4"]):
        done = run(cli, *args)
        assert done.returncode == 2 and "Usage" in done.stderr, args
    assert "No GB300 device" in run(cli, "--dt", "1e-2", "--time", "0.04", "--threads",
                                    "8", "--exact-ledger", "0").stderr


def test_argument_checks_come_before_the_device(cli):
    done = run(cli, "--dt", "0.03", "--time", "0.1")
    assert done.returncode == 2 and "whole number of --dt steps" in done.stderr
    done = run(cli, "--model", "edges", "--edges", os.path.join(ROOT, "no-such-file"), "--n", "4")
    assert done.returncode == 2 and "Usage" in done.stderr
    done = run(cli, "--threshold", "-1")
    assert done.returncode == 2 and "Usage" in done.stderr
    done = run(cli, "--initial", "sideways")
    assert done.returncode == 2 and "Usage" in done.stderr
    done = run(cli, "--restart", os.path.join(ROOT, "no-such-checkpoint"))
    assert done.returncode == 2 and "Cannot restart" in done.stderr


REST = ["--model", "edges", "--n", "16", "--initial", "local", "--dt", "0.01",
        "--threshold", "1e-6"]


def capped_record(tmp_path, cap):
    """The reference CLI's record with a term cap set (written by the library, host only)."""
    import ctypes as C

    from ddevol_gb300 import native
    lib = native.load()
    rec = native.GbCheckpoint()
    err = C.create_string_buffer(256)
    assert lib.tpgp_gb_checkpoint_load(CHECKPOINT.encode(), C.byref(rec), err, 256) == 0
    rec.max_terms = cap
    out = str(tmp_path / "capped.tpgpck")
    assert lib.tpgp_gb_checkpoint_write(out.encode(), C.byref(rec), err, 256) == 0, err.value
    lib.tpgp_gb_checkpoint_free(C.byref(rec))
    return out


def test_restart_options_must_match_the_record(cli, tmp_path):
    """cli_rev.c:365-399: options given again on a restart must equal the
    record's, except that the horizon may grow and the cap may be raised."""
    def restart(*extra, record=CHECKPOINT):
        return run(cli, "--restart", record, *extra)

    # the record: edges model, 16 spins, local X_0, dt 0.01, threshold 1e-6,
    # 20 steps, the reference CLI's default cap of 10^6 terms
    same = restart(*REST, "--time", "0.3")
    assert same.returncode == 2 and "No GB300 device" in same.stderr
    for bad in (["--dt", "0.02"], ["--threshold", "1e-5"], ["--initial", "global"],
                ["--n", "17"], ["--model", "ring"], ["--time", "0.1"], ["--cap", "1000"],  # a lower cap
                ["--drop-budget", "1"], ["--j2", "0.5"]):
        done = restart(*bad)
        assert done.returncode == 2 and "Cannot restart" in done.stderr, bad
    capped = capped_record(tmp_path, 5000)
    assert "No GB300 device" in restart("--cap", "9000", record=capped).stderr  # raised
    assert "No GB300 device" in restart("--cap", "5000", record=capped).stderr
    assert "Cannot restart" in restart("--cap", "4000", record=capped).stderr  # lowered
    assert "No GB300 device" in restart("--cap", "0", record=capped).stderr  # 0 lifts the cap


MODELS = {
    "ring_n6": [],
    "ring_n9": ["--model", "ring", "--n", "9"],
    "j1j2_n8": ["--model", "j1j2", "--n", "8"],
    "j1j2_n10_j2_0125": ["--model", "j1j2", "--n", "10", "--j2", "0.125"],
    "ising_n5": ["--model", "ising", "--n", "5"],
    "xy_n7": ["--model", "xy", "--n", "7"],
    "cubic_l3": ["--model", "cubic", "--linear-size", "3"],
    "cubic_l4": ["--model", "cubic", "--linear-size", "4"],
    "edges_ring16": ["--model", "edges", "--edges",
                     os.path.join(ROOT, "tests", "golden", "ring16.edges"), "--n", "16"],
}


@pytest.mark.parametrize("name", sorted(MODELS))
def test_models_build_the_reference_term_lists(cli, name):
    """Every model's term list (order, sites, labels, h bit for bit) as the
    reference CLI builds it (cli_rev.c:108-245), from the records of its own
    one-step runs (tests/golden/cli_terms.npz, made by make_cli.py)."""
    import numpy as np
    golden = np.load(os.path.join(ROOT, "tests", "golden", "cli_terms.npz"))
    done = run(cli, *MODELS[name], "--list-terms")
    assert done.returncode == 0, done.stderr
    rows = [line.split() for line in done.stdout.splitlines()]
    ijq = np.array([[int(x) for x in r[:4]] for r in rows], np.uint64).reshape(-1, 4)
    h = np.array([float.fromhex(r[4]) for r in rows], np.float64)
    assert np.array_equal(ijq, golden[name + "_ijq"])
    assert np.array_equal(h.view(np.uint64), golden[name + "_h"].view(np.uint64))


def test_valid_runs_need_the_device(cli):
    done = run(cli, "--model", "j1j2", "--n", "8", "--time", "0.02")
    assert done.returncode == 2 and "No GB300 device" in done.stderr
    assert done.stdout == ""  # no CSV header before the device exists
    # the reference CLI's checkpoint is read on the host, then the device is needed
    done = run(cli, "--restart", CHECKPOINT)
    assert done.returncode == 2 and "No GB300 device" in done.stderr
