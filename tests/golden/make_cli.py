"""Golden outputs of the reference CLI's time loop and checkpoint.

Runs the reference CLI (oracle/_ref/tpgp_rev, compiled from DDevol's
engine/src/cli_rev.c by `make -C oracle ref`) on the 16-spin J1-J2 ring of
the plain-method benchmark: the edges file below gives d' = 2d, so the CLI's
secular edge (ZZ d'/2, XX -d'/4, YY -d'/4, cli_rev.c:125-132) builds exactly
the benchmark's term list (ZZ d, XX -d/2, YY -d/2 for d = 1 and 1/8).  Local
X_0, dt = 0.01, 20 steps, threshold 1e-6, serial backend.  Writes:

* ring16.edges            -- the edge list;
* cli_ring16.csv          -- the CLI's CSV (comment lines kept);
* cli_ring16.tpgpck       -- its checkpoint after step 20 (version-2 record);
* cli_terms.npz           -- the term list the reference CLI builds for each of
                             its models (ring, j1j2, ising, xy, cubic, edges),
                             read back from the records of one-step runs: per
                             model `<name>_ijq` (i, j, qi, qj) and `<name>_h`.

    DDEVOL_REFERENCE=<checkout> make -C oracle ref
    python tests/golden/make_cli.py [--terms-only]
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CLI = os.path.join(ROOT, "oracle", "_ref", "tpgp_rev")
EDGES = os.path.join(HERE, "ring16.edges")
CSV = os.path.join(HERE, "cli_ring16.csv")
CKPT = os.path.join(HERE, "cli_ring16.tpgpck")
ARGS = ["--model", "edges", "--edges", EDGES, "--n", "16", "--initial", "local", "--dt", "0.01",
        "--time", "0.2", "--threshold", "1e-6"]


def write_edges():
    with open(EDGES, "w") as f:
        f.write("# 16-spin ring, J1 = 1, J2 = 1/8, as d' = 2d for the secular edge\n")
        for i in range(16):
            f.write(f"{i} {(i + 1) % 16} 2\n")
            f.write(f"{i} {(i + 2) % 16} 0.25\n")


MODELS = {
    "ring_n6": [],  # the CLI's defaults: ring, 6 spins
    "ring_n9": ["--model", "ring", "--n", "9"],
    "j1j2_n8": ["--model", "j1j2", "--n", "8"],
    "j1j2_n10_j2_0125": ["--model", "j1j2", "--n", "10", "--j2", "0.125"],
    "ising_n5": ["--model", "ising", "--n", "5"],
    "xy_n7": ["--model", "xy", "--n", "7"],
    "cubic_l3": ["--model", "cubic", "--linear-size", "3"],
    "cubic_l4": ["--model", "cubic", "--linear-size", "4"],
    "edges_ring16": ["--model", "edges", "--edges", EDGES, "--n", "16"],
}


def model_terms(tmp):
    """Each model's term list from the record of a one-step reference run
    (read with the GB300 library's record loader, which reads the
    reference's records byte for byte)."""
    import ctypes as C

    import numpy as np

    sys.path.insert(0, ROOT)
    from ddevol_gb300 import native
    lib = native.load()
    out = {}
    for name, args in MODELS.items():
        ck = os.path.join(tmp, name + ".tpgpck")
        subprocess.run([CLI, *args, "--dt", "0.01", "--time", "0.01", "--initial", "local",
                        "--threshold", "1e-4", "--backend", "serial",
                        "--output", os.path.join(tmp, name + ".csv"), "--checkpoint", ck],
                       check=True)
        rec = native.GbCheckpoint()
        err = C.create_string_buffer(256)
        assert lib.tpgp_gb_checkpoint_load(ck.encode(), C.byref(rec), err, 256) == 0, err.value
        terms = [rec.terms[k] for k in range(rec.term_count)]
        out[name + "_ijq"] = np.array([(t.i, t.j, t.qi, t.qj) for t in terms], np.uint64)
        out[name + "_h"] = np.array([t.h for t in terms], np.float64)
        lib.tpgp_gb_checkpoint_free(C.byref(rec))
    np.savez(os.path.join(HERE, "cli_terms.npz"), **out)


def main(argv):
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        model_terms(tmp)
    if "--terms-only" in argv:  # the CSV carries wall times: keep the committed one
        return 0
    write_edges()
    # the reference CLI refuses to overwrite an output or to reuse a locked record
    for p in (CSV, CKPT, CKPT + ".manifest.json", CKPT + ".lock"):
        if os.path.exists(p):
            os.remove(p)
    subprocess.run([CLI, *ARGS, "--backend", "serial", "--output", CSV, "--checkpoint", CKPT],
                   check=True)
    for p in (CKPT + ".manifest.json", CKPT + ".lock"):
        if os.path.exists(p):
            os.remove(p)
    print(open(CSV).read().splitlines()[-1])


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
