"""Golden outputs of the reference CLI's time loop and checkpoint.

Runs the reference CLI (oracle/_ref/tpgp_rev, compiled from DDevol's
engine/src/cli_rev.c by `make -C oracle ref`) on the 16-spin J1-J2 ring of
the plain-method benchmark: the edges file below gives d' = 2d, so the CLI's
secular edge (ZZ d'/2, XX -d'/4, YY -d'/4, cli_rev.c:125-132) builds exactly
the benchmark's term list (ZZ d, XX -d/2, YY -d/2 for d = 1 and 1/8).  Local
X_0, dt = 0.01, 20 steps, threshold 1e-6, serial backend.  Writes:

* ring16.edges            -- the edge list;
* cli_ring16.csv          -- the CLI's CSV (comment lines kept);
* cli_ring16.tpgpck       -- its checkpoint after step 20 (version-2 record).

    DDEVOL_REFERENCE=<checkout> make -C oracle ref
    python tests/golden/make_cli.py
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


def main():
    write_edges()
    for p in (CKPT, CKPT + ".manifest.json", CKPT + ".lock"):
        if os.path.exists(p):
            os.remove(p)
    subprocess.run([CLI, *ARGS, "--backend", "serial", "--output", CSV, "--checkpoint", CKPT],
                   check=True)
    for p in (CKPT + ".manifest.json", CKPT + ".lock"):
        if os.path.exists(p):
            os.remove(p)
    print(open(CSV).read().splitlines()[-1])


if __name__ == "__main__":
    sys.exit(main())
