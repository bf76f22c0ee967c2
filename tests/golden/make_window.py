"""The 64-spin all-pairs ring window: a committed mid-trajectory state and the
reference engine's result of one full Strang step from it.

Files written next to this script:

* ``ring64_window.npz`` (``--state``, needs a GB300): the 64-spin periodic
  ring with all-pairs couplings d = 1/r^3 (chord), X_0, dt = 0.005,
  threshold 1e-5, evolved from X_0 by the device engine until the map holds
  at least 10^5 terms (step 311, 100,947 terms).  Keys and values do not
  depend on the ledger mode; the device trajectory is bitwise the
  reference's (tests/test_strang_gpu.py), so this is a reference state.
  The same file is the workload state of bench.py's ring64 lines (both
  arms start from it).
* ``ring64_window_step.npz`` (``--expect``, needs the reference checkout):
  one tpgp_strang_step (12,096 rotations) of the reference engine itself
  (DDevol engine/src/tpgp_rev.c, built by ``make -C oracle ref``) from that
  state: output keys, values, ledger (from a zero ledger), FID sum.

    python tests/golden/make_window.py --state      # on a machine with a GB300
    DDEVOL_REFERENCE=<checkout> make -C oracle ref
    python tests/golden/make_window.py --expect     # a few minutes on the CPU
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ddevol_gb300 import hamiltonians as H  # noqa: E402

STATE = os.path.join(HERE, "ring64_window.npz")
STEP = os.path.join(HERE, "ring64_window_step.npz")
N, DT, THRESHOLD, TARGET = 64, 0.005, 1e-5, 100_000


def make_state():
    from ddevol_gb300.engine import Engine, GbLedger, options
    terms = H.ring_all_pairs(N)
    eng = Engine(0)
    m = eng.map(N, *H.single_site_operator(N))
    opts, led, steps = options(THRESHOLD, exact_ledger=False), GbLedger(), 0
    while len(m) < TARGET:
        st, _, led, msg = m.evolve(terms, DT, 1, opts, led, record_fid=False)
        if st:
            raise RuntimeError(msg)
        steps += 1
    k, v = m.download()
    m.close()
    eng.close()
    np.savez_compressed(STATE, keys=k, values=v, steps=steps)
    print(f"{STATE}: step {steps}, {len(v)} terms")


def make_expect():
    from oracle.oracle import LedgerStruct, Reference
    z = np.load(STATE)
    fids = []
    ref = Reference()
    st, k, v, led = ref.strang_step(z["keys"], z["values"], N, H.ring_all_pairs(N), DT,
                                    threshold=THRESHOLD, threads=os.cpu_count() or 1, backend=2,
                                    on_step=lambda s, f, n: fids.append(f))
    assert st == 0
    ledger = np.array([float(getattr(led, f)) for f, _ in LedgerStruct._fields_], np.float64)
    np.savez_compressed(STEP, keys=k, values=v, ledger=ledger, fid_sum=np.array(fids))
    print(f"{STEP}: {len(z['values'])} -> {len(v)} terms, FID sum {fids[0]:.17g}")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--state", action="store_true")
    ap.add_argument("--expect", action="store_true")
    a = ap.parse_args()
    if a.state:
        make_state()
    if a.expect:
        make_expect()
