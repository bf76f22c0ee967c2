"""One full Strang step of the 64-spin all-pairs ring from a mid-trajectory state.

The state (tests/golden/ring64_window.npz, step 311 of the benchmark
trajectory, 100,947 terms, 128-bit keys) is the benchmark's workload state;
the expected result is the reference engine's own tpgp_strang_step (12,096
rotations) from it (tests/golden/ring64_window_step.npz, made by
tests/golden/make_window.py).  Both step engines must reproduce it with the
exact ledger, everything bitwise, ledger included: the sorted per-rotation
kernels and the hash-table step (whose removed terms, about 1.7e8 in this
step, are logged, sorted per rotation and added in the reference's order;
rotation segments run far past one shared-memory chunk, so the merge rounds
run).  With the bound ledger: keys, values, FID and integer ledger fields
bitwise; removed-weight sums -- an upper bound of the exact sums, as the
reference's sequential upward sums are -- within a few ulps.
"""
import os

import numpy as np
import pytest

from ddevol_gb300 import hamiltonians as H
from ddevol_gb300.engine import GbLedger, options

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIELDS = [name for name, _ in GbLedger._fields_]


@pytest.mark.parametrize("exact_ledger,hash_exact", [(True, "1"), (True, "0"), (False, "1")])
def test_window_step_matches_reference_engine(engine, exact_ledger, hash_exact):
    z = np.load(os.path.join(GOLDEN, "ring64_window.npz"))
    want = np.load(os.path.join(GOLDEN, "ring64_window_step.npz"))
    os.environ["TPGP_GB_HASH_EXACT"] = hash_exact  # "0": exact-ledger steps on the sorted kernels
    try:
        m = engine.map(64, z["keys"], z["values"])
    finally:
        os.environ.pop("TPGP_GB_HASH_EXACT", None)
    st, fids, led, msg = m.evolve(H.ring_all_pairs(64), 0.005, 1,
                                  options(1e-5, exact_ledger=exact_ledger), GbLedger())
    assert st == 0, msg
    k, v = m.download()
    m.close()
    assert np.array_equal(k, want["keys"])
    assert np.array_equal(v.view(np.uint64), want["values"].view(np.uint64))
    assert np.array_equal(np.asarray(fids).view(np.uint64), want["fid_sum"].view(np.uint64))
    got = np.array([float(getattr(led, f)) for f in FIELDS])
    ref = want["ledger"]
    if exact_ledger:
        assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))
    else:
        for f in ("rotations", "removal_events", "peak_terms"):
            i = FIELDS.index(f)
            assert got[i] == ref[i], f
        for f in ("dropped_l1", "dropped_l2", "dropped_l2_squared"):
            i = FIELDS.index(f)
            assert abs(got[i] - ref[i]) <= 1e-11 * ref[i], f
