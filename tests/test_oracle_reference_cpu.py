"""The oracle against the reference engine itself, live, on every workload family.

The committed fixtures (tests/golden/) pin the oracle on 117 rotations and
six trajectories.  Where the reference checkout is present (DDEVOL_REFERENCE),
this test compiles the reference engine from its own sources (``make -C
oracle ref``: engine/src/tpgp_rev.c) and runs it beside the oracle on the
term lists of every workload the device is checked on, bit for bit (keys,
values, every ledger field, status and FID sum after each step):

* the 16-spin J1-J2 ring from the sum of X (64-bit keys);
* a 4x4x4 [111] cubic lattice and powder items (cubic fragments of 8..64
  spins, field directions from the seeded sphere draw), 128-bit keys;
* serving requests (rings and chains of 16..96 spins with Gaussian disorder
  factors and their own thresholds), keys of 1..3 words;
* a 100-spin chain (four-word keys);
* the cap and removed-weight budget statuses mid-trajectory.

The device paths are checked against the oracle on the same families by the
GPU tests; this closes the chain from the device to the reference engine.
"""
import os
import subprocess

import numpy as np
import pytest

from ddevol_gb300 import hamiltonians as H

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("DDEVOL_REFERENCE", "")

pytestmark = pytest.mark.skipif(not (REF and os.path.isdir(os.path.join(REF, "engine"))),
                                reason="DDEVOL_REFERENCE does not name the reference checkout")


@pytest.fixture(scope="module")
def reference():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True,
                   capture_output=True)
    from oracle.oracle import Reference
    return Reference()


def same_run(oracle, reference, keys, values, n, terms, dt, threshold, steps, max_terms=0,
             max_drop_l2=0.0):
    fo, fr = [], []
    so, ko, vo, lo = oracle.strang_step(keys, values, n, terms, dt, threshold=threshold,
                                        max_terms=max_terms, max_drop_l2=max_drop_l2,
                                        steps=steps, on_step=lambda s, f, m: fo.append((f, m)))
    sr, kr, vr, lr = reference.strang_step(keys, values, n, terms, dt, threshold=threshold,
                                           max_terms=max_terms, max_drop_l2=max_drop_l2,
                                           steps=steps, on_step=lambda s, f, m: fr.append((f, m)))
    assert so == sr
    assert np.array_equal(np.asarray(fo), np.asarray(fr))
    assert np.array_equal(ko, kr)
    assert np.array_equal(vo.view(np.uint64), vr.view(np.uint64))
    assert lo.as_dict() == lr.as_dict()
    return so, len(vo)


def test_ring16_from_global_x(oracle, reference):
    st, n = same_run(oracle, reference, *H.global_x_operator(16), 16, H.ring_j1j2(16), 0.01,
                     1e-6, 12)
    assert st == 0 and n > 1000


def test_cubic_lattice_and_powder_items(oracle, reference):
    k0, v0 = H.single_site_operator(64)
    st, size = same_run(oracle, reference, k0, v0, 64, H.cubic_111(4), 0.005, 1e-5, 12)
    assert st == 0 and size > 1000
    rng = np.random.default_rng(7)
    directions = H.sphere_directions(512)
    for item in rng.choice(512, 6, replace=False):
        n = int(rng.integers(8, 65))
        terms = H.cubic_fragment(n, directions[item])
        k0, v0 = H.single_site_operator(n)
        assert same_run(oracle, reference, k0, v0, n, terms, 0.01, 1e-5, 8)[0] == 0


def test_serving_requests(oracle, reference):
    rng = np.random.default_rng(2024)
    widths = set()
    for _ in range(8):
        n, terms, threshold, _, dt = H.serving_request(rng)
        widths.add((n + 31) // 32)
        k0, v0 = H.global_x_operator(n)
        assert same_run(oracle, reference, k0, v0, n, terms, dt, threshold, 5)[0] == 0
    assert len(widths) >= 2


def test_four_word_keys(oracle, reference):
    terms = H.chain_all_pairs(100, cutoff=2)
    k0, v0 = H.single_site_operator(100, site=50)
    st, size = same_run(oracle, reference, k0, v0, 100, terms, 0.02, 1e-6, 12)
    assert st == 0 and size > 1000


def test_cap_and_budget_statuses(oracle, reference):
    terms = H.ring_j1j2(12)
    k0, v0 = H.global_x_operator(12)
    assert same_run(oracle, reference, k0, v0, 12, terms, 0.05, 1e-4, 6, max_terms=300)[0] == 3
    assert same_run(oracle, reference, k0, v0, 12, terms, 0.05, 1e-3, 6,
                    max_drop_l2=1e-3)[0] == 6
