"""Batched maps (tpgp_gb_batch): every item equals the same solve run alone.

Items of different spin counts (one- and two-word keys), couplings and
thresholds are advanced together by one clustered launch per step; each
item's keys, values, per-step FID and ledger must equal those of
tpgp_gb_strang_step on that item alone, for every cluster size the
autotuner may pick.
"""
import os

import numpy as np
import pytest

from ddevol_gb300 import hamiltonians as H
from ddevol_gb300.engine import Batch, options

pytestmark = pytest.mark.gpu


def powder_items(count, seed=3):
    rng = np.random.default_rng(seed)
    dirs = H.sphere_directions(count, seed=seed)
    items = []
    for k in range(count):
        n = int(rng.integers(8, 25)) if k % 3 else int(rng.integers(33, 41))
        terms = H.cubic_fragment(n, dirs[k])
        thr = float(10.0 ** rng.uniform(-6, -4))
        items.append((n, terms, thr))
    return items


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.fixture
def smem_off():
    """Batches created inside run every item on the clustered sorted path."""
    os.environ["TPGP_GB_BATCH_SMEM"] = "0"
    yield
    os.environ.pop("TPGP_GB_BATCH_SMEM", None)


@pytest.mark.parametrize("path", ["auto", "clustered"])
@pytest.mark.parametrize("exact", [False, True])
def test_batch_matches_single_solves(engine, exact, path, request):
    """Bound-ledger items run in CTA-local hash tables (auto), or all items on
    the clustered sorted path; exact-ledger items always take the latter."""
    if path == "clustered":
        request.getfixturevalue("smem_off")
    items = powder_items(12)
    steps, dt = 6, 0.02
    batch = Batch(engine, [n for n, _, _ in items])
    for k, (n, terms, thr) in enumerate(items):
        batch.upload(k, *H.single_site_operator(n, 0))
        batch.set_terms(k, terms, dt, options(thr, exact_ledger=exact))
    fids = batch.step(steps)
    for k, (n, terms, thr) in enumerate(items):
        assert batch.item_status(k) == 0
        m = engine.map(n, *H.single_site_operator(n, 0))
        st, f1, led1, msg = m.evolve(terms, dt, steps, options(thr, exact_ledger=exact))
        assert st == 0, msg
        k1, v1 = m.download()
        m.close()
        k2, v2 = batch.download(k)
        assert np.array_equal(k1, k2), k
        assert np.array_equal(bits(v1), bits(v2)), k
        assert np.array_equal(bits(f1), bits(fids[:, k])), k
        led2 = batch.ledger(k)
        assert led1.as_dict() == led2.as_dict(), k
    batch.close()


@pytest.mark.parametrize("shape", ["autotune", (1, 0), (2, 0), (4, 64), (8, 32), (1, 16)])
def test_batch_cluster_sizes_agree(engine, shape, smem_off):
    """Every cluster shape gives the single-solve result: autotuned base
    sizes, forced base sizes, and small terms-per-CTA so that the size rule
    puts the larger items on 8- and 16-CTA clusters."""
    items = powder_items(9, seed=5)
    dt = 0.02
    batch = Batch(engine, [n for n, _, _ in items])
    for k, (n, terms, thr) in enumerate(items):
        batch.upload(k, *H.single_site_operator(n, 0))
        batch.set_terms(k, terms, dt, options(thr, exact_ledger=False))
    if shape != "autotune":
        base, per_cta = shape
        for w in (1, 2):
            batch.set_cluster(w, min(base, batch.max_cluster(w)), per_cta)
    batch.step(3)
    if shape == "autotune":
        chosen = batch.autotune()
        assert chosen[1] in (1, 2, 4, 8)
        tuned = batch.tuning()[1]
        assert tuned["cluster"] == chosen[1]
        assert tuned["terms_per_cta"] in (4096, 8192, 16384)
        assert tuned["table_slots_per_claim"] in (2.0, 4.0)
    fids = batch.step(3)
    assert batch.max_cluster(1) in (8, 16)
    for k, (n, terms, thr) in enumerate(items):
        m = engine.map(n, *H.single_site_operator(n, 0))
        st, f1, _, msg = m.evolve(terms, dt, 6, options(thr, exact_ledger=False))
        assert st == 0, msg
        k1, v1 = m.download()
        m.close()
        k2, v2 = batch.download(k)
        assert np.array_equal(k1, k2) and np.array_equal(bits(v1), bits(v2)), k
        assert np.array_equal(bits(f1[3:]), bits(fids[:, k])), k
    batch.close()


def test_batch_item_failure_is_isolated(engine):
    items = powder_items(4, seed=7)
    dt = 0.02
    batch = Batch(engine, [n for n, _, _ in items])
    for k, (n, terms, thr) in enumerate(items):
        batch.upload(k, *H.single_site_operator(n, 0))
        # item 1 gets a cap it must exceed: it fails alone with ECAP
        batch.set_terms(k, terms, dt, options(thr, max_terms=3 if k == 1 else 0,
                                              exact_ledger=False))
    batch.step(2)
    assert batch.item_status(1) == 3
    k1, v1 = batch.download(1)
    assert len(v1) == 1  # still the initial operator
    for k in (0, 2, 3):
        assert batch.item_status(k) == 0 and batch.item_len(k) > 1
    batch.close()


def test_cta_table_overflow_falls_back(engine):
    """Items that outgrow their CTA-local table within a step (global X on
    eight spins, threshold 0: 8 terms to thousands) are re-run on the
    clustered path; results equal the single-map solve."""
    n, dt, steps = 8, 0.05, 3
    terms = H.ring_j1j2(n)
    batch = Batch(engine, [n, n, 20])
    k8, v8 = H.global_x_operator(n)
    batch.upload(0, k8, v8)
    batch.set_terms(0, terms, dt, options(0.0, exact_ledger=False))
    batch.upload(1, k8, v8)
    batch.set_terms(1, terms, dt, options(1e-3, exact_ledger=False))
    k20, v20 = H.single_site_operator(20, 0)
    batch.upload(2, k20, v20)
    batch.set_terms(2, H.ring_j1j2(20), dt, options(1e-5, exact_ledger=False))
    fids = batch.step(steps)
    for item, (nn, kk, vv, tt, thr) in enumerate([(n, k8, v8, terms, 0.0), (n, k8, v8, terms, 1e-3),
                                                   (20, k20, v20, H.ring_j1j2(20), 1e-5)]):
        assert batch.item_status(item) == 0
        m = engine.map(nn, kk, vv)
        st, f1, led1, msg = m.evolve(tt, dt, steps, options(thr, exact_ledger=False))
        assert st == 0, msg
        k1, v1 = m.download()
        m.close()
        k2, v2 = batch.download(item)
        assert np.array_equal(k1, k2) and np.array_equal(bits(v1), bits(v2)), item
        assert np.array_equal(bits(f1), bits(fids[:, item])), item
        assert led1.as_dict() == batch.ledger(item).as_dict(), item
    assert batch.item_len(0) > 4096
    batch.close()


@pytest.mark.parametrize("exact", [False, True])
def test_batch_items_match_oracle(engine, oracle, exact):
    """Each item against the CPU oracle (the reference algorithm) on its own
    inputs: powder items as the batched benchmark builds them -- cubic
    fragments of 8..64 spins (one- and two-word keys) whose couplings are
    rescaled by their own field direction, dt = 0.01, threshold 1e-5.  Keys,
    values and per-step FIDs bitwise; the ledger bitwise with the exact
    ledger; with the fixed-point ledger the removed-weight sums (an upper
    bound of the exact sums, like the reference's sequential upward sums)
    within a few ulps of the reference's."""
    sizes = [8, 13, 24, 31, 32, 33, 40, 50, 64, 64]
    dirs = H.sphere_directions(len(sizes), seed=20260711)
    items = [(n, H.cubic_fragment(n, d)) for n, d in zip(sizes, dirs)]
    steps, dt, thr = 6, 0.01, 1e-5
    batch = Batch(engine, [n for n, _ in items])
    for k, (n, terms) in enumerate(items):
        batch.upload(k, *H.single_site_operator(n, 0))
        batch.set_terms(k, terms, dt, options(thr, exact_ledger=exact))
    fids = batch.step(steps)
    for k, (n, terms) in enumerate(items):
        assert batch.item_status(k) == 0
        fo = []
        st, ok, ov, oled = oracle.strang_step(*H.single_site_operator(n, 0), n, terms, dt,
                                              threshold=thr, steps=steps,
                                              on_step=lambda s, f, nn: fo.append(f))
        assert st == 0
        kb, vb = batch.download(k)
        assert np.array_equal(kb, ok), k
        assert np.array_equal(bits(vb), bits(ov)), k
        assert np.array_equal(bits(fids[:, k]), bits(fo)), k
        led = batch.ledger(k)
        assert (led.rotations, led.removal_events, led.peak_terms) == \
            (oled.rotations, oled.removal_events, oled.peak_terms), k
        for f in ("dropped_l1", "dropped_l2", "dropped_l2_squared"):
            a, b = getattr(led, f), getattr(oled, f)
            if exact:
                assert bits([a]) == bits([b]), (k, f)
            else:  # both are upper bounds of the exact sum, a few ulps apart
                assert abs(a - b) <= 1e-11 * b, (k, f)
    batch.close()
