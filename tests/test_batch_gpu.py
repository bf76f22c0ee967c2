"""Batched maps (tpgp_gb_batch): every item equals the same solve run alone.

Items of different spin counts (one- and two-word keys), couplings and
thresholds are advanced together by one clustered launch per step; each
item's keys, values, per-step FID and ledger must equal those of
tpgp_gb_strang_step on that item alone, for every cluster size the
autotuner may pick.
"""
import numpy as np
import pytest

from ddevol_gb300 import hamiltonians as H
from ddevol_gb300.engine import Batch, GbLedger, options

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


@pytest.mark.parametrize("exact", [False, True])
def test_batch_matches_single_solves(engine, exact):
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
def test_batch_cluster_sizes_agree(engine, shape):
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
