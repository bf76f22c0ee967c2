"""Helpers shared by the GPU parity tests (seeded random maps, comparisons)."""
import numpy as np

from ddevol_gb300.engine import GbLedger, options

LEDGER_FIELDS = [name for name, _ in GbLedger._fields_]


def ledger_vec(led):
    return np.array([float(getattr(led, f)) for f in LEDGER_FIELDS], np.float64)


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def sort_keys(keys, words):
    k = keys.reshape(-1, words)
    order = np.lexsort(tuple(k[:, w] for w in range(words)))
    return order


def random_map(rng, n_spins, count, active_sites=None, dense=False):
    """Distinct sorted keys and values spread over many decades.

    ``active_sites`` limits nonidentity symbols to those sites (keeps the key
    population realistic); ``dense`` draws every site.
    """
    words = (n_spins + 31) // 32
    sites = np.arange(n_spins) if active_sites is None else np.asarray(active_sites)
    raw = np.zeros((int(count * 1.3) + 16, words), np.uint64)
    for r in range(raw.shape[0]):
        if dense:
            chosen = sites
        else:
            chosen = rng.choice(sites, size=int(rng.integers(1, min(8, len(sites)) + 1)),
                                replace=False)
        for s in chosen:
            sym = int(rng.integers(0 if dense else 1, 4))
            raw[r, s // 32] |= np.uint64(sym) << np.uint64(2 * (s % 32))
    uniq = np.unique(raw, axis=0)
    if len(uniq) > count:
        uniq = uniq[rng.choice(len(uniq), count, replace=False)]
    order = np.lexsort(tuple(uniq[:, w] for w in range(words)))
    keys = np.ascontiguousarray(uniq[order]).reshape(-1)
    vals = rng.standard_normal(len(order)) * 10.0 ** rng.uniform(-7, 0, len(order))
    return keys, vals


def fast_random_map(rng, n_spins, count):
    """Large random maps quickly: random 64-bit words masked to the spin count."""
    words = (n_spins + 31) // 32
    raw = rng.integers(0, 2 ** 63, size=(int(count * 1.05) + 8, words), dtype=np.int64)
    raw = raw.astype(np.uint64) ^ (rng.integers(0, 2, size=raw.shape, dtype=np.int64).astype(
        np.uint64) << np.uint64(63))
    rem = n_spins % 32
    if rem:
        raw[:, -1] &= np.uint64((1 << (2 * rem)) - 1)
    uniq = np.unique(raw, axis=0)[:count]
    order = np.lexsort(tuple(uniq[:, w] for w in range(words)))
    keys = np.ascontiguousarray(uniq[order]).reshape(-1)
    vals = rng.standard_normal(len(order)) * 10.0 ** rng.uniform(-6, 0, len(order))
    return keys, vals


def gpu_rotate(engine, keys, vals, n_spins, i, j, qi, qj, theta, threshold=0.0, max_terms=0,
               max_drop_l2=0.0, exact_ledger=True):
    m = engine.map(n_spins, keys, vals)
    try:
        st, led, msg = m.rotate(i, j, qi, qj, theta,
                                options(threshold, max_terms, max_drop_l2, exact_ledger),
                                GbLedger())
        k, v = m.download()
    finally:
        m.close()
    return st, k, v, led, msg


def sparse_random_map(rng, n_spins, count, max_active=6):
    """Vectorised: each key has 1..max_active random non-identity sites."""
    words = (n_spins + 31) // 32
    rows = int(count * 1.2) + 16
    raw = np.zeros((rows, words), np.uint64)
    active = rng.integers(1, max_active + 1, rows)
    for c in range(max_active):
        use = active > c
        sites = rng.integers(0, n_spins, rows)
        syms = rng.integers(1, 4, rows).astype(np.uint64)
        word = sites // 32
        shift = (2 * (sites % 32)).astype(np.uint64)
        cleared = raw[np.arange(rows), word] & ~(np.uint64(3) << shift)
        newv = cleared | (syms << shift)
        raw[np.arange(rows)[use], word[use]] = newv[use]
    uniq = np.unique(raw, axis=0)
    if len(uniq) > count:
        uniq = uniq[np.sort(rng.choice(len(uniq), count, replace=False))]
    order = np.lexsort(tuple(uniq[:, w] for w in range(words)))
    keys = np.ascontiguousarray(uniq[order]).reshape(-1)
    vals = rng.standard_normal(len(order)) * 10.0 ** rng.uniform(-7, 0, len(order))
    return keys, vals
