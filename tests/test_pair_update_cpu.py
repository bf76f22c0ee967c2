"""The hash-table step's pair update, restated in Python, against the oracle.

The device hash-table step (csrc/hash_kernels.cuh) does not sort: for a
rotation by Q it pairs every anticommuting key K with K xor Q and sets

    new[K] = RN(RN(v_K c) + s_P RN(v_P s))      (both present)
    new[K] = RN(v_K c)                          (partner absent)
    new[P] = s_K RN(v_K s)                      (P absent: inserted)

keeps commuting keys (v + 0 = v), then drops exact zeros and removes
|v| <= threshold (identity exempt) -- commuting keys included.  This test
runs that rule with Python floats (binary64, round to nearest, no
contraction) on random maps, and requires bitwise the reference's
branch / stable sort / merge result from the oracle, on every generator
type and on maps holding sub-threshold values, the identity key and
commuting keys.  It is the CPU check of the claim that the sort-free
pair update is exact.
"""
import numpy as np
import pytest

from gpu_helpers import bits, random_map


def phase_of(q, p):
    if not q or not p or q == p:
        return 0
    return 1 if (q % 3) + 1 == p else 3


def anticommutes(q, p):
    return bool(q and p and q != p)


def key_ints(keys, words):
    k = np.asarray(keys, dtype=np.uint64).reshape(-1, words)
    return [sum(int(row[w]) << (64 * w) for w in range(words)) for row in k]


def pair_rotation(mapping, i, j, qi, qj, c, s, threshold):
    """One rotation by the pair rule.  mapping: {key int: value}, all nonzero."""
    Q = (qi << (2 * i)) ^ (qj << (2 * j))
    new = {}
    for K, v in mapping.items():
        pi, pj = (K >> (2 * i)) & 3, (K >> (2 * j)) & 3
        if anticommutes(qi, pi) == anticommutes(qj, pj):
            new[K] = v  # commuting: v + 0
            continue
        P = K ^ Q
        if P in mapping and P < K:
            continue  # the smaller key of a present pair updates both
        plus_k = (phase_of(qi, pi) + phase_of(qj, pj)) & 3 == 1
        sk = v * s if plus_k else -(v * s)
        nk, np_ = v * c, sk
        if P in mapping:
            vp = mapping[P]
            ppi, ppj = (P >> (2 * i)) & 3, (P >> (2 * j)) & 3
            plus_p = (phase_of(qi, ppi) + phase_of(qj, ppj)) & 3 == 1
            sp = vp * s if plus_p else -(vp * s)
            nk = nk + sp
            np_ = vp * c + sk
        new[K] = nk
        new[P] = np_
    kept, removed = {}, []
    for K, x in new.items():
        if x == 0.0:
            continue  # exact zero: dropped
        if K != 0 and abs(x) <= threshold:
            removed.append(abs(x))
            continue
        kept[K] = x
    return kept, removed


GENERATORS = [(3, 3), (1, 1), (2, 2), (1, 3), (2, 1), (3, 2), (0, 3)]


@pytest.mark.parametrize("n_spins", [12, 40])
def test_pair_update_matches_reference_merge(oracle, n_spins):
    rng = np.random.default_rng(1000 + n_spins)
    words = (n_spins + 31) // 32
    for trial in range(24):
        keys, vals = random_map(rng, n_spins, int(rng.integers(50, 1500)),
                                active_sites=range(min(n_spins, 10)))
        if trial % 3 == 0:  # the identity key is never removed by the threshold
            ks = key_ints(keys, words)
            if 0 not in ks:
                keys = np.concatenate([np.zeros(words, np.uint64), keys])
                vals = np.concatenate([[1e-9], vals])
        i, j = (int(x) for x in rng.choice(min(n_spins, 10), 2, replace=False))
        qi, qj = GENERATORS[trial % len(GENERATORS)]
        h = float(rng.uniform(-2.0, 2.0))
        threshold = float(10.0 ** rng.uniform(-6, -2))
        c, s = oracle.trig(h, 1.0)
        mapping = dict(zip(key_ints(keys, words), (float(x) for x in vals)))
        kept, removed = pair_rotation(mapping, i, j, qi, qj, c, s, threshold)
        st, ok, ov, led = oracle.rotate(keys, vals, n_spins, i, j, qi, qj, h, 1.0,
                                        threshold=threshold)
        assert st == 0
        model_keys = sorted(kept)
        assert model_keys == key_ints(ok, words), trial
        model_vals = np.array([kept[k] for k in model_keys], np.float64)
        assert np.array_equal(bits(model_vals), bits(ov)), trial
        assert (len(removed) > 0) == (led.removal_events > 0), trial
        # the removed weight: the reference's sequential upward sum is an
        # upper bound of the exact sum of the same removed values
        assert led.dropped_l1 >= sum(removed) * (1 - 1e-15), trial


def coset_run(mapping, i, j, rots, threshold):
    """Several consecutive rotations on one site pair, applied coset by coset.

    rots: [(qi, qj, c, s)].  The masks generate a group G of XOR patterns on
    the four bits of sites i and j; K's coset K xor G is closed under every
    rotation of the run, so each coset is updated on its own, rotation by
    rotation with the same pair rule and the same per-rotation zero drop and
    threshold.  Returns the kept map and the removed |v| per rotation."""
    masks = [(qi << (2 * i)) ^ (qj << (2 * j)) for qi, qj, _, _ in rots]
    group = {0}
    for m in masks:
        group |= {g ^ m for g in group}
    site_bits = (3 << (2 * i)) | (3 << (2 * j))
    cosets = {}
    for K, v in mapping.items():
        base = min(K ^ g for g in group)  # canonical member
        cosets.setdefault(base, {})[K] = v
    kept, removed = {}, [[] for _ in rots]
    for members in cosets.values():
        cur = dict(members)
        for r, (qi, qj, c, s) in enumerate(rots):
            new_vals, rem = pair_rotation(cur, i, j, qi, qj, c, s, threshold)
            removed[r] += rem
            cur = new_vals
        kept.update(cur)
        assert all((K & ~site_bits) == (next(iter(members)) & ~site_bits) for K in cur)
    return kept, removed


@pytest.mark.parametrize("n_spins", [10, 36])
def test_edge_run_by_cosets_matches_sequential(oracle, n_spins):
    """The three rotations of a secular edge (ZZ, XX, YY on one pair) applied
    coset by coset equal the reference's three sequential rotations, bitwise;
    this is what lets a future step fuse an edge's rotations into one pass."""
    rng = np.random.default_rng(77 + n_spins)
    words = (n_spins + 31) // 32
    for trial in range(12):
        keys, vals = random_map(rng, n_spins, int(rng.integers(50, 800)),
                                active_sites=range(min(n_spins, 8)))
        i, j = (int(x) for x in rng.choice(min(n_spins, 8), 2, replace=False))
        d = float(rng.uniform(0.2, 1.5))
        edge = [(3, 3, d / 2), (1, 1, -d / 4), (2, 2, -d / 4)]
        duration = 0.05
        threshold = float(10.0 ** rng.uniform(-6, -3))
        rots = [(qi, qj) + oracle.trig(h, duration) for qi, qj, h in edge]
        mapping = dict(zip(key_ints(keys, words), (float(x) for x in vals)))
        kept, removed = coset_run(mapping, i, j, rots, threshold)
        k, v = keys, vals
        for qi, qj, h in edge:
            st, k, v, led = oracle.rotate(k, v, n_spins, i, j, qi, qj, h, duration,
                                          threshold=threshold)
            assert st == 0
        model_keys = sorted(kept)
        assert model_keys == key_ints(k, words), trial
        model_vals = np.array([kept[x] for x in model_keys], np.float64)
        assert np.array_equal(bits(model_vals), bits(v)), trial
