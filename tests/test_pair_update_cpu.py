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
