"""Input builders: term counts and shells of the benchmark configurations."""
import math

import numpy as np

from ddevol_gb300 import hamiltonians as H


def test_ring16_j1j2_terms():
    terms = H.ring_j1j2(16)
    assert len(terms) == 96
    # the configurations' d (2ZZ - XX - YY) / 2 convention, passed to the reference edge as d' = 2d
    assert terms[0] == (0, 1, 3, 3, 1.0)
    assert terms[1] == (0, 1, 1, 1, -0.5)
    assert terms[3] == (0, 2, 3, 3, 0.125)


def test_ring64_all_pairs_terms():
    terms = H.ring_all_pairs(64)
    assert len(terms) == 3 * 2016
    # nearest neighbour: chord(1) on a circle of circumference 64
    r = (64 / math.pi) * math.sin(math.pi / 64)
    assert terms[0][4] == 1.0 / r ** 3


def test_cubic_111_shells():
    terms = H.cubic_111(4)
    assert len(terms) == 3 * 640
    neighbours = {}
    for i, j, *_ in terms[::3]:
        neighbours[i] = neighbours.get(i, 0) + 1
        neighbours[j] = neighbours.get(j, 0) + 1
    assert set(neighbours.values()) == {20}


def test_sphere_directions_unit():
    d = np.array(H.sphere_directions(512))
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0)
    assert abs(d[:, 2].mean()) < 0.1


def test_initial_operators():
    k, v = H.single_site_operator(64, 0)
    assert list(k) == [1, 0] and list(v) == [1.0]
    k, v = H.global_x_operator(6)
    assert list(k) == [1, 4, 16, 64, 256, 1024]


def test_serving_request_matches_all_pairs_builders():
    """The serving stream's fast pair walk builds the same term list as the
    all-pairs builders with the same cutoff, for rings and chains."""
    seen = set()
    for seed in range(12):
        rng = np.random.default_rng(seed)
        n, terms, thr, steps, dt = H.serving_request(rng)
        rng = np.random.default_rng(seed)
        n2 = int(rng.integers(16, 97))
        scale = rng.normal(1.0, 0.1, size=(n2, n2))
        ring = bool(rng.random() < 0.5)
        seen.add(ring)
        build = H.ring_all_pairs if ring else H.chain_all_pairs
        assert n == n2 and terms == build(n, scale=scale, cutoff=3)
        assert 1e-6 <= thr <= 1e-4 and 20 <= steps <= 80 and dt == 0.01
    assert seen == {True, False}
