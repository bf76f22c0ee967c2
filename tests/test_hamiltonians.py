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


def test_term_builders_match_the_reference_cli():
    """The benchmark's 16-spin term list is bitwise the reference CLI's for the
    committed edges file, and the J1-J2 builder reproduces the CLI's j1j2
    model (its d = 2 J convention: J = 1/2, J2 = ratio / 2), from the
    reference CLI's own records (tests/golden/cli_terms.npz)."""
    import os

    import numpy as np
    golden = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                  "cli_terms.npz"))

    def same(terms, name):
        ijq = np.array([t[:4] for t in terms], np.uint64)
        h = np.array([t[4] for t in terms], np.float64)
        return (np.array_equal(ijq, golden[name + "_ijq"]) and
                np.array_equal(h.view(np.uint64), golden[name + "_h"].view(np.uint64)))

    assert same(H.ring_j1j2(16), "edges_ring16")
    assert same(H.ring_j1j2(10, 0.5, 0.0625), "j1j2_n10_j2_0125")
    assert same(H.ring_j1j2(8, 0.5, 0.15), "j1j2_n8")
