"""Secular dipolar term lists and initial operators.

A term is ``(i, j, qi, qj, h)``: the Hamiltonian contribution ``h * Q`` with
``Q = sigma^qi_i sigma^qj_j`` (I=0, X=1, Y=2, Z=3).  Array order is
authoritative: the Strang step applies the terms forward, then backward.

Coupling convention.  The reference builds each secular edge as
``d (2 ZZ - XX - YY) / 4``, i.e. three terms ``(ZZ, d/2), (XX, -d/4),
(YY, -d/4)`` in that order, and drops exact zeros (DDevol
engine/src/cli_rev.c:108-132).  The benchmark configurations write the
Hamiltonian as ``sum d_ij (2 ZZ - XX - YY) / 2``, twice that; so every builder
here takes the physical coupling ``d`` of that convention and passes
``2 d`` through :func:`edge_terms`, exactly as one would feed the reference's
``--model edges`` input.
"""
from __future__ import annotations

import math

import numpy as np

X, Y, Z = 1, 2, 3


def edge_terms(i: int, j: int, d_ref: float):
    """Reference secular edge (cli_rev.c:125-132): ZZ d/2, XX -d/4, YY -d/4.

    Terms with h == 0 are skipped, as ``append`` does (cli_rev.c:108-110).
    """
    out = []
    for q, h in ((Z, d_ref / 2), (X, -d_ref / 4), (Y, -d_ref / 4)):
        if h != 0:
            out.append((i, j, q, q, h))
    return out


def ring_j1j2(n: int = 16, j1: float = 1.0, j2: float = 0.125):
    """Periodic ring with nearest (j1) and next-nearest (j2) couplings.

    Edge order follows the reference's ``models`` loop (cli_rev.c:239-244):
    for each site i, the (i, i+1) edge then the (i, i+2) edge.
    """
    terms = []
    for i in range(n):
        terms += edge_terms(i, (i + 1) % n, 2 * j1)
        if j2:
            terms += edge_terms(i, (i + 2) % n, 2 * j2)
    return terms


def chord(n: int, i: int, j: int) -> float:
    """Chord length between sites i, j on a circle of circumference n."""
    return (n / math.pi) * math.sin(math.pi * abs(i - j) / n)


def ring_all_pairs(n: int = 64, scale=None, cutoff: int | None = None):
    """Periodic ring with all-pairs couplings d_ij = g_ij / r_ij^3.

    r_ij is the chord length on a unit-spacing circle of circumference n.
    ``scale`` is an optional (n, n) array of disorder factors g_ij; ``cutoff``
    keeps only pairs whose ring distance min(|i-j|, n-|i-j|) <= cutoff.
    Pairs are ordered i < j lexicographically.
    """
    terms = []
    for i in range(n):
        for j in range(i + 1, n):
            sep = min(j - i, n - (j - i))
            if cutoff is not None and sep > cutoff:
                continue
            d = 1.0 / chord(n, i, j) ** 3
            if scale is not None:
                d *= float(scale[i, j])
            terms += edge_terms(i, j, 2 * d)
    return terms


def chain_all_pairs(n: int, scale=None, cutoff: int | None = None):
    """Open chain with couplings d_ij = g_ij / |i-j|^3 (pairs i < j)."""
    terms = []
    for i in range(n):
        for j in range(i + 1, n):
            if cutoff is not None and j - i > cutoff:
                continue
            d = 1.0 / float(j - i) ** 3
            if scale is not None:
                d *= float(scale[i, j])
            terms += edge_terms(i, j, 2 * d)
    return terms


def _cubic_coords(site: int, L: int):
    return site % L, (site // L) % L, site // (L * L)


def cubic_111(L: int = 4, max_r2: int = 4):
    """Periodic L^3 simple cubic lattice, field along [111], cutoff r^2 <= max_r2.

    d_ij = (1 - 3 cos^2 theta) / r^3 with cos^2 theta = (dx+dy+dz)^2 / (3 r^2)
    under the minimum image.  The angular factor is evaluated as the integer
    ratio (r^2 - (dx+dy+dz)^2) / r^2 so that vanishing shells are exact zeros
    (the r^2 = 1 and r^2 = 4 shells), which the edge builder then drops.
    Site index s = x + L y + L^2 z, as in the reference's cubic model
    (cli_rev.c:183-206); pairs ordered i < j.
    """
    n = L ** 3
    terms = []
    for i in range(n):
        a = _cubic_coords(i, L)
        for j in range(i + 1, n):
            b = _cubic_coords(j, L)
            d = []
            for k in range(3):
                x = b[k] - a[k]
                if x > L // 2:
                    x -= L
                if x < -(L // 2):
                    x += L
                d.append(x)
            r2 = d[0] ** 2 + d[1] ** 2 + d[2] ** 2
            if r2 == 0 or r2 > max_r2:
                continue
            num = r2 - (d[0] + d[1] + d[2]) ** 2
            if num == 0:
                continue
            coupling = (num / r2) / (r2 * math.sqrt(r2))
            terms += edge_terms(i, j, 2 * coupling)
    return terms


def cubic_fragment(n: int, direction, L: int = 4, max_r2: int = 4):
    """First n sites of an open L^3 block, field along unit vector ``direction``.

    d_ij = (1 - 3 cos^2 theta) / r^3 with cos theta = (r_ij . b) / r, r^2 <= max_r2.
    """
    bx, by, bz = (float(v) for v in direction)
    terms = []
    for i in range(n):
        a = _cubic_coords(i, L)
        for j in range(i + 1, n):
            b = _cubic_coords(j, L)
            dx, dy, dz = b[0] - a[0], b[1] - a[1], b[2] - a[2]
            r2 = dx * dx + dy * dy + dz * dz
            if r2 > max_r2:
                continue
            proj = dx * bx + dy * by + dz * bz
            coupling = (1.0 - 3.0 * (proj * proj) / r2) / (r2 * math.sqrt(r2))
            if coupling == 0:
                continue
            terms += edge_terms(i, j, 2 * coupling)
    return terms


def splitmix64(state: int):
    """One splitmix64 step: returns (next_state, output), both uint64."""
    state = (state + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = state
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return state, z ^ (z >> 31)


def sphere_directions(count: int, seed: int = 20260711):
    """Uniform unit vectors: z ~ U(-1,1), phi ~ U(0, 2 pi) from splitmix64."""
    state = seed
    out = []
    for _ in range(count):
        state, a = splitmix64(state)
        state, b = splitmix64(state)
        z = -1.0 + 2.0 * ((a >> 11) * 2.0 ** -53)
        phi = 2.0 * math.pi * ((b >> 11) * 2.0 ** -53)
        rho = math.sqrt(max(0.0, 1.0 - z * z))
        out.append((rho * math.cos(phi), rho * math.sin(phi), z))
    return out


def single_site_operator(n_spins: int, site: int = 0, pauli: int = X, value: float = 1.0):
    """Map holding one term value * sigma^pauli_site (``--initial local``)."""
    words = (n_spins + 31) // 32
    key = np.zeros(words, np.uint64)
    key[site // 32] = np.uint64(pauli) << np.uint64(2 * (site % 32))
    return key, np.array([value], np.float64)


def global_x_operator(n_spins: int):
    """Map holding sum_i X_i (``--initial global``), keys ascending."""
    words = (n_spins + 31) // 32
    keys = np.zeros((n_spins, words), np.uint64)
    for s in range(n_spins):
        keys[s, s // 32] = np.uint64(X) << np.uint64(2 * (s % 32))
    order = sorted(range(n_spins), key=lambda r: tuple(int(x) for x in keys[r][::-1]))
    return keys[order].reshape(-1), np.ones(n_spins, np.float64)


def _pairs_within(n: int, cutoff: int, periodic: bool):
    """Pairs i < j (lexicographic) with ring (periodic) or chain distance <= cutoff."""
    out = []
    for i in range(n):
        js = set(range(i + 1, min(n, i + cutoff + 1)))
        if periodic:
            js.update(range(max(i + 1, n - cutoff + i), n))
        out += [(i, j) for j in sorted(js)]
    return out


def serving_request(rng, steps_range=(20, 80), cutoff=3, dt=0.01):
    """One FID-solve request of the serving stream: a ring or an open chain
    (p = 1/2) of N uniform in {16..96} spins, couplings d = g_ij / r^3 with a
    Gaussian disorder factor g ~ N(1, 0.1) per pair, pairs up to ring/chain
    distance ``cutoff`` (the term list equals ``ring_all_pairs`` /
    ``chain_all_pairs`` with that cutoff), threshold log-uniform in
    [1e-6, 1e-4], X on site 0.  Returns (n, terms, threshold, steps, dt)."""
    n = int(rng.integers(16, 97))
    scale = rng.normal(1.0, 0.1, size=(n, n))
    ring = bool(rng.random() < 0.5)
    terms = []
    for i, j in _pairs_within(n, cutoff, ring):
        d = 1.0 / (chord(n, i, j) ** 3 if ring else float(j - i) ** 3)
        terms += edge_terms(i, j, 2 * (d * float(scale[i, j])))
    threshold = float(10.0 ** rng.uniform(-6, -4))
    steps = int(rng.integers(steps_range[0], steps_range[1] + 1))
    return n, terms, threshold, steps, dt
