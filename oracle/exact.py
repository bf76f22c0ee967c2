"""Exact and Krylov FID references for small rings (test infrastructure only).

Independent of Pauli propagation: these compute the free-induction decay of a
secular dipolar spin system in the computational basis, so they check the
propagated FID (Strang splitting plus truncation) from outside.  Only tests/
and the golden-fixture scripts import this module.

Convention.  H = sum over edges of d (2 Z_i Z_j - X_i X_j - Y_i Y_j) / 4, the
reference's secular edge (DDevol engine/src/cli_rev.c:125-132); M = sum_i X_i;
F(t) = Tr[M(t) M] / Tr[M M] with M(t) = exp(iHt) M exp(-iHt).  For a
translation-invariant ring F equals the propagated "fid" column of a local
X_0 start (the sum of the weight-one X coefficients, cli_rev.c:576), because
Tr[X_i(t) M] does not depend on i.

Functions:

* :func:`sector_fid` restates engine/tests/sector_reference_rev.cpp:14-38 --
  H is block diagonal in the magnetisation sectors, M couples adjacent
  sectors, F(t) = sum over eigenpairs (a in sector p-1, b in sector p) of
  2 |<a|M|b>|^2 / (n 2^n) cos((E_a - E_b) t), evaluated with the Chebyshev
  recursion cos(k x) = 2 cos(x) cos((k-1) x) - cos((k-2) x) -- with any list
  of couplings instead of the file's hard-coded J1 = 1, J2 = 0.3 (:17).
* :func:`momentum_sector_fid` is the same sum for a periodic ring whose
  couplings depend only on the ring distance, with each magnetisation sector
  further split by the ring's translation (momentum) quantum number, which H
  and M both conserve.  Blocks shrink by about n, so N = 16 takes seconds.
* :func:`dense_fid` diagonalises the full 2^n Hamiltonian (n <= 10): the
  plain density-matrix reference, for cross-checks.
* :func:`lanczos_fid` restates engine/src/lanczos_reference.cpp:14-200: a
  stochastic trace over random-phase vectors, each propagated by a Lanczos
  basis, with the t = 0 control variate and a Student-t 95% interval over the
  samples -- with parametrised couplings instead of the file's fixed ring.
"""
from __future__ import annotations

import math

import numpy as np


# ------------------------------------------------------------------ couplings
def ring_couplings(n: int, by_distance: dict[int, float]):
    """Edges (i, (i + r) % n, d) of a periodic ring in the reference's edge order
    (for each site i, distances ascending), d in the /4 convention."""
    edges = []
    for i in range(n):
        for r in sorted(by_distance):
            if by_distance[r] != 0.0:
                edges.append((i, (i + r) % n, float(by_distance[r])))
    return edges


# --------------------------------------------------------- magnetisation sectors
def _sector_states(n: int, pop: int):
    states = np.array([x for x in range(1 << n) if bin(x).count("1") == pop], dtype=np.int64)
    index = -np.ones(1 << n, dtype=np.int64)
    index[states] = np.arange(len(states))
    return states, index


def _sector_hamiltonian(n: int, states, index, edges):
    """H restricted to one sector: diagonal +-d/2, flip-flop -d/2 (both spins
    of the edge differ), sector_reference_rev.cpp:16-17 with general edges."""
    d = len(states)
    h = np.zeros((d, d))
    for i, j, J in edges:
        bi = (states >> i) & 1
        bj = (states >> j) & 1
        diff = bi != bj
        h[np.arange(d), np.arange(d)] += np.where(diff, -J / 2.0, J / 2.0)
        src = np.nonzero(diff)[0]
        dst = index[states[src] ^ ((1 << i) | (1 << j))]
        np.add.at(h, (dst, src), -J / 2.0)
    return h


def _chebyshev_sum(weights, delta, steps, dt):
    """sum_p w_p cos(delta_p k dt) for k = 0..steps, by the recursion the
    reference uses (sector_reference_rev.cpp:35), in chunks."""
    out = np.zeros(steps + 1)
    w = np.asarray(weights, dtype=np.float64).ravel()
    z = np.cos(np.asarray(delta, dtype=np.float64).ravel() * dt)
    for a in range(0, len(w), 1 << 20):
        ww, zz = w[a:a + (1 << 20)], z[a:a + (1 << 20)]
        p = np.ones_like(zz)
        q = zz.copy()
        out[0] += ww.sum()
        if steps >= 1:
            out[1] += ww @ q
        for k in range(2, steps + 1):
            y = 2.0 * zz * q - p
            out[k] += ww @ y
            p, q = q, y
    return out


def sector_fid(n: int, edges, steps: int, dt: float):
    """F(k dt), k = 0..steps, by magnetisation sectors (any couplings, n <= 12)."""
    f = np.zeros(steps + 1)
    prev_states, prev_index = _sector_states(n, 0)
    prev_e, prev_v = np.linalg.eigh(_sector_hamiltonian(n, prev_states, prev_index, edges))
    for pop in range(1, n + 1):
        states, index = _sector_states(n, pop)
        e, v = np.linalg.eigh(_sector_hamiltonian(n, states, index, edges))
        # <prev state| M |cur state>: clear one set bit of the current state
        mx = np.zeros((len(prev_states), len(states)))
        for b in range(n):
            has = np.nonzero((states >> b) & 1)[0]
            np.add.at(mx, (prev_index[states[has] ^ (1 << b)], has), 1.0)
        mat = prev_v.T @ mx @ v
        w = mat * mat * 2.0 / (n * float(1 << n))
        f += _chebyshev_sum(w, prev_e[:, None] - e[None, :], steps, dt)
        prev_states, prev_index, prev_e, prev_v = states, index, e, v
    return f


# ------------------------------------------------------- momentum-resolved sectors
def _rotate(x, r, n):
    """Bit rotation: site s -> site (s + r) mod n (the ring translation T^r)."""
    mask = (1 << n) - 1
    return ((x << r) | (x >> (n - r))) & mask


def _orbits(n: int, pop: int):
    """Translation orbits of a sector: representative (smallest member),
    period, and for every state its representative and the shift l with
    T^l state = representative."""
    states, index = _sector_states(n, pop)
    rep = np.full(len(states), -1, dtype=np.int64)
    shift = np.zeros(len(states), dtype=np.int64)
    reps, periods = [], []
    for a, x in enumerate(states):
        if rep[a] >= 0:
            continue
        orbit = [_rotate(int(x), r, n) for r in range(n)]
        r0 = min(orbit)
        period = next(p for p in range(1, n + 1) if orbit[p % n] == orbit[0])
        reps.append(r0)
        periods.append(period)
        for l in range(n):
            y = _rotate(r0, l, n)  # y = T^l r0, so T^(n-l) y = r0
            b = index[y]
            if rep[b] < 0:
                rep[b] = len(reps) - 1
                shift[b] = (n - l) % n
    return states, index, np.array(reps, dtype=np.int64), np.array(periods), rep, shift


def _momentum_blocks(n, orbit_data, k):
    """Orbits that carry momentum k (k * period = 0 mod n) and their block index."""
    _, _, reps, periods, _, _ = orbit_data
    ok = (k * periods) % n == 0
    pos = -np.ones(len(reps), dtype=np.int64)
    pos[ok] = np.arange(int(ok.sum()))
    return ok, pos


def momentum_sector_fid(n: int, by_distance: dict[int, float], steps: int, dt: float):
    """F(k dt), k = 0..steps, for a periodic ring with distance couplings
    ``by_distance`` (/4 convention), by magnetisation and momentum sectors.

    In the momentum basis |r,k> = R_r^(-1/2) sum_{p<R_r} w^(-kp) T^p |r>
    (w = exp(2 pi i / n), R_r the orbit period, k R_r = 0 mod n) a
    translation-invariant operator A has <r',k|A|r,k> = sum over basis states
    s of A|r> with representative r' and T^l s = r' of a_s w^(-k l)
    sqrt(R_r / R_r')."""
    edges = ring_couplings(n, by_distance)
    w = np.exp(2j * np.pi / n)
    orb = [_orbits(n, pop) for pop in range(n + 1)]
    f = np.zeros(steps + 1)
    norm = 2.0 / (n * float(1 << n))

    def apply_terms(pop, k):
        """H_k of sector pop (complex Hermitian)."""
        states, index, reps, periods, rep, shift = orb[pop]
        ok, pos = _momentum_blocks(n, orb[pop], k)
        dk = int(ok.sum())
        h = np.zeros((dk, dk), dtype=np.complex128)
        for a in np.nonzero(ok)[0]:
            x = int(reps[a])
            col = pos[a]
            for i, j, J in edges:
                bi, bj = (x >> i) & 1, (x >> j) & 1
                if bi == bj:
                    h[col, col] += J / 2.0
                    continue
                h[col, col] -= J / 2.0
                s = x ^ ((1 << i) | (1 << j))
                b = index[s]
                ra = rep[b]
                if not ok[ra]:
                    continue
                h[pos[ra], col] += -J / 2.0 * w ** (-k * shift[b]) * math.sqrt(
                    periods[a] / periods[ra])
        return h

    for k in range(n):
        prev = None
        for pop in range(n + 1):
            ok, pos = _momentum_blocks(n, orb[pop], k)
            if not ok.any():
                prev = None
                continue
            e, v = np.linalg.eigh(apply_terms(pop, k))
            if prev is not None:
                pe, pv, pok, ppos = prev
                states, index, reps, periods, rep, shift = orb[pop]
                _, pindex, preps, pperiods, prep, pshift = orb[pop - 1]
                mx = np.zeros((int(pok.sum()), int(ok.sum())), dtype=np.complex128)
                for a in np.nonzero(ok)[0]:
                    x = int(reps[a])
                    for bit in range(n):
                        if not (x >> bit) & 1:
                            continue
                        b = pindex[x ^ (1 << bit)]
                        ra = prep[b]
                        if not pok[ra]:
                            continue
                        mx[ppos[ra], pos[a]] += w ** (-k * pshift[b]) * math.sqrt(
                            periods[a] / pperiods[ra])
                mat = pv.conj().T @ mx @ v
                wts = (mat.real ** 2 + mat.imag ** 2) * norm
                f += _chebyshev_sum(wts, pe[:, None] - e[None, :], steps, dt)
            prev = (e, v, ok, pos)
    return f


# ------------------------------------------------------------------- dense
def _full_hamiltonian(n: int, edges):
    dim = 1 << n
    x = np.arange(dim, dtype=np.int64)
    h = np.zeros((dim, dim))
    for i, j, J in edges:
        diff = ((x >> i) & 1) != ((x >> j) & 1)
        h[x, x] += np.where(diff, -J / 2.0, J / 2.0)
        src = x[diff]
        h[src ^ ((1 << i) | (1 << j)), src] += -J / 2.0
    return h


def dense_fid(n: int, edges, times):
    """F(t) on the full 2^n space (n <= 10): Tr[M(t) M] / (n 2^n)."""
    dim = 1 << n
    x = np.arange(dim, dtype=np.int64)
    m = np.zeros((dim, dim))
    for b in range(n):
        m[x ^ (1 << b), x] += 1.0
    e, v = np.linalg.eigh(_full_hamiltonian(n, edges))
    mt = v.T @ m @ v
    w = mt * mt / (n * float(dim))
    de = e[:, None] - e[None, :]
    return np.array([float((w * np.cos(de * t)).sum()) for t in times])


# ------------------------------------------------------------------- Krylov
def _apply_h(vec, n, edges):
    x = np.arange(1 << n, dtype=np.int64)
    out = np.zeros_like(vec)
    for i, j, J in edges:
        diff = ((x >> i) & 1) != ((x >> j) & 1)
        out += np.where(diff, -J / 2.0, J / 2.0) * vec
        flip = x ^ ((1 << i) | (1 << j))
        out[flip[diff]] += -J / 2.0 * vec[diff]
    return out


def _apply_sx(vec, n):
    """sum_i S^x_i = M / 2 (lanczos_reference.cpp:14-21)."""
    x = np.arange(1 << n, dtype=np.int64)
    out = np.zeros_like(vec)
    for b in range(n):
        out += 0.5 * vec[x ^ (1 << b)]
    return out


def _lanczos_trajectory(v0, n, edges, dimension, times):
    """exp(-iHt) v0 at each time from a Lanczos basis with full
    reorthogonalisation against the two previous vectors, as
    lanczos_reference.cpp:42-120 does; returns (vectors, residual bound)."""
    norm = math.sqrt(float(np.vdot(v0, v0).real))
    basis = [v0 / norm]
    alpha, beta = [], []
    prev = None
    prevbeta = 0.0
    next_beta = 0.0
    for k in range(dimension):
        cur = basis[-1]
        r = _apply_h(cur, n, edges)
        a = float(np.vdot(cur, r).real)
        r = r - a * cur
        if prev is not None:
            r = r - prevbeta * prev
        r = r - np.vdot(cur, r) * cur
        if prev is not None:
            r = r - np.vdot(prev, r) * prev
        next_beta = math.sqrt(float(np.vdot(r, r).real))
        alpha.append(a)
        if k + 1 == dimension or next_beta < 1e-14:
            break
        beta.append(next_beta)
        prev = cur
        prevbeta = next_beta
        basis.append(r / next_beta)
    size = len(alpha)
    tri = np.diag(alpha) + np.diag(beta[:size - 1], 1) + np.diag(beta[:size - 1], -1)
    e, u = np.linalg.eigh(tri)
    q = np.array(basis[:size])
    out, residual = [], 0.0
    for t in times:
        z = u @ (np.exp(-1j * t * e) * u[0, :].conj())
        residual = max(residual, next_beta * abs(z[-1]))
        out.append(norm * (z @ q))
    return out, residual


def lanczos_fid(n: int, edges, times, samples: int = 8, dimension: int = 64, seed: int = 20260711):
    """Stochastic-trace Krylov estimate of F(t): mean, standard error, the
    Student-t 95% half-width over ``samples`` random-phase vectors, and the
    largest Lanczos residual bound (lanczos_reference.cpp:131-200).  Each
    sample uses the t = 0 control variate 1 + (C(t) - C(0)) / (n/4)."""
    rng = np.random.default_rng(seed)
    dim = 1 << n
    vals = np.zeros((len(times), samples))
    worst = 0.0
    for s in range(samples):
        r = np.exp(0.5j * np.pi * rng.integers(0, 4, dim)) / math.sqrt(dim)
        partner = _apply_sx(r, n)
        c0 = float(np.vdot(r, _apply_sx(partner, n)).real)
        left, res_l = _lanczos_trajectory(r, n, edges, dimension, times)
        right, res_r = _lanczos_trajectory(partner, n, edges, dimension, times)
        worst = max(worst, res_l, res_r)
        for k in range(len(times)):
            corr = float(np.vdot(left[k], _apply_sx(right[k], n)).real)
            vals[k, s] = 1.0 + (corr - c0) / (n / 4.0)
    mean = vals.mean(axis=1)
    se = vals.std(axis=1, ddof=1) / math.sqrt(samples)
    t975 = {8: 2.3646242515927844}.get(samples, 2.0)
    return mean, se, t975 * se, worst, vals
