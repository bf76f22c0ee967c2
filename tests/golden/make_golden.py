"""Generate the golden fixtures that pin the CPU oracle to the reference engine.

Runs the reference engine itself -- DDevol engine/src/tpgp_rev.c compiled from
its own sources by ``make -C oracle ref`` into ``oracle/_ref/`` -- on seeded
inputs and stores inputs and outputs as small ``.npz`` files next to this
script.  It needs the reference checkout, so it runs only where that exists;
the fixtures it writes are committed and travel with the tests.

    make -C oracle ref && python tests/golden/make_golden.py

Cases:
* rotations.npz   -- single tpgp_rotate calls on random sorted maps (N from 2
                     to 100, every generator pair, three thresholds), crafted
                     exact cancellations, and every failure status.
* trajectories.npz -- tpgp_strang_step trajectories: the benchmark ring
                     (N=16 J1-J2, X_0, dt=0.01, threshold 1e-6), the
                     reference's own N=6 CUDA-trajectory case, a 64-site
                     all-pairs ring step and a 4x4x4 [111] cubic step.
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import LedgerStruct, Oracle, Reference  # noqa: E402
from ddevol_gb300 import hamiltonians as H  # noqa: E402

LEDGER_FIELDS = [name for name, _ in LedgerStruct._fields_]


def pack_keys(symbol_rows, n_spins):
    words = (n_spins + 31) // 32
    packed = []
    for row in symbol_rows:
        k = [0] * words
        for s, p in enumerate(row):
            k[s // 32] |= int(p) << (2 * (s % 32))
        packed.append(k)
    packed.sort(key=lambda x: tuple(reversed(x)))
    return np.array(packed, np.uint64).reshape(-1)


def random_map(rng, n_spins, count, local_bias=False):
    """Distinct random keys (sorted) with values spread over 9 decades."""
    count = min(count, 4 ** n_spins // 2) if n_spins < 16 else count
    rows = set()
    while len(rows) < count:
        if local_bias:
            # mostly identity with a few active sites, like propagated operators
            row = [0] * n_spins
            for s in rng.choice(n_spins, int(rng.integers(1, min(6, n_spins) + 1)),
                                replace=False):
                row[s] = int(rng.integers(1, 4))
        else:
            row = [int(x) for x in rng.integers(0, 4, size=n_spins)]
        rows.add(tuple(row))
    keys = pack_keys(sorted(rows), n_spins)
    values = rng.standard_normal(count) * 10.0 ** rng.uniform(-9, 0, count)
    return keys, values


def ledger_array(led):
    return np.array([float(getattr(led, f)) for f in LEDGER_FIELDS], np.float64)


def rotation_cases(ref: Reference, port: Oracle):
    rng = np.random.default_rng(20261203)
    cases = []
    sizes = [2, 3, 5, 16, 31, 32, 33, 64, 65, 96, 100]
    for trial in range(72):
        n = sizes[trial % len(sizes)]
        count = int(rng.integers(1, 400))
        keys, values = random_map(rng, n, count, local_bias=bool(trial % 2))
        if trial % 9 == 0:
            # the identity key, never truncated
            words = (n + 31) // 32
            if not np.any(np.all(keys.reshape(-1, words) == 0, axis=1)):
                keys = np.concatenate([np.zeros(words, np.uint64), keys])
                values = np.concatenate([[1e-12], values])
        i, j = (int(x) for x in rng.choice(n, 2, replace=False))
        qi, qj = int(rng.integers(0, 4)), int(rng.integers(0, 4))
        theta = float(rng.uniform(-1.6, 1.6))
        threshold = float([0.0, 1e-6, 1e-3][trial % 3])
        cases.append(dict(n=n, keys=keys, values=values, i=i, j=j, qi=qi, qj=qj,
                          theta=theta, threshold=threshold, max_terms=0, max_drop_l2=0.0))
    # exact cancellation: values (s, c) on a flipped pair cancel to an exact zero
    n = 4
    c, s = port.trig(0.3, 1.0)
    for qi, qj in ((3, 3), (1, 1), (2, 2), (1, 3)):
        for base in ([1, 0, 0, 0], [2, 3, 1, 0], [1, 1, 2, 3]):
            partner = list(base)
            partner[0] ^= qi
            partner[1] ^= qj
            rows = sorted({tuple(base), tuple(partner)})
            if len(rows) != 2:
                continue
            keys = pack_keys(rows, n)
            for sv in ((s, c), (s, -c), (-s, c)):
                cases.append(dict(n=n, keys=keys, values=np.array(sv, np.float64), i=0, j=1,
                                  qi=qi, qj=qj, theta=0.3, threshold=0.0, max_terms=0,
                                  max_drop_l2=0.0))
    # failure statuses: cap, budget, invalid, nonfinite, overflow, no-op angle
    keys, values = random_map(rng, 16, 50, local_bias=True)
    cases.append(dict(n=16, keys=keys, values=values, i=0, j=1, qi=3, qj=3, theta=0.4,
                      threshold=0.0, max_terms=3, max_drop_l2=0.0))
    cases.append(dict(n=16, keys=keys, values=values, i=0, j=1, qi=1, qj=1, theta=0.4,
                      threshold=1e-3, max_terms=0, max_drop_l2=1e-300))
    cases.append(dict(n=16, keys=keys, values=values, i=3, j=3, qi=1, qj=1, theta=0.4,
                      threshold=0.0, max_terms=0, max_drop_l2=0.0))
    cases.append(dict(n=16, keys=keys, values=values, i=3, j=4, qi=5, qj=1, theta=0.4,
                      threshold=0.0, max_terms=0, max_drop_l2=0.0))
    cases.append(dict(n=16, keys=keys, values=values, i=3, j=4, qi=1, qj=1, theta=0.4,
                      threshold=-1.0, max_terms=0, max_drop_l2=0.0))
    cases.append(dict(n=16, keys=keys, values=values, i=3, j=4, qi=1, qj=1, theta=0.0,
                      threshold=0.0, max_terms=0, max_drop_l2=0.0))
    cases.append(dict(n=16, keys=keys, values=values, i=3, j=4, qi=1, qj=1, theta=1e308,
                      threshold=0.0, max_terms=0, max_drop_l2=0.0))
    bad = values.copy()
    bad[7] = np.nan
    cases.append(dict(n=16, keys=keys, values=bad, i=3, j=4, qi=1, qj=1, theta=0.4,
                      threshold=0.0, max_terms=0, max_drop_l2=0.0))
    big_keys = pack_keys([[1, 0, 0], [2, 3, 0]], 3)
    cases.append(dict(n=3, keys=big_keys, values=np.array([1.7e308, 1.7e308]), i=0, j=1,
                      qi=3, qj=3, theta=0.7, threshold=0.0, max_terms=0, max_drop_l2=0.0))

    out = {}
    for idx, case in enumerate(cases):
        st, k, v, led = ref.rotate(case["keys"], case["values"], case["n"], case["i"],
                                   case["j"], case["qi"], case["qj"], case["theta"],
                                   threshold=case["threshold"], max_terms=case["max_terms"],
                                   max_drop_l2=case["max_drop_l2"])
        p = f"c{idx:03d}_"
        out[p + "n"] = np.array(case["n"])
        out[p + "in_keys"] = case["keys"]
        out[p + "in_values"] = case["values"]
        out[p + "params"] = np.array([case["i"], case["j"], case["qi"], case["qj"]], np.int64)
        out[p + "theta"] = np.array(case["theta"])
        out[p + "threshold"] = np.array(case["threshold"])
        out[p + "max_terms"] = np.array(case["max_terms"])
        out[p + "max_drop_l2"] = np.array(case["max_drop_l2"])
        out[p + "status"] = np.array(st)
        out[p + "out_keys"] = k
        out[p + "out_values"] = v
        out[p + "ledger"] = ledger_array(led)
    out["count"] = np.array(len(cases))
    return out


def trajectory_cases(ref: Reference):
    out = {}
    cases = []
    # benchmark ring: N=16 J1-J2 (1, 1/8), X_0, dt=0.01, threshold 1e-6
    k, v = H.single_site_operator(16)
    cases.append(("ring16", 16, k, v, H.ring_j1j2(16), 0.01, 1e-6, 20))
    # the reference's own N=6 CUDA-trajectory case (test_cuda_trajectory_rev.c:13-71)
    terms6 = []
    for s in range(6):
        for rng_ in (1, 2):
            d = 1.0 if rng_ == 1 else 0.3
            terms6 += [(s, (s + rng_) % 6, 3, 3, d / 2), (s, (s + rng_) % 6, 1, 1, -d / 4),
                       (s, (s + rng_) % 6, 2, 2, -d / 4)]
    k6, v6 = H.global_x_operator(6)
    cases.append(("n6_thr0", 6, k6, v6, terms6, 1.0 / 64, 0.0, 3))
    cases.append(("n6_thr1e-5", 6, k6, v6, terms6, 1.0 / 64, 1e-5, 3))
    # 64-site all-pairs ring, one step
    k64, v64 = H.single_site_operator(64)
    cases.append(("ring64_allpairs", 64, k64, v64, H.ring_all_pairs(64), 0.005, 1e-5, 1))
    # 4x4x4 [111] cubic, two steps
    cases.append(("cubic4", 64, k64, v64, H.cubic_111(4), 0.005, 1e-5, 2))
    # 96-site chain with short range (three-word keys), two steps
    k96, v96 = H.single_site_operator(96, site=40)
    cases.append(("chain96", 96, k96, v96, H.chain_all_pairs(96, cutoff=3), 0.01, 1e-5, 2))
    names = []
    for name, n, k0, v0, terms, dt, thr, steps in cases:
        fids, lens = [], []
        st, k, v, led = ref.strang_step(k0, v0, n, terms, dt, threshold=thr, steps=steps,
                                        on_step=lambda s, f, ln: (fids.append(f),
                                                                  lens.append(ln)))
        assert st == 0, (name, st)
        p = name + "__"
        out[p + "n"] = np.array(n)
        out[p + "in_keys"] = k0
        out[p + "in_values"] = v0
        out[p + "terms"] = np.array([[t[0], t[1], t[2], t[3]] for t in terms], np.int64)
        out[p + "h"] = np.array([t[4] for t in terms], np.float64)
        out[p + "dt"] = np.array(dt)
        out[p + "threshold"] = np.array(thr)
        out[p + "steps"] = np.array(steps)
        out[p + "out_keys"] = k
        out[p + "out_values"] = v
        out[p + "ledger"] = ledger_array(led)
        out[p + "fid_sum"] = np.array(fids, np.float64)
        out[p + "len"] = np.array(lens, np.int64)
        names.append(name)
        print(f"{name}: {len(v)} terms after {steps} steps, ledger {led.as_dict()}")
    out["names"] = np.array(names)
    return out


def main():
    ref = Reference()
    port = Oracle()
    rot = rotation_cases(ref, port)
    np.savez_compressed(os.path.join(HERE, "rotations.npz"), **rot)
    print("rotations:", int(rot["count"]), "cases")
    traj = trajectory_cases(ref)
    np.savez_compressed(os.path.join(HERE, "trajectories.npz"), **traj)


if __name__ == "__main__":
    main()
