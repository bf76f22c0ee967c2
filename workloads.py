"""Benchmark trajectories as a command-line driver (used for profiling).

    python workloads.py --config ring16 --setup-steps 200 --steps 1 [--events]
    python workloads.py --config ring64 --target-terms 1e5 --save-state S.npz
    python workloads.py --config ring64 --load-state tests/golden/ring64_window.npz --steps 1
    python workloads.py --batch serve --items 16 --setup-steps 10 --steps 1

Single-map mode evolves the configuration from its initial operator for
--setup-steps Strang steps (or until the map holds --target-terms terms),
then runs --steps more and prints one JSON line: map sizes, device time,
input terms, rotations, launches; with --events the measured steps run with
per-kernel CUDA events and the line carries per-kernel times and shares.
--save-state writes the map after the set-up (keys, values, steps) and
--load-state starts from such a file instead of a set-up, so a profiler
capture sees only the measured steps' launches: 1 (upload check) + 1 (first
classify) + 3 per rotation.  The kernel launch sequence is deterministic.

Batch mode (--batch serve) builds --items requests of the serving stream
(seeded ring/chain mixes of 16..96 spins), advances them together for
--setup-steps batched steps, then --steps more, and prints per-step device
times; a batched step is 2 launches per (key width, cluster size) group.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from ddevol_gb300 import hamiltonians as H  # noqa: E402
from ddevol_gb300.engine import Engine, GbLedger, options  # noqa: E402

CONFIGS = {
    "ring64": (64, lambda: H.ring_all_pairs(64), 0.005, 1e-5),
    "ring16": (16, lambda: H.ring_j1j2(16), 0.01, 1e-6),
    "cubic": (64, lambda: H.cubic_111(4), 0.005, 1e-5),
}


def run(config: str, setup_steps: int, steps: int, events: bool, exact_ledger: bool = False,
        target_terms: float = 0.0, save_state: str = "", load_state: str = ""):
    n, make_terms, dt, thr = CONFIGS[config]
    terms = make_terms()
    eng = Engine(0)
    opts = options(thr, exact_ledger=exact_ledger)
    led = GbLedger()
    if load_state:
        z = np.load(load_state)
        m = eng.map(n, z["keys"], z["values"])
        setup_steps = int(z["steps"])
    else:
        m = eng.map(n, *H.single_site_operator(n))
        done = 0
        while done < setup_steps or (target_terms and len(m) < target_terms):
            st, _, led, msg = m.evolve(terms, dt, 1, opts, led, record_fid=False)
            if st:
                raise RuntimeError(msg)
            done += 1
        setup_steps = done
        if save_state:
            k, v = m.download()
            np.savez(save_state, keys=k, values=v, steps=setup_steps)
    n0 = len(m)
    if events:
        m.set_profiling(True)
    st, _, led, msg = m.evolve(terms, dt, steps, opts, led, record_fid=False)
    if st:
        raise RuntimeError(msg)
    out = dict(config=config, setup_steps=setup_steps, n0=n0, n1=len(m), ms=m.last_elapsed_ms(),
               terms=m.last_terms(), launches=m.last_launches(),
               rotations=2 * len(terms) * steps)
    out["terms_per_s"] = out["terms"] / (out["ms"] / 1e3)
    out["us_per_rotation"] = out["ms"] * 1e3 / out["rotations"]
    if events:
        prof = m.kernel_profile()
        tot = sum(v[0] for v in prof.values()) or 1.0
        out["kernel_us_per_launch"] = {k: round(v[0] * 1e3 / max(1, v[1]), 2)
                                       for k, v in prof.items()}
        out["kernel_share"] = {k: round(v[0] / tot, 3) for k, v in prof.items()}
    m.close()
    eng.close()
    return out


def run_batch(items: int, setup_steps: int, steps: int, seed: int = 20261203):
    from ddevol_gb300.engine import Batch
    rng = np.random.default_rng(seed)
    reqs = [H.serving_request(rng) for _ in range(items)]
    eng = Engine(0)
    batch = Batch(eng, [r[0] for r in reqs])
    for k, (n, terms, thr, _, dt) in enumerate(reqs):
        batch.upload(k, *H.single_site_operator(n, 0))
        batch.set_terms(k, terms, dt, options(thr, exact_ledger=False))
    if setup_steps:
        batch.step(setup_steps, record_fid=False)
    lens0 = [batch.item_len(k) for k in range(items)]
    per_step = []
    for _ in range(steps):
        batch.step(1, record_fid=False)
        per_step.append(dict(ms=round(batch.last_elapsed_ms(), 3), terms=batch.last_terms(),
                             launches=batch.last_launches()))
    out = dict(batch="serve", items=items, setup_steps=setup_steps,
               rotations_max=max(2 * len(r[1]) for r in reqs),
               len_median=int(np.median(lens0)), len_max=int(max(lens0)), steps=per_step)
    batch.close()
    eng.close()
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--config", choices=sorted(CONFIGS), default="ring16")
    ap.add_argument("--setup-steps", type=int, default=140)
    ap.add_argument("--target-terms", type=float, default=0.0)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--events", action="store_true")
    ap.add_argument("--exact-ledger", action="store_true")
    ap.add_argument("--save-state", default="")
    ap.add_argument("--load-state", default="")
    ap.add_argument("--batch", choices=["serve"], default=None)
    ap.add_argument("--items", type=int, default=16)
    a = ap.parse_args()
    if a.batch:
        out = run_batch(a.items, a.setup_steps, a.steps)
    else:
        out = run(a.config, a.setup_steps, a.steps, a.events, a.exact_ledger, a.target_terms,
                  a.save_state, a.load_state)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
