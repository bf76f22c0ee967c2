"""Benchmark trajectories as a command-line driver (used for profiling).

    python -m ddevol_gb300.workloads --config ring16 --setup-steps 200 --steps 1 [--events]

Evolves the configuration from its initial operator for --setup-steps Strang
steps, then runs --steps more and prints one JSON line: map sizes, device
time, input terms, rotations, launches; with --events the measured steps run
with per-kernel CUDA events and the line carries per-kernel times and
shares.  The kernel launch sequence is deterministic, so an ncu capture can
skip the set-up launches by count: 1 (upload check) + setup_steps x
(3 x rotations_per_step + 1) launches precede the measured steps.
"""
from __future__ import annotations

import argparse
import json

from . import hamiltonians as H
from .engine import Engine, GbLedger, options

CONFIGS = {
    "ring64": (64, lambda: H.ring_all_pairs(64), 0.005, 1e-5),
    "ring16": (16, lambda: H.ring_j1j2(16), 0.01, 1e-6),
    "cubic": (64, lambda: H.cubic_111(4), 0.005, 1e-5),
}


def run(config: str, setup_steps: int, steps: int, events: bool, exact_ledger: bool = False):
    n, make_terms, dt, thr = CONFIGS[config]
    terms = make_terms()
    eng = Engine(0)
    m = eng.map(n, *H.single_site_operator(n))
    led = GbLedger()
    opts = options(thr, exact_ledger=exact_ledger)
    st, _, led, msg = m.evolve(terms, dt, setup_steps, opts, led, record_fid=False)
    if st:
        raise RuntimeError(msg)
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


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--config", choices=sorted(CONFIGS), default="ring16")
    ap.add_argument("--setup-steps", type=int, default=140)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--events", action="store_true")
    ap.add_argument("--exact-ledger", action="store_true")
    a = ap.parse_args()
    print(json.dumps(run(a.config, a.setup_steps, a.steps, a.events, a.exact_ledger)), flush=True)


if __name__ == "__main__":
    main()
