#!/usr/bin/env python
"""Pauli terms/s of the device-resident branch step on GB300.

Workload (default): the 64-spin periodic ring with all-pairs secular dipolar
couplings d = 1/r^3 (r the chord on a unit-spacing circle), observable X_0,
dt = 0.005, threshold 1e-5, 128-bit keys -- the larger plain-method benchmark
configuration.  Its full 1000-step trajectory is far too long for one bench
run, so a bench "step" is one Strang step (12,096 rotations) of a window of
that trajectory.  Both arms start from the same committed state,
tests/golden/ring64_window.npz (the trajectory at step 311, 100,947 terms;
bitwise the reference engine's trajectory): W warm-up steps run, then
exactly K steps are timed.

Metric: Pauli terms/s = (sum over the timed rotations of the rotation's input
terms) / device time of the K steps (CUDA events on the engine's stream).
The timed steps use the fixed-point (bound) removed-weight ledger: keys,
values and FIDs are bitwise the reference's, the ledger's removed-weight
sums are upper bounds within a few ulps of the reference's sequential sums.
The ABI's default exact ledger (every output bitwise, the ledger included)
is the `exact_ledger` sub-line; --exact-ledger times it instead.

Extra keys: e2e (the same K steps from the same state through the C-ABI
with pinned host buffers, L2 flushed before each step as in the device leg:
every step uploads the map, runs the step, reads its FID and downloads the
map), roofline (HBM bound: the dominant kernel's algorithmic bytes per
launch over its mean launch time, from CUDA events captured into the timed
steps' graphs), cpu_baseline (the CPU implementation on rotations spread
over one whole step of the window state), clocks (nvidia-smi sampled during
the timed region), gpu_launches, and forms: the plain single solve (16-spin
ring, 400 steps), one step with the other ledger, the batched powder
average and the serving stream, each bounded in time, with FID solves/s,
roofline fraction and clocks.

--impl reference times the reference algorithm on the host cores instead
(the reference engine where it was compiled here, else the oracle's
restatement of it) on the same window state; it loads no GPU library.
Multi-GPU: independent replicas (the path has no data-parallel exchange).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from ddevol_gb300 import hamiltonians as H  # noqa: E402

METRIC = "Pauli terms/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0

CONFIGS = {
    "ring64": dict(
        n=64, dt=0.005, threshold=1e-5,
        terms=lambda: H.ring_all_pairs(64),
        init=lambda: H.single_site_operator(64, 0),
        label="64-spin periodic ring, all-pairs d=1/r^3 (chord), X_0, dt=0.005, "
              "threshold 1e-5, 128-bit keys"),
    "ring16": dict(
        n=16, dt=0.01, threshold=1e-6,
        terms=lambda: H.ring_j1j2(16),
        init=lambda: H.single_site_operator(16, 0),
        label="16-spin periodic ring, J1=1, J2=1/8, X_0, dt=0.01, threshold 1e-6, "
              "64-bit keys"),
    "cubic": dict(
        n=64, dt=0.005, threshold=1e-5,
        terms=lambda: H.cubic_111(4),
        init=lambda: H.single_site_operator(64, 0),
        label="4x4x4 periodic simple cubic, field [111], r<=2, X on site 0, dt=0.005, "
              "threshold 1e-5, 128-bit keys"),
}


def profiler_range(on: bool):
    """cudaProfilerStart/Stop around the timed region, so that
    `ncu --profile-from-start off` captures exactly the timed launches
    (no effect without a profiler)."""
    try:
        from ddevol_gb300 import native
        lib = native.load(build_if_needed=False)
        (lib.cudaProfilerStart if on else lib.cudaProfilerStop)()
    except Exception:
        pass


def repo_libraries():
    """Shared libraries of this repository mapped into the process (Linux)."""
    libs = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if len(line.split()) >= 6 else ""
                if path.endswith(".so") and path.startswith(ROOT):
                    libs.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(libs)


def peaks():
    try:
        with open(PEAKS_FILE) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples during the timed region (read-only queries)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def physical_gpu_index(local_rank):
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        items = [v.strip() for v in vis.split(",") if v.strip()]
        if local_rank < len(items) and items[local_rank].isdigit():
            return int(items[local_rank])
    return local_rank


# ------------------------------------------------------------ distributed
class Dist:
    """Ranks of a multi-GPU run (torchrun env).  Replicas only: the process
    group carries the barrier around the timed region and the max / sum of
    the per-rank results, never solve data.  backend: "nccl" (GPUs) or
    "gloo" (host; the CPU tests of this class)."""

    def __init__(self, backend=None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            backend = backend or ("nccl" if torch.cuda.is_available() else "gloo")
            if backend == "nccl":
                torch.cuda.set_device(self.local_rank)
            dist.init_process_group(backend)
            self.device = "cuda" if backend == "nccl" else "cpu"
            self.dist = dist
            self.torch = torch
            self.pg = True

    def barrier(self):
        if self.pg:
            self.dist.barrier()

    def reduce(self, value, op="max"):
        if not self.pg:
            return value
        t = self.torch.tensor([float(value)], dtype=self.torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX if op == "max" else self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.dist.destroy_process_group()


# ------------------------------------------------------------- CPU samples
class L2Flush:
    """Writes a 512 MB device buffer (four times the 129 MB L2) and waits."""

    def __init__(self, device):
        import torch
        self.torch = torch
        self.buf = torch.empty(512 << 20, dtype=torch.uint8, device=f"cuda:{device}")

    def __call__(self):
        self.buf.fill_(1)
        self.torch.cuda.synchronize()


def cpu_engine():
    """The CPU implementation a sample runs on: the reference engine compiled
    from its own sources (oracle/_ref, only where the reference checkout was
    present at build time), else the oracle's restatement of it."""
    ref_so = os.path.join(ROOT, "oracle", "_ref", "libtpgp_ref.so")
    if os.path.exists(ref_so):
        try:
            from oracle.oracle import Reference
            return Reference(ref_so), "reference"
        except OSError:
            pass
    from oracle.oracle import Oracle, build_oracle
    build_oracle()
    return Oracle(), "port"


def cpu_sample(impl, keys, vals, n, terms, dt, threshold, budget_s, cores, offset=0, per_rot_s=None):
    """Rotations spread over one whole Strang step (forward then reverse
    list), each applied to the given state, on the host cores: every
    stride-th rotation from `offset`, the stride chosen so the sample fits
    the wall budget.  Only the rotation calls themselves are timed.  Returns
    (input terms, seconds, rotations, stride)."""
    half = dt * 0.5
    order = list(terms) + list(reversed(terms))
    if per_rot_s is None:
        i, j, qi, qj, h = order[0]
        st, _, per_rot_s = impl.rotate_timed(keys, vals, n, i, j, qi, qj, h, half, threshold, cores)
        if st:
            raise RuntimeError(f"CPU rotation failed with status {st}")
    count = max(1, int(budget_s / max(per_rot_s, 1e-6)))
    stride = max(1, math.ceil(len(order) / count))
    done_terms, secs, rots = 0, 0.0, 0
    n_in = len(vals)
    t_wall = time.perf_counter()
    for r in range(offset % stride, len(order), stride):
        i, j, qi, qj, h = order[r]
        st, _, dt_s = impl.rotate_timed(keys, vals, n, i, j, qi, qj, h, half, threshold, cores)
        if st:
            raise RuntimeError(f"CPU sample rotation failed with status {st}")
        done_terms += n_in
        secs += dt_s
        rots += 1
        if time.perf_counter() - t_wall > 2.0 * budget_s:
            break
    return done_terms, secs, rots, stride


# ------------------------------------------------------------------ set-up
# Committed mid-trajectory state of the ring64 workload (made by
# tests/golden/make_window.py): both arms of the default line start from it,
# so neither needs the other's engine to reach the window.
WINDOW_STATE = {"ring64": os.path.join(ROOT, "tests", "golden", "ring64_window.npz")}


def window_state(cfg_name):
    """(keys, values, step) of the committed window state, or None."""
    path = WINDOW_STATE.get(cfg_name)
    if not path or not os.path.exists(path):
        return None
    z = np.load(path)
    return z["keys"], z["values"], int(z["steps"])


def workload_config(args, cfg, terms, words, start):
    """The `config` object shared by both arms (the workload only)."""
    c = {"workload": f"{args.config}_trajectory_window", "description": cfg["label"],
         "n_spins": cfg["n"], "key_words": words, "hamiltonian_terms": len(terms),
         "rotations_per_step": 2 * len(terms)}
    c.update(start)
    return c


def prepare_state(eng, cfg, target_terms, max_setup_steps, opts):
    terms = cfg["terms"]()
    k0, v0 = cfg["init"]()
    m = eng.map(cfg["n"], k0, v0)
    from ddevol_gb300.engine import GbLedger
    led = GbLedger()
    steps = 0
    while len(m) < target_terms and steps < max_setup_steps:
        chunk = 1 if len(m) > target_terms * 0.9 else 5
        st, _, led, msg = m.evolve(terms, cfg["dt"], chunk, opts, led, record_fid=False)
        if st:
            raise RuntimeError(f"set-up evolve failed: {msg}")
        steps += chunk
    return m, terms, led, steps


def algorithmic_bytes(words, n_in_sum, n_out_sum):
    return (8 * words + 8) * (n_in_sum + n_out_sum)


def read_traffic_profile(kernel, cfg_name, key="dram_bytes_per_input_term"):
    """Per-input-term bytes of `kernel` from the committed ncu summary
    (profiles/<kernel>_<config>.md, line '<key>: X'; DRAM by default)."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{cfg_name}.md")
    try:
        with open(path) as f:
            for line in f:
                if line.strip().startswith(key + ":"):
                    return float(line.split(":", 1)[1])
    except OSError:
        return None
    return None


def clocks_during(fn):
    """Runs fn() while nvidia-smi samples the clocks; returns (result, clocks)."""
    import torch
    sampler = ClockSampler(physical_gpu_index(torch.cuda.current_device() if torch.cuda.is_available()
                                              else 0))
    sampler.start()
    time.sleep(0.3)
    try:
        out = fn()
    finally:
        clocks = sampler.stop()
    return out, clocks


def run_gb300(args, dist):
    from ddevol_gb300.engine import Engine, GbLedger, options
    cfg = CONFIGS[args.config]
    words = (cfg["n"] + 31) // 32
    terms = cfg["terms"]()
    eng = Engine(dist.local_rank)
    exact = args.exact_ledger
    opts = options(cfg["threshold"], exact_ledger=exact, use_graphs=True)
    win = window_state(args.config) if not args.setup else None
    if win is not None:
        k_win, v_win, step0 = win
        m = eng.map(cfg["n"], k_win, v_win)
        led = GbLedger()
        start = {"window_state": os.path.relpath(WINDOW_STATE[args.config], ROOT),
                 "window_state_step": step0, "window_state_terms": int(len(v_win))}
    else:
        m, terms, led, step0 = prepare_state(eng, cfg, args.target_terms, args.max_setup_steps, opts)
        k_win, v_win = m.download()
        start = {"setup_steps": step0, "setup_target_terms": args.target_terms}
    # the engine's launch configuration for this workload: one timed step per
    # candidate from the start state (kept), the fastest applied (before the
    # warm-up; the e2e leg steps the same map)
    tuning, tuned = None, None
    if not args.no_autotune:
        t = m.autotune(terms, cfg["dt"], opts)
        tuned = t["chosen"]
        name = lambda c: (f"hash ctas={c['hash_ctas']} pdl={c['hash_pdl']} fuse={c['hash_fuse']}"
                          if c["hash_step"] else f"sorted pdl={c['sorted_pdl']}")
        tuning = {"chosen": name(t["chosen"]), "chosen_ms": round(t["chosen"]["step_ms"], 3),
                  "default": name(t["before"]), "default_ms": round(t["before"]["step_ms"], 3),
                  "tried_ms": {name(c): round(c["step_ms"], 3) for c in t["tried"][1:]},
                  "basis": "device time of one Strang step from the start state per candidate, "
                           "after one untimed step"}
    # With the hash-table step the per-phase CUDA events are part of each
    # step's graph, so the dominant kernel's launch time is measured on the
    # timed steps themselves; the warm-up steps capture that same graph.
    live_profile = m.engine_config()["hash_step"] == 1
    m.set_profiling(live_profile)
    for _ in range(args.warmup):
        st, _, led, msg = m.evolve(terms, cfg["dt"], 1, opts, led)
        if st:
            raise RuntimeError(msg)
    # the map at the start of the timed window: the e2e leg replays the same steps from it
    k_t0, v_t0 = m.download()
    led_t0 = GbLedger.from_buffer_copy(led)
    # ---- timed region: exactly K steps
    sampler = ClockSampler(physical_gpu_index(dist.local_rank))
    sampler.start()
    time.sleep(0.3)
    n_before = len(m)
    flush = L2Flush(dist.local_rank)
    ms, terms_done, launches, fids = 0.0, 0, 0, []
    m.set_profiling(live_profile)  # counters from zero
    flush()
    dist.barrier()
    profiler_range(True)
    for _ in range(args.steps):
        # one Strang step per call, device-timed on the engine's stream; the
        # L2 is flushed between timed steps (outside the timed interval)
        st, f, led, msg = m.evolve(terms, cfg["dt"], 1, opts, led)
        if st:
            raise RuntimeError(msg)
        ms += m.last_elapsed_ms()
        terms_done += m.last_terms()
        launches += m.last_launches()
        fids.extend(f)
        flush()
    profiler_range(False)
    dist.barrier()
    n_after = len(m)
    clocks = sampler.stop()
    t_max = dist.reduce(ms / 1e3, "max")
    terms_all = dist.reduce(float(terms_done), "sum")
    value = terms_all / t_max
    if live_profile:
        prof = m.kernel_profile()
        prof_terms, prof_n0, prof_n1 = terms_done, n_before, n_after
    else:
        # the sorted path's per-kernel events break its graph: one extra
        # profiled step after the timed region
        m.set_profiling(True)
        prof_n0 = len(m)
        st, _, led, msg = m.evolve(terms, cfg["dt"], 1, opts, led, record_fid=False)
        prof = m.kernel_profile()
        prof_terms, prof_n1 = m.last_terms(), len(m)
    m.set_profiling(False)
    rot_kernel = "k_hash_rotate" if "k_hash_rotate" in prof else "k_merge"
    rot = prof[rot_kernel][1] or 1
    total_ms = sum(v[0] for v in prof.values())
    dominant = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_n = prof[dominant]
    n_in_sum = prof_terms
    n_out_sum = prof_terms + (prof_n1 - prof_n0)
    bytes_per_launch = algorithmic_bytes(words, n_in_sum, n_out_sum) / rot
    peak, peak_kind = peaks()
    achieved = bytes_per_launch / (dom_ms / dom_n / 1e3) / 1e9
    path_achieved = algorithmic_bytes(words, n_in_sum, n_out_sum) / (total_ms / 1e3) / 1e9
    traffic_per_term = read_traffic_profile(dominant, args.config)
    traffic = None if traffic_per_term is None else traffic_per_term * (n_in_sum / rot)
    l2_per_term = read_traffic_profile(dominant, args.config, "l2_bytes_per_input_term")
    l2_traffic = None if l2_per_term is None else l2_per_term * (n_in_sum / rot)

    # ---- end to end through the C-ABI with pinned host buffers: the same K
    # steps from the same state, L2 flushed before each (outside the timed
    # interval), each step uploading the map, stepping, reading the FID and
    # downloading the map
    e2e = None
    try:
        import ctypes as C

        import torch

        from ddevol_gb300.engine import _f64p, _u64p
        cap = int(max(len(v_t0), n_after) * 1.6) + 4096
        hk = torch.empty(cap * words, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
        hv = torch.empty(cap, dtype=torch.float64, pin_memory=True).numpy()
        hk[:len(k_t0)] = k_t0
        hv[:len(v_t0)] = v_t0
        n_host = len(v_t0)
        led = GbLedger.from_buffer_copy(led_t0)
        e2e_terms, e2e_s, h2d, d2h, e2e_fids = 0, 0.0, 0, 0, []
        got = C.c_size_t()
        err = C.create_string_buffer(256)
        dist.barrier()
        for _ in range(args.steps):
            flush()
            t0 = time.perf_counter()
            st, msg = m.upload(hk[:n_host * words], hv[:n_host])
            if st:
                raise RuntimeError(msg)
            st, f, led, msg = m.evolve(terms, cfg["dt"], 1, opts, led)
            if st:
                raise RuntimeError(msg)
            if len(m) > cap:
                raise RuntimeError("e2e host buffer too small")
            st = m.lib.tpgp_gb_map_download(m.ptr, _u64p(hk), _f64p(hv), cap, C.byref(got), err, 256)
            if st:
                raise RuntimeError(err.value.decode())
            e2e_s += time.perf_counter() - t0
            e2e_terms += m.last_terms()
            e2e_fids.extend(f)
            h2d += n_host * (8 * words + 8)
            d2h += got.value * (8 * words + 8) + 8  # the map and the step's FID
            n_host = got.value
        dist.barrier()
        e2e_t = dist.reduce(e2e_s, "max")
        e2e_all = dist.reduce(float(e2e_terms), "sum")
        same = bool(np.array_equal(np.asarray(e2e_fids).view(np.uint64),
                                   np.asarray(fids).view(np.uint64)))
        e2e = {"value": e2e_all / e2e_t, "unit": METRIC, "h2d_bytes_per_step": h2d // args.steps,
               "d2h_bytes_per_step": d2h // args.steps, "steps": args.steps,
               "conditions": "same K steps from the same state; L2 flushed before each step; "
                             "FID read every step",
               "fids_equal_device_leg": same}
    except Exception as exc:  # reported, never silently replaced
        e2e = {"value": None, "unit": METRIC, "error": str(exc)[:200]}

    # ---- CPU baseline on a bounded sample of the window state (rank 0, N=1)
    cpu = None
    forms = None
    if dist.rank == 0 and dist.world == 1:
        if not args.no_cpu_baseline:
            impl, kind = cpu_engine()
            cores = os.cpu_count() or 1
            t_terms, secs, rots, stride = cpu_sample(impl, k_win, v_win, cfg["n"], terms, cfg["dt"],
                                                     cfg["threshold"], args.cpu_budget, cores)
            cpu = {"value": t_terms / secs, "unit": METRIC, "cores": cores, "kind": kind,
                   "sample": f"every {stride}th of the {2 * len(terms)} rotations of one Strang "
                             f"step ({rots} rotations, {t_terms} input terms, {secs:.1f} s of "
                             f"rotation calls), each applied to the {len(v_win)}-term window "
                             f"state"}
        if not args.no_forms:
            forms = run_forms(args, eng, k_win, v_win, terms, cfg, peak, tuned)
    m.close()
    eng.close()
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (trajectory generated from X_0; no dataset)",
        "config": workload_config(args, cfg, terms, words, start),
        "window": {"timed_steps_after_state": [args.warmup, args.warmup + args.steps],
                   "terms_at_timed_start": n_before, "terms_after": n_after,
                   "ledger": "exact (sequential, bitwise the reference's)" if exact
                             else "bound (fixed-point)",
                   "l2": f"map {n_before * (8 * words + 8) / 1e6:.1f} MB per buffer; L2 flushed "
                         f"(512 MB write) between timed steps"},
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": {
            "bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
            "l2_traffic": l2_traffic,
            "bytes_per_launch": bytes_per_launch, "launch_ms": dom_ms / dom_n,
            "kernel_share": dom_ms / total_ms,
            "measured_on": "the timed steps (events captured in the step graph)" if live_profile
                           else "one profiled step after the timed region",
            "path_achieved": path_achieved, "path_frac": path_achieved / peak,
            "kernel_ms": {k2: round(v2[0], 3) for k2, v2 in prof.items()}},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "engine_tuning": tuning,
        "fid_last": float(fids[-1]) if len(fids) else None,
        "forms": forms,
        "libraries": repo_libraries(),
    }
    return line


EXACT_FILE = os.path.join(ROOT, "tests", "golden", "exact.npz")


def plain_solve(eng, peak, budget_s=None, warm=True):
    """The plain single-solve path on the 16-spin J1-J2 ring: X_0, dt = 0.01,
    400 steps to t = 4, threshold 1e-6, 64-bit keys, through the public API
    (map created from host arrays, every step's FID returned to the host,
    the final map downloaded).  The map reaches ~1.3e8 terms, so the full
    solve takes minutes; with `budget_s` the solve stops after the step that
    crosses the wall budget and reports the steps it reached."""
    from ddevol_gb300.engine import GbLedger, options
    n, dt, steps, thr = 16, 0.01, 400, 1e-6
    terms = H.ring_j1j2(n)
    k0, v0 = H.single_site_operator(n)
    opts = options(thr, exact_ledger=False)

    def solve(limit):
        t0 = time.perf_counter()
        m = eng.map(n, k0, v0)
        led, fids, dev_ms, terms_done, launches, done = GbLedger(), [], 0.0, 0, 0, 0
        while done < steps and (limit is None or time.perf_counter() - t0 < limit):
            chunk = min(10, steps - done)
            st, f, led, msg = m.evolve(terms, dt, chunk, opts, led)
            if st:
                raise RuntimeError(msg)
            fids.extend(f)
            dev_ms += m.last_elapsed_ms()
            terms_done += m.last_terms()
            launches += m.last_launches()
            done += chunk
        k, v = m.download()
        wall = time.perf_counter() - t0
        out = dict(wall=wall, dev_ms=dev_ms, terms=terms_done, launches=launches,
                   fids=np.asarray(fids), peak=led.peak_terms, final=len(v), steps=done)
        m.close()
        return out

    if warm:
        solve(min(5.0, budget_s) if budget_s else 5.0)  # graph captures of the early table sizes
    r, clocks = clocks_during(lambda: solve(budget_s))
    path_bytes = algorithmic_bytes(1, r["terms"], r["terms"])
    complete = r["steps"] >= steps
    out = {"workload": "ring16 J1=1 J2=1/8, X_0, dt=0.01, 400 steps, threshold 1e-6",
           "ledger": "bound (fixed-point)",
           "steps_reached": r["steps"], "steps_total": steps, "complete": complete,
           "value": r["terms"] / r["wall"], "unit": METRIC,
           "device_value": r["terms"] / (r["dev_ms"] / 1e3),
           "wall_s": r["wall"], "device_s": r["dev_ms"] / 1e3, "peak_terms": int(r["peak"]),
           "final_terms": int(r["final"]), "gpu_launches": int(r["launches"]),
           "roofline": {"bound": "hbm", "achieved": path_bytes / (r["dev_ms"] / 1e3) / 1e9,
                        "peak": peak, "unit": "GB/s",
                        "frac": path_bytes / (r["dev_ms"] / 1e3) / 1e9 / peak,
                        "basis": "the steps run: (8W+8)(n_in+n_out) per rotation over device time"},
           "clocks": clocks}
    if complete:
        out["fid_solves_per_s"] = 1.0 / r["wall"]
    try:
        exact = np.load(EXACT_FILE)["ring16_exact"]
        k = r["steps"]
        out["fid_max_abs_dev_from_exact"] = float(np.max(np.abs(r["fids"][:k] - exact[1:k + 1])))
    except Exception:
        pass
    return out


def run_plain_solve(args, dist):
    """--config plain_solve: the full 400-step solve of the 16-spin ring as its own line."""
    from ddevol_gb300.engine import Engine
    eng = Engine(dist.local_rank)
    dist.barrier()
    r = plain_solve(eng, peaks()[0], budget_s=None, warm=False)
    dist.barrier()
    eng.close()
    return {"metric": METRIC, "value": r["value"], "unit": METRIC, "n_gpus": dist.world,
            "steps": r["steps_reached"], "warmup": 0, "ms_per_step": r["wall_s"] * 1e3 / r["steps_reached"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (X_0; no dataset)",
            "config": {"workload": "plain_solve", "description": r["workload"],
                       "ledger": "bound (fixed-point)", "parallelism": f"replicas x{dist.world}"},
            "plain_solve": r, "gpu_launches": r["gpu_launches"], "clocks": r["clocks"]}


def form_ledger(eng, k_win, v_win, terms, cfg, peak, exact, tuned):
    """One Strang step of the window with the given ledger (exact: the
    sequential, bitwise-reference sums, the ABI's default; else the
    fixed-point bound), under the headline's tuned engine configuration,
    after two untimed steps from the same state (graph capture, log and
    table sizing)."""
    from ddevol_gb300.engine import GbLedger, options
    opts = options(cfg["threshold"], exact_ledger=exact)
    m = eng.map(cfg["n"], k_win, v_win)
    if tuned:
        m.set_engine_config(**{k: v for k, v in tuned.items() if k != "step_ms"})
    for _ in range(2):
        st, _, _, msg = m.evolve(terms, cfg["dt"], 1, opts, GbLedger())
        if st:
            raise RuntimeError(msg)
        m.upload(k_win, v_win)
    st, _, _, msg = m.evolve(terms, cfg["dt"], 1, opts, GbLedger())
    if st:
        raise RuntimeError(msg)
    words = (cfg["n"] + 31) // 32
    t = m.last_terms()
    n1 = len(m)
    ms = m.last_elapsed_ms()
    m.close()
    b = algorithmic_bytes(words, t, t + n1 - len(v_win))
    return {"workload": "the ring64 window, one Strang step, "
                        + ("exact ledger" if exact else "bound ledger"), "value": t / (ms / 1e3),
            "unit": METRIC, "ms_per_step": ms,
            "roofline": {"bound": "hbm", "frac": b / (ms / 1e3) / 1e9 / peak, "peak": peak,
                         "basis": "whole step over device time"}}


def form_branch_abi(reps=10):
    """The reference-facing CUDA branch ABI (tpgp_cuda_branches, the
    reference's branch-backend interface) on 10^6 two-word terms from host
    memory: copies in, branch kernel, copies out, per call, timed on the
    host; beside it the branch loop of the CPU implementation (one thread)
    on the same input, and the bytes the call moves over the host link."""
    import ctypes as C

    from ddevol_gb300.engine import CudaBranchContext, _f64p, _u64p
    n, count, words = 64, 1_000_000, 2
    rng = np.random.default_rng(11)
    keys = rng.integers(0, 2 ** 63, size=count * words, dtype=np.int64).astype(np.uint64)
    vals = rng.standard_normal(count)
    i, j, qi, qj = 3, 40, 1, 1
    c, s = math.cos(0.01), math.sin(0.01)
    ok = np.zeros(2 * count * words, np.uint64)
    ov = np.zeros(2 * count, np.float64)
    orad = np.zeros(2 * count, np.float64)
    err = C.create_string_buffer(256)
    ctx = CudaBranchContext(0)
    try:
        def call():
            st = ctx.lib.tpgp_cuda_branches(ctx.ptr, _u64p(keys), _f64p(vals), count, words, n, i, j,
                                            qi, qj, c, s, 0.0, 0.0, 0, _u64p(ok), _f64p(ov),
                                            _f64p(orad), err, len(err))
            if st:
                raise RuntimeError(err.value.decode())
        for _ in range(2):
            call()
        t0 = time.perf_counter()
        for _ in range(reps):
            call()
        dt = (time.perf_counter() - t0) / reps
    finally:
        ctx.close()
    from oracle.oracle import Oracle, build_oracle
    build_oracle()
    impl, kind = Oracle(), "port"
    t0 = time.perf_counter()
    st, _, _, _ = impl.branches(keys, vals, n, i, j, qi, qj, c, s)
    cpu_dt = time.perf_counter() - t0
    moved = count * (8 * words + 8) + 2 * count * (8 * words + 8 + 8)  # in; keys, values, radii out
    return {"workload": "tpgp_cuda_branches, 10^6 terms, 128-bit keys, host arrays in and out",
            "value": count / dt, "unit": METRIC, "ms_per_call": dt * 1e3,
            "host_link_gbs": moved / dt / 1e9, "bytes_per_call": moved,
            "cpu_branch": {"value": count / cpu_dt, "unit": METRIC, "cores": 1, "kind": kind,
                           "status": st}}


def run_forms(args, eng, k_win, v_win, terms, cfg, peak, tuned=None):
    """Bounded sub-lines of the other forms, and one step of the window with
    the other ledger than the headline's."""
    forms = {}
    other = "bound_ledger" if args.exact_ledger else "exact_ledger"
    todo = [("plain_solve", lambda: plain_solve(eng, peak, budget_s=args.form_seconds)),
            (other, lambda: form_ledger(eng, k_win, v_win, terms, cfg, peak, not args.exact_ledger,
                                        tuned)),
            ("powder", lambda: powder_form(args, eng, peak)),
            ("serve", lambda: serve_form(args, eng, peak)),
            ("branch_abi", lambda: form_branch_abi())]
    for name, fn in todo:
        try:
            forms[name] = fn()
        except Exception as exc:  # reported, never silently replaced
            forms[name] = {"error": str(exc)[:300]}
    return forms


POWDER = dict(items=512, dt=0.01, threshold=1e-5, steps_total=300, seed=20260711,
              label="512 orientations uniform on the sphere (splitmix64 seed 20260711); each item "
                    "a cubic fragment of N uniform in {8..64} sites (first N sites of an open "
                    "4x4x4 block, r<=2, d=(1-3cos^2)/r^3 along the item's field), X_0, dt=0.01, "
                    "threshold 1e-5; 300 steps per solve")


def powder_items(count=POWDER["items"], seed=POWDER["seed"]):
    dirs = H.sphere_directions(count, seed=seed)
    rng = np.random.default_rng(seed)
    sizes = rng.integers(8, 65, size=count)
    return [(int(n), H.cubic_fragment(int(n), d)) for n, d in zip(sizes, dirs)]


def powder_run(args, eng, seed, budget_s):
    """The batched form: every orientation advanced per Strang step by one
    clustered launch per key width, replayed from a CUDA graph, for up to
    300 steps or `budget_s` of wall time after the warm-up and autotune."""
    from ddevol_gb300.engine import Batch, options
    items = powder_items(seed=seed)
    batch = Batch(eng, [n for n, _ in items])
    opts = options(POWDER["threshold"], exact_ledger=False)
    for k, (n, terms) in enumerate(items):
        batch.upload(k, *H.single_site_operator(n, 0))
        batch.set_terms(k, terms, POWDER["dt"], opts)
    t_start = time.perf_counter()
    batch.step(args.warmup)
    clusters = batch.autotune()
    tables = bool(batch.lib.tpgp_gb_batch_uses_tables(batch.ptr))
    widths = sorted({(n + 31) // 32 for n, _ in items})
    tuning = {w: t for w, t in batch.tuning().items() if w in widths}
    done = args.warmup
    ms, terms_done, launches, steps_timed = 0.0, 0, 0, 0
    t0 = time.perf_counter()
    while done < POWDER["steps_total"] and (steps_timed < args.steps or
                                            time.perf_counter() - t0 < budget_s):
        batch.step(1, record_fid=True)
        ms += batch.last_elapsed_ms()
        terms_done += batch.last_terms()
        launches += batch.last_launches()
        done += 1
        steps_timed += 1
    wall_all = time.perf_counter() - t_start
    sizes = [batch.item_len(k) for k in range(len(items))]
    failed = sum(1 for k in range(len(items)) if batch.item_status(k))
    batch.close()
    return dict(items=len(items), ms=ms, terms=terms_done, launches=launches, steps=steps_timed,
                reached=done, wall_all=wall_all, sizes=sizes, failed=failed, clusters=clusters,
                tables=tables, tuning=tuning)


def powder_summary(r, peak):
    complete = r["reached"] >= POWDER["steps_total"]
    per_step_s = r["ms"] / 1e3 / max(1, r["steps"])
    b = algorithmic_bytes(1.5, r["terms"], r["terms"])  # W = 1 or 2 per item: 40 B per term
    out = {"workload": "powder_batch", "ledger": "bound (fixed-point)", "items": r["items"],
           "value": r["terms"] / (r["ms"] / 1e3),
           "unit": METRIC, "steps_timed": r["steps"], "steps_reached": r["reached"],
           "steps_total": POWDER["steps_total"], "complete": complete,
           "ms_per_batched_step": per_step_s * 1e3,
           "fid_solves_per_s": r["items"] / (per_step_s * POWDER["steps_total"]),
           "fid_solves_per_s_basis": "items / (mean device time per batched step x 300 steps) "
                                     "over the steps timed",
           "terms_per_item_after": {"min": int(min(r["sizes"])), "median": int(np.median(r["sizes"])),
                                    "max": int(max(r["sizes"]))},
           "failed_items": r["failed"], "cluster_ctas_per_item": r["clusters"],
           "cta_local_tables": r["tables"], "gpu_launches": r["launches"],
           "autotuned": {str(w): v for w, v in r.get("tuning", {}).items()},
           "roofline": {"bound": "hbm", "peak": peak, "unit": "GB/s",
                        "achieved": b / (r["ms"] / 1e3) / 1e9,
                        "frac": b / (r["ms"] / 1e3) / 1e9 / peak,
                        "basis": "40 B per input term per rotation (W=1 and W=2 items) over "
                                 "device time"}}
    if complete:
        out["full_solve_wall_s"] = r["wall_all"]
        out["fid_solves_per_s_wall"] = r["items"] / r["wall_all"]
    return out


def powder_form(args, eng, peak):
    r, clocks = clocks_during(lambda: powder_run(args, eng, POWDER["seed"], args.form_seconds))
    out = powder_summary(r, peak)
    out["clocks"] = clocks
    return out


def run_powder(args, dist):
    """--config powder: the batched form as its own line."""
    from ddevol_gb300.engine import Engine
    eng = Engine(dist.local_rank)
    sampler = ClockSampler(physical_gpu_index(dist.local_rank))
    sampler.start()
    time.sleep(0.3)
    dist.barrier()
    r = powder_run(args, eng, POWDER["seed"] + 7919 * dist.rank,  # each replica its own orientations
                   args.full_budget if args.full_solve else 0.0)
    dist.barrier()
    clocks = sampler.stop()
    eng.close()
    t_max = dist.reduce(r["ms"] / 1e3, "max")
    terms_all = dist.reduce(float(r["terms"]), "sum")
    summary = powder_summary(r, peaks()[0])
    return {
        "metric": METRIC, "value": terms_all / t_max, "unit": METRIC, "n_gpus": dist.world,
        "steps": r["steps"], "warmup": args.warmup, "ms_per_step": t_max * 1e3 / max(1, r["steps"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded orientations and fragments; no dataset)",
        "config": {"workload": "powder_batch", "description": POWDER["label"],
                   "items": r["items"], "ledger": "bound (fixed-point)",
                   "parallelism": f"replicas x{dist.world}"},
        "powder": summary, "gpu_launches": r["launches"], "clocks": clocks,
    }


SERVE = dict(dt=0.01, cutoff=3, steps=(20, 80), slots=(32, 64, 64), seed=20261203,
             target_busy=0.8, memory_budget=200 << 30,
             label="Poisson stream of FID solves: ring or chain (p=1/2), N uniform in {16..96} "
                   "(key widths 1-3 words), d=g/r^3 with g~N(1,0.1) per pair, pairs within "
                   "ring/chain distance 3, threshold log-uniform in [1e-6,1e-4], steps uniform "
                   "in {20..80}, dt=0.01, X_0; slots 32/64/64 of 32/64/96 spins")


def serve_requests(count, rate, seed):
    from ddevol_gb300.engine import options
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=count)) if rate > 0 else np.zeros(count)
    reqs = []
    for k in range(count):
        n, terms, thr, steps, dt = H.serving_request(rng, steps_range=SERVE["steps"],
                                                     cutoff=SERVE["cutoff"], dt=SERVE["dt"])
        keys, vals = H.single_site_operator(n, 0)
        reqs.append(dict(arrival=float(arrivals[k]), n_spins=n, terms=terms, dt=dt, steps=steps,
                         options=options(thr, exact_ledger=False), keys=keys, values=vals))
    return reqs


def serve_run(eng, seed, seconds):
    """The serving form: a Poisson stream of FID solves through tpgp_gb_serve
    (continuous batching over the batched kernel) at 80% load.  Load is
    utilisation of the server's capacity: a saturation burst that fills
    every slot at t = 0 gives the service rate mu (solves/s with all slots
    busy), and requests arrive at 0.8 mu.  (The fraction of wall time with a
    tick running, reported as busy_fraction, is near 1 at any load that keeps
    one request in flight, so it cannot set the rate.)  Latency is finish
    minus arrival."""
    slots, budget = SERVE["slots"], SERVE["memory_budget"]
    reqs0 = serve_requests(int(sum(slots)), 0.0, seed + 1)
    _, _, st0 = eng.serve(reqs0, slots=slots, memory_budget=budget, record_fid=False)
    mu = len(reqs0) / st0["wall_seconds"]
    rate = SERVE["target_busy"] * mu
    calib = [{"saturation_requests": len(reqs0), "saturation_wall_s": st0["wall_seconds"],
              "service_rate_per_s": mu, "utilisation": SERVE["target_busy"]}]
    count = int(min(10000, max(32, rate * seconds)))
    reqs = serve_requests(count, rate, seed)
    resp, fids, st = eng.serve(reqs, slots=slots, memory_budget=budget)
    lat = np.array([r["finished"] - q["arrival"] for r, q in zip(resp, reqs)])
    wait = np.array([r["admitted"] - q["arrival"] for r, q in zip(resp, reqs)])
    failed = sum(1 for r in resp if r["status"])
    # replay a few requests alone: the served FIDs must be bitwise the same
    rng = np.random.default_rng(seed + 99)
    picks = sorted(rng.choice(count, size=min(4, count), replace=False).tolist())
    same = True
    for r in picks:
        _, f1, _ = eng.serve([dict(reqs[r], arrival=0.0)], slots=(1, 1, 1), memory_budget=budget)
        same &= bool(np.array_equal(f1[0].view(np.uint64), fids[r].view(np.uint64)))
    widths = np.array([(q["n_spins"] + 31) // 32 for q in reqs])
    return dict(count=count, rate=rate, calib=calib, st=st, lat=lat, wait=wait, failed=failed,
                picks=picks, same=same, widths=widths)


def serve_summary(r, peak):
    st = r["st"]
    b = algorithmic_bytes(2, st["terms"], st["terms"])  # key widths 1-3 words: 48 B per term
    return {"workload": "serve_stream", "ledger": "bound (fixed-point)", "requests": r["count"],
            "rate_per_s": r["rate"],
            "value": st["terms"] / st["wall_seconds"], "unit": METRIC,
            "fid_solves_per_s": (r["count"] - r["failed"]) / st["wall_seconds"],
            "latency_s_p50": float(np.percentile(r["lat"], 50)),
            "latency_s_p99": float(np.percentile(r["lat"], 99)),
            "queue_s_p50": float(np.percentile(r["wait"], 50)),
            "queue_s_p99": float(np.percentile(r["wait"], 99)),
            "busy_fraction": st["busy_seconds"] / st["wall_seconds"],
            "wall_s": st["wall_seconds"], "ticks": int(st["ticks"]),
            "max_active": int(st["max_active"]), "failed": r["failed"],
            "width_mix": {int(w): int((r["widths"] == w).sum()) for w in (1, 2, 3)},
            "calibration": r["calib"], "gpu_launches": int(st["launches"]),
            "replayed_alone_bitwise": {"requests": r["picks"], "equal": r["same"]},
            "roofline": {"bound": "hbm", "peak": peak, "unit": "GB/s",
                         "achieved": b / st["busy_seconds"] / 1e9,
                         "frac": b / st["busy_seconds"] / 1e9 / peak,
                         "basis": "48 B per input term per rotation over device-busy time"}}


def serve_form(args, eng, peak):
    r, clocks = clocks_during(lambda: serve_run(eng, SERVE["seed"], args.form_seconds))
    out = serve_summary(r, peak)
    out["clocks"] = clocks
    return out


def run_serve(args, dist):
    """--config serve: the serving form as its own line."""
    from ddevol_gb300.engine import Engine
    eng = Engine(dist.local_rank)
    seed = SERVE["seed"] + 7919 * dist.rank
    sampler = ClockSampler(physical_gpu_index(dist.local_rank))
    sampler.start()
    time.sleep(0.3)
    dist.barrier()
    r = serve_run(eng, seed, args.serve_seconds)
    dist.barrier()
    clocks = sampler.stop()
    eng.close()
    st = r["st"]
    wall = dist.reduce(st["wall_seconds"], "max")
    terms_all = dist.reduce(float(st["terms"]), "sum")
    return {
        "metric": METRIC, "value": terms_all / wall, "unit": METRIC, "n_gpus": dist.world,
        "steps": int(st["ticks"]), "warmup": len(r["calib"]) + 1,
        "ms_per_step": st["wall_seconds"] * 1e3 / max(1, st["ticks"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded request stream; no dataset)",
        "config": {"workload": "serve_stream", "description": SERVE["label"],
                   "ledger": "bound (fixed-point)", "parallelism": f"replicas x{dist.world}"},
        "serve": serve_summary(r, peaks()[0]), "gpu_launches": int(st["launches"]),
        "clocks": clocks,
    }


def run_reference(args, dist):
    """The reference algorithm on the host cores (rank 0 only), from the same
    committed window state as the device arm: each step is a bounded sample
    of rotations spread over one whole Strang step (every stride-th of the
    forward and reverse lists), each applied to the window state, with all
    host threads.  No GPU library is loaded."""
    if dist.rank != 0:
        return None
    cfg = CONFIGS[args.config]
    words = (cfg["n"] + 31) // 32
    terms = cfg["terms"]()
    win = window_state(args.config)
    if win is None:
        return {"impl": "reference",
                "unavailable": f"no committed window state for config {args.config}"}
    k, v, step0 = win
    start = {"window_state": os.path.relpath(WINDOW_STATE[args.config], ROOT),
             "window_state_step": step0, "window_state_terms": int(len(v))}
    impl, kind = cpu_engine()
    cores = os.cpu_count() or 1
    budget = max(2.0, args.cpu_budget / max(1, args.steps))
    i, j, qi, qj, h = terms[0]
    _, _, per_rot = impl.rotate_timed(k, v, cfg["n"], i, j, qi, qj, h, cfg["dt"] * 0.5,
                                      cfg["threshold"], cores)
    for w in range(args.warmup):
        cpu_sample(impl, k, v, cfg["n"], terms, cfg["dt"], cfg["threshold"], 0.5, cores,
                   offset=w, per_rot_s=per_rot)
    tot_terms, tot_s, tot_rot, stride = 0, 0.0, 0, 1
    for step in range(args.steps):
        t_terms, secs, rots, stride = cpu_sample(impl, k, v, cfg["n"], terms, cfg["dt"],
                                                 cfg["threshold"], budget, cores,
                                                 offset=step * 7919, per_rot_s=per_rot)
        tot_terms += t_terms
        tot_s += secs
        tot_rot += rots
    value = tot_terms / tot_s
    sample = (f"{args.steps} samples, each every {stride}th of the {2 * len(terms)} rotations of "
              f"one Strang step from a different offset ({tot_rot} rotations, {tot_terms} input "
              f"terms, {tot_s:.1f} s of rotation calls), each rotation applied to the "
              f"{len(v)}-term window state")
    # the serial backend beside the threaded one (the reference's serial and
    # openmp backends differ only in the branch loop's threads)
    s_terms, s_secs, s_rots, s_stride = cpu_sample(impl, k, v, cfg["n"], terms, cfg["dt"],
                                                   cfg["threshold"], min(5.0, budget), 1,
                                                   offset=3)
    backends = {
        "threads": {"value": value, "threads": cores,
                    "how": "branch loop on all host threads (OpenMP), sort and merge serial"},
        "serial": {"value": s_terms / s_secs, "threads": 1,
                   "sample": f"every {s_stride}th rotation of the step ({s_rots} rotations)"},
    }
    return {
        "metric": METRIC, "value": value, "unit": METRIC, "impl": "reference", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_s * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (trajectory generated from X_0; no dataset)",
        "config": workload_config(args, cfg, terms, words, start),
        "window": {"ledger": "exact (sequential)", "parallelism": f"{cores} host threads"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": kind,
                         "sample": sample},
        "backends": backends,
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "libraries": repo_libraries(),
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--config", choices=sorted(CONFIGS) + ["powder", "serve", "plain_solve"],
                    default="ring64")
    ap.add_argument("--full-solve", action="store_true",
                    help="powder: continue to 300 steps and report FID solves/s")
    ap.add_argument("--full-budget", type=float, default=120.0,
                    help="powder: wall-second budget for --full-solve")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="serve: length of the measured request stream at the calibrated rate")
    ap.add_argument("--setup", action="store_true",
                    help="evolve from the initial operator to --target-terms instead of "
                         "loading the committed window state")
    ap.add_argument("--target-terms", type=float, default=1e5,
                    help="set-up evolves until the map holds this many terms")
    ap.add_argument("--max-setup-steps", type=int, default=400)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the engine's default launch configuration (no tpgp_gb_map_autotune)")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the plain-solve, other-ledger, powder and serving sub-lines")
    ap.add_argument("--form-seconds", type=float, default=15.0,
                    help="wall budget of the plain-solve, powder and serving sub-lines")
    ap.add_argument("--exact-ledger", action="store_true",
                    help="time the ABI's default exact ledger (bitwise the reference's sequential "
                         "sums) instead of the fixed-point bound")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    dist = Dist()
    try:
        if args.config == "powder":
            line = run_powder(args, dist)
        elif args.config == "serve":
            line = run_serve(args, dist)
        elif args.config == "plain_solve":
            line = run_plain_solve(args, dist)
        elif args.impl == "reference":
            line = run_reference(args, dist)
        else:
            line = run_gb300(args, dist)
    finally:
        dist.close()
    if line is not None and dist.rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
