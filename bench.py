#!/usr/bin/env python
"""Pauli terms/s of the device-resident branch step on GB300.

Workload (default): the 64-spin periodic ring with all-pairs secular dipolar
couplings d = 1/r^3 (r the chord on a unit-spacing circle), observable X_0,
dt = 0.005, threshold 1e-5, 128-bit keys -- the larger plain-method benchmark
configuration.  Its full 1000-step trajectory is far too long for one bench
run, so a bench "step" is one Strang step (12,096 rotations) of a window of
that trajectory: the map is first evolved from X_0 (untimed set-up) until it
holds at least --target-terms terms, then W warm-up steps run, then exactly
K steps are timed.

Metric: Pauli terms/s = (sum over the timed rotations of the rotation's input
terms) / device time of the K steps (CUDA events on the engine's stream).

Extra keys: e2e (same metric through the C-ABI with host
buffers: every step uploads the map from pinned host memory, runs the step
and downloads the result), roofline (HBM bound, the dominant kernel's
algorithmic bytes per launch over its average launch time, from a profiled
step), cpu_baseline (the CPU oracle on a bounded sample of the same state),
clocks (nvidia-smi sampled during the timed region), gpu_launches.

--impl reference times the reference algorithm on the host cores instead
(the oracle port, or the reference engine itself where it was compiled).
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


def cpu_sample(keys, vals, n, terms, dt, threshold, budget_s, cores):
    """Rotations of one Strang step (forward order) on the CPU oracle, from the
    given state, until the wall budget is spent.  Returns (terms, seconds,
    rotations, kind)."""
    half = dt * 0.5
    impl, kind = None, "port"
    ref_so = os.path.join(ROOT, "oracle", "_ref", "libtpgp_ref.so")
    from oracle.oracle import Oracle
    impl = Oracle()
    if os.path.exists(ref_so):
        try:
            from oracle.oracle import Reference
            ref = Reference(ref_so)
            kind = "reference"
        except OSError:
            ref = None
    else:
        ref = None
    done_terms, rot = 0, 0
    k, v = keys, vals
    t0 = time.perf_counter()
    order = list(terms) + list(reversed(terms))
    while rot < len(order):
        i, j, qi, qj, h = order[rot]
        n_in = len(v)
        if ref is not None:
            # the reference engine, OpenMP backend, all cores (tpgp_rev.c:668-678)
            st, k, v, _ = ref.rotate(k, v, n, i, j, qi, qj, h * half, threshold=threshold,
                                     threads=cores, backend=2)
        else:
            st, k, v, _ = impl.rotate(k, v, n, i, j, qi, qj, h, half, threshold=threshold,
                                      threads=cores)
        if st:
            raise RuntimeError(f"CPU sample rotation failed with status {st}")
        done_terms += n_in
        rot += 1
        if time.perf_counter() - t0 > budget_s:
            break
    return done_terms, time.perf_counter() - t0, rot, kind


# ------------------------------------------------------------------ set-up
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


def run_gb300(args, dist):
    from ddevol_gb300.engine import Engine, options
    cfg = CONFIGS[args.config]
    words = (cfg["n"] + 31) // 32
    eng = Engine(dist.local_rank)
    opts = options(cfg["threshold"], exact_ledger=args.exact_ledger, use_graphs=True)
    m, terms, led, setup_steps = prepare_state(eng, cfg, args.target_terms, args.max_setup_steps,
                                               opts)
    n_start_window = len(m)
    for _ in range(args.warmup):
        st, _, led, msg = m.evolve(terms, cfg["dt"], 1, opts, led)
        if st:
            raise RuntimeError(msg)
    # ---- timed region: exactly K steps
    sampler = ClockSampler(physical_gpu_index(dist.local_rank))
    sampler.start()
    time.sleep(0.3)
    n_before = len(m)
    flush = L2Flush(dist.local_rank)
    ms, terms_done, launches, fids = 0.0, 0, 0, []
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

    # ---- profiled step (per-kernel CUDA events) for the roofline
    m.set_profiling(True)
    n_p0 = len(m)
    st, _, led, msg = m.evolve(terms, cfg["dt"], 1, opts, led, record_fid=False)
    prof = m.kernel_profile()
    prof_terms = m.last_terms()
    n_p1 = len(m)
    m.set_profiling(False)
    rot_kernel = "k_hash_rotate" if "k_hash_rotate" in prof else "k_merge"
    rot = prof[rot_kernel][1] or 1
    total_ms = sum(v[0] for v in prof.values())
    dominant = max(prof, key=lambda k: prof[k][0])
    dom_ms, dom_n = prof[dominant]
    n_in_sum = prof_terms
    n_out_sum = prof_terms + (n_p1 - n_p0)
    bytes_per_launch = algorithmic_bytes(words, n_in_sum, n_out_sum) / rot
    peak, peak_kind = peaks()
    achieved = bytes_per_launch / (dom_ms / dom_n / 1e3) / 1e9
    path_achieved = algorithmic_bytes(words, n_in_sum, n_out_sum) / (total_ms / 1e3) / 1e9
    traffic_per_term = read_traffic_profile(dominant, args.config)
    traffic = None if traffic_per_term is None else traffic_per_term * (n_in_sum / rot)
    l2_per_term = read_traffic_profile(dominant, args.config, "l2_bytes_per_input_term")
    l2_traffic = None if l2_per_term is None else l2_per_term * (n_in_sum / rot)

    # ---- end to end through the C-ABI with pinned host buffers
    e2e = None
    try:
        import torch
        cap = int(len(m) * 1.6) + 4096
        hk = torch.empty(cap * words, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
        hv = torch.empty(cap, dtype=torch.float64, pin_memory=True).numpy()
        k, v = m.download()
        hk[:len(k)] = k
        hv[:len(v)] = v
        n_host = len(v)
        e2e_terms, e2e_s, h2d, d2h = 0, 0.0, 0, 0
        e2e_steps = max(1, args.steps)
        dist.barrier()
        for _ in range(e2e_steps):
            t0 = time.perf_counter()
            st, msg = m.upload(hk[:n_host * words], hv[:n_host])
            if st:
                raise RuntimeError(msg)
            st, led, msg = m.strang_step(terms, cfg["dt"], opts, led)
            if st:
                raise RuntimeError(msg)
            n_new = len(m)
            if n_new > cap:
                raise RuntimeError("e2e host buffer too small")
            from ddevol_gb300.engine import _f64p, _u64p
            import ctypes as C
            got = C.c_size_t()
            err = C.create_string_buffer(256)
            st = m.lib.tpgp_gb_map_download(m.ptr, _u64p(hk), _f64p(hv), cap, C.byref(got), err,
                                            256)
            if st:
                raise RuntimeError(err.value.decode())
            e2e_s += time.perf_counter() - t0
            e2e_terms += m.last_terms()
            h2d += n_host * (8 * words + 8)
            d2h += got.value * (8 * words + 8)
            n_host = got.value
        dist.barrier()
        e2e_t = dist.reduce(e2e_s, "max")
        e2e_all = dist.reduce(float(e2e_terms), "sum")
        e2e = {"value": e2e_all / e2e_t, "unit": METRIC, "h2d_bytes_per_step": h2d // e2e_steps,
               "d2h_bytes_per_step": d2h // e2e_steps, "steps": e2e_steps}
    except Exception as exc:  # reported, never silently replaced
        e2e = {"value": None, "unit": METRIC, "error": str(exc)[:200]}

    # ---- CPU baseline on a bounded sample of the same state (rank 0, N=1)
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        k, v = m.download()
        cores = os.cpu_count() or 1
        t_terms, secs, rots, kind = cpu_sample(k, v, cfg["n"], terms, cfg["dt"], cfg["threshold"],
                                               args.cpu_budget, cores)
        cpu = {"value": t_terms / secs, "unit": METRIC, "cores": cores, "kind": kind,
               "sample": f"first {rots} rotations of one Strang step from the {len(v)}-term "
                         f"window state ({t_terms} input terms, {secs:.1f} s)"}
    m.close()
    eng.close()
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (trajectory generated from X_0; no dataset)",
        "config": {
            "workload": f"{args.config}_trajectory_window", "description": cfg["label"],
            "n_spins": cfg["n"], "key_words": words, "hamiltonian_terms": len(terms),
            "rotations_per_step": 2 * len(terms), "setup_steps": setup_steps,
            "window_start_step": setup_steps + args.warmup,
            "terms_at_window_start": n_before, "terms_after_window": n_after,
            "ledger": "exact (sequential)" if args.exact_ledger else "bound (fixed-point)",
            "l2": f"map {n_before * (8 * words + 8) / 1e6:.1f} MB per buffer; L2 flushed "
                  f"(512 MB write) between timed steps",
            "parallelism": f"replicas x{dist.world}"},
        "e2e": e2e,
        "gpu_launches": launches,
        "roofline": {
            "bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
            "l2_traffic": l2_traffic,
            "bytes_per_launch": bytes_per_launch, "launch_ms": dom_ms / dom_n,
            "kernel_share": dom_ms / total_ms,
            "path_achieved": path_achieved, "path_frac": path_achieved / peak,
            "kernel_ms": {k2: round(v2[0], 3) for k2, v2 in prof.items()}},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "fid_last": float(fids[-1]) if len(fids) else None,
    }
    return line


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


def run_powder(args, dist):
    """Batched form: every orientation advanced per Strang step by one
    clustered launch (per key width) replayed from a CUDA graph."""
    from ddevol_gb300.engine import Batch, Engine, options
    eng = Engine(dist.local_rank)
    items = powder_items(seed=POWDER["seed"] + 7919 * dist.rank)  # each replica its own orientations
    batch = Batch(eng, [n for n, _ in items])
    opts = options(POWDER["threshold"], exact_ledger=False)
    for k, (n, terms) in enumerate(items):
        batch.upload(k, *H.single_site_operator(n, 0))
        batch.set_terms(k, terms, POWDER["dt"], opts)
    batch.step(args.warmup)
    clusters = batch.autotune()
    tables = bool(batch.lib.tpgp_gb_batch_uses_tables(batch.ptr))
    sampler = ClockSampler(physical_gpu_index(dist.local_rank))
    sampler.start()
    time.sleep(0.3)
    flush = L2Flush(dist.local_rank)
    ms, terms_done, launches = 0.0, 0, 0
    flush()
    dist.barrier()
    profiler_range(True)
    for _ in range(args.steps):
        batch.step(1, record_fid=True)
        ms += batch.last_elapsed_ms()
        terms_done += batch.last_terms()
        launches += batch.last_launches()
        flush()
    profiler_range(False)
    dist.barrier()
    clocks = sampler.stop()
    t_max = dist.reduce(ms / 1e3, "max")
    terms_all = dist.reduce(float(terms_done), "sum")
    sizes = [batch.item_len(k) for k in range(len(items))]
    failed = sum(1 for k in range(len(items)) if batch.item_status(k))
    full = None
    if args.full_solve:
        # continue to the full 300 steps, bounded by a wall budget
        done = args.warmup + args.steps
        t0 = time.perf_counter()
        dev_ms = 0.0
        while done < POWDER["steps_total"] and time.perf_counter() - t0 < args.full_budget:
            batch.step(1, record_fid=True)
            dev_ms += batch.last_elapsed_ms()
            done += 1
        full = {"items": len(items), "steps_reached": done, "steps_total": POWDER["steps_total"],
                "device_s_after_window": dev_ms / 1e3,
                "complete": done >= POWDER["steps_total"]}
        if full["complete"]:
            # warm-up steps ran untimed: charge them at the first timed step's rate
            total_s = (ms + dev_ms) / 1e3 + args.warmup * (ms / 1e3 / args.steps)
            full["fid_solves_per_s"] = len(items) / total_s
    batch.close()
    eng.close()
    return {
        "metric": METRIC, "value": terms_all / t_max, "unit": METRIC, "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded orientations and fragments; no dataset)",
        "config": {"workload": "powder_batch", "description": POWDER["label"],
                   "items": len(items), "window_steps": [args.warmup, args.warmup + args.steps],
                   "terms_per_item_after": {"min": int(min(sizes)), "median": int(np.median(sizes)),
                                            "max": int(max(sizes))},
                   "cluster_ctas_per_item": clusters, "cta_local_tables": tables,
                   "failed_items": failed,
                   "ledger": "bound (fixed-point)",
                   "l2": "L2 flushed (512 MB write) between timed steps",
                   "parallelism": f"replicas x{dist.world}"},
        "item_step_solves_per_s": len(items) * args.steps / t_max,
        "full_solve": full,
        "gpu_launches": launches, "clocks": clocks,
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


def run_serve(args, dist):
    """Serving form: a Poisson stream of FID solves through tpgp_gb_serve
    (continuous batching over the batched kernel).  The arrival rate is
    calibrated in two short runs so that the device is busy about 80% of
    the wall time; latency is finish minus arrival."""
    from ddevol_gb300.engine import Engine
    eng = Engine(dist.local_rank)
    seed = SERVE["seed"] + 7919 * dist.rank
    slots, budget = SERVE["slots"], SERVE["memory_budget"]
    # saturation: every request present at t = 0
    burst = serve_requests(96, 0.0, seed + 1)
    _, _, st0 = eng.serve(burst, slots=slots, memory_budget=budget, record_fid=False)
    mu = len(burst) / st0["wall_seconds"]
    rate = SERVE["target_busy"] * mu
    calib = []
    for _ in range(2):
        trial = serve_requests(max(48, int(rate * 8)), rate, seed + 2 + len(calib))
        _, _, st1 = eng.serve(trial, slots=slots, memory_budget=budget, record_fid=False)
        busy = st1["busy_seconds"] / st1["wall_seconds"]
        calib.append({"rate": rate, "requests": len(trial), "busy": busy})
        rate *= SERVE["target_busy"] / max(busy, 1e-3)
    count = int(min(10000, max(64, rate * args.serve_seconds)))
    reqs = serve_requests(count, rate, seed)
    sampler = ClockSampler(physical_gpu_index(dist.local_rank))
    sampler.start()
    time.sleep(0.3)
    dist.barrier()
    profiler_range(True)
    resp, fids, st = eng.serve(reqs, slots=slots, memory_budget=budget)
    profiler_range(False)
    dist.barrier()
    clocks = sampler.stop()
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
    eng.close()
    wall = dist.reduce(st["wall_seconds"], "max")
    terms_all = dist.reduce(float(st["terms"]), "sum")
    solves_all = dist.reduce(float(count - failed), "sum")
    widths = np.array([(q["n_spins"] + 31) // 32 for q in reqs])
    return {
        "metric": METRIC, "value": terms_all / wall, "unit": METRIC, "n_gpus": dist.world,
        "steps": int(st["ticks"]), "warmup": len(calib) + 1,
        "ms_per_step": st["wall_seconds"] * 1e3 / max(1, st["ticks"]),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded request stream; no dataset)",
        "config": {"workload": "serve_stream", "description": SERVE["label"], "requests": count,
                   "rate_per_s": rate, "width_mix": {w: int((widths == w).sum()) for w in (1, 2, 3)},
                   "calibration": calib, "ledger": "bound (fixed-point)",
                   "parallelism": f"replicas x{dist.world}"},
        "serve": {"solves_per_s": solves_all / wall, "latency_s_p50": float(np.percentile(lat, 50)),
                  "latency_s_p99": float(np.percentile(lat, 99)),
                  "queue_s_p50": float(np.percentile(wait, 50)),
                  "queue_s_p99": float(np.percentile(wait, 99)),
                  "busy_fraction": st["busy_seconds"] / st["wall_seconds"],
                  "wall_s": st["wall_seconds"], "ticks": int(st["ticks"]),
                  "max_active": int(st["max_active"]), "failed": failed,
                  "replayed_alone_bitwise": {"requests": picks, "equal": same}},
        "gpu_launches": int(st["launches"]), "clocks": clocks,
    }


def run_reference(args, dist):
    """The reference algorithm on the host cores, on samples of the same state."""
    if dist.rank != 0:
        return None
    from ddevol_gb300.engine import Engine, options
    cfg = CONFIGS[args.config]
    words = (cfg["n"] + 31) // 32
    # set-up only: the window-start state comes from the device engine (untimed);
    # keys and values do not depend on the ledger mode, so the fast ledger is used
    eng = Engine(dist.local_rank)
    opts = options(cfg["threshold"], exact_ledger=False)
    m, terms, _, setup_steps = prepare_state(eng, cfg, args.target_terms, args.max_setup_steps,
                                             opts)
    k, v = m.download()
    m.close()
    eng.close()
    cores = os.cpu_count() or 1
    budget = max(2.0, args.cpu_budget / max(1, args.steps))
    for _ in range(args.warmup):
        cpu_sample(k, v, cfg["n"], terms, cfg["dt"], cfg["threshold"], min(budget, 2.0), cores)
    tot_terms, tot_s, tot_rot, kind = 0, 0.0, 0, "port"
    for _ in range(args.steps):
        t_terms, secs, rots, kind = cpu_sample(k, v, cfg["n"], terms, cfg["dt"], cfg["threshold"],
                                               budget, cores)
        tot_terms += t_terms
        tot_s += secs
        tot_rot += rots
    value = tot_terms / tot_s
    sample = (f"{args.steps} samples of the first rotations of one Strang step from the "
              f"{len(v)}-term window state ({tot_rot} rotations, {tot_terms} input terms)")
    return {
        "metric": METRIC, "value": value, "unit": METRIC, "impl": "reference", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_s * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (trajectory generated from X_0; no dataset)",
        "config": {"workload": f"{args.config}_trajectory_window", "description": cfg["label"],
                   "n_spins": cfg["n"], "key_words": words, "hamiltonian_terms": len(terms),
                   "rotations_per_step": 2 * len(terms), "setup_steps": setup_steps,
                   "terms_at_window_start": len(v), "ledger": "exact (sequential)",
                   "parallelism": "host cores"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--config", choices=sorted(CONFIGS) + ["powder", "serve"], default="ring64")
    ap.add_argument("--full-solve", action="store_true",
                    help="powder: continue to 300 steps and report FID solves/s")
    ap.add_argument("--full-budget", type=float, default=120.0,
                    help="powder: wall-second budget for --full-solve")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="serve: length of the measured request stream at the calibrated rate")
    ap.add_argument("--target-terms", type=float, default=1e5,
                    help="set-up evolves until the map holds this many terms")
    ap.add_argument("--max-setup-steps", type=int, default=400)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--exact-ledger", action="store_true",
                    help="bitwise reference ledger (one sequential sum per rotation)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    dist = Dist()
    try:
        if args.config == "powder":
            line = run_powder(args, dist)
        elif args.config == "serve":
            line = run_serve(args, dist)
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
