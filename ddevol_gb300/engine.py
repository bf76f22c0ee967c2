"""Python mirror of the reference engine's operator interface, on the GB300 library.

The names follow DDevol's C API (engine/include/tpgp_rev.h and
engine/include/tpgp_cuda_rev.h) so that tests and drivers read like the
reference's own:

* :class:`CudaBranchContext` -- ``tpgp_cuda_create`` / ``tpgp_cuda_branches``
  (the raw branch backend the reference engine calls per rotation);
* :class:`Engine` / :class:`DeviceMap` -- a device-resident ``tpgp_map`` with
  ``rotate`` (``tpgp_rotate``), ``strang_step`` (``tpgp_strang_step``),
  ``evolve`` (the CLI time loop) and ``single_sum`` (``tpgp_map_single_sum``).

Statuses are returned as the reference's integers (0 = ok, 1 = EINVAL, ...);
``STATUS_NAMES`` maps them to names.  Every call runs on the GPU; nothing
here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native
from .native import (CUDA_STATUS_NAMES, STATUS_NAMES, GbLedger, GbOptions, GbRequest,
                     GbResponse, GbServeStats, GbTerm)

__all__ = ["CudaBranchContext", "Engine", "DeviceMap", "Batch", "options", "terms_array",
           "STATUS_NAMES", "CUDA_STATUS_NAMES", "GbLedger"]


def _u64p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


def _f64p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def options(threshold=0.0, max_terms=0, max_drop_l2=0.0, exact_ledger=True, use_graphs=True,
            wait_polls=0):
    """tpgp_gb_options.  exact_ledger=True: the reference's sequential
    removed-weight ledger, bitwise; exact_ledger=False: the fixed-point bound
    ledger (a certified upper bound a few ulps from it).  Keys, values and
    FIDs are the same either way, and with either ledger maps up to 6e5 terms
    step on the hash-table kernels.  wait_polls: poll limit of the
    device-side waits (0: the defaults)."""
    return GbOptions(float(threshold), int(max_terms), float(max_drop_l2), int(bool(exact_ledger)),
                     int(bool(use_graphs)), int(wait_polls))


def terms_array(terms):
    terms = list(terms)
    arr = (GbTerm * max(1, len(terms)))()
    for k, (i, j, qi, qj, h) in enumerate(terms):
        arr[k] = GbTerm(i, j, qi, qj, h, k)
    return arr, len(terms)


class CudaBranchContext:
    """Reference-compatible branch backend context (tpgp_cuda_rev.h)."""

    def __init__(self, device: int = 0):
        self.lib = native.load()
        err = C.create_string_buffer(512)
        self.ptr = self.lib.tpgp_cuda_create(device, err, len(err))
        if not self.ptr:
            raise RuntimeError(f"tpgp_cuda_create failed: {err.value.decode()}")

    @property
    def name(self) -> str:
        return self.lib.tpgp_cuda_device_name(self.ptr).decode()

    def branches(self, keys, values, n_spins, i, j, qi, qj, c, s, rc=0.0, rs=0.0, enclose=0,
                 words=None):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        values = np.ascontiguousarray(values, dtype=np.float64)
        words = (n_spins + 31) // 32 if words is None else words
        count = len(values)
        ok = np.zeros(max(1, 2 * count * words), np.uint64)
        ov = np.zeros(max(1, 2 * count), np.float64)
        orad = np.zeros(max(1, 2 * count), np.float64)
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_cuda_branches(self.ptr, _u64p(keys), _f64p(values), count, words,
                                         n_spins, i, j, qi, qj, c, s, rc, rs, enclose, _u64p(ok),
                                         _f64p(ov), _f64p(orad), err, len(err))
        return st, ok[:2 * count * words], ov[:2 * count], orad[:2 * count], err.value.decode()

    def close(self):
        if self.ptr:
            self.lib.tpgp_cuda_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine:
    """One GB300 device and stream (tpgp_gb_create)."""

    def __init__(self, device: int = 0):
        self.lib = native.load()
        err = C.create_string_buffer(512)
        self.ptr = self.lib.tpgp_gb_create(device, err, len(err))
        if not self.ptr:
            raise RuntimeError(f"tpgp_gb_create failed: {err.value.decode()}")

    @property
    def name(self) -> str:
        return self.lib.tpgp_gb_device_name(self.ptr).decode()

    def map(self, n_spins: int, keys=None, values=None) -> "DeviceMap":
        m = DeviceMap(self, n_spins)
        if keys is not None:
            st, msg = m.upload(keys, values)
            if st:
                m.close()
                raise ValueError(f"upload failed ({STATUS_NAMES[st]}): {msg}")
        return m

    def upward_sums(self, x, chain):
        """Upward sums of consecutive chains of `chain` addends on the device
        (tpgp_gb_upward_sums): bit for bit the sequential upadd chain."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.zeros(max(0, -(-len(x) // chain)), dtype=np.float64)
        f64p = C.POINTER(C.c_double)
        st = self.lib.tpgp_gb_upward_sums(self.ptr, x.ctypes.data_as(f64p), len(x), chain,
                                          out.ctypes.data_as(f64p))
        if st:
            raise RuntimeError(f"tpgp_gb_upward_sums failed ({STATUS_NAMES[st]})")
        return out

    def serve(self, requests, slots=(8, 8, 8), memory_budget=64 << 30, record_fid=True):
        """Serves FID-solve requests with continuous batching (tpgp_gb_serve).

        requests: dicts with arrival (s), n_spins, terms, dt, steps, options,
        keys, values.  Returns (responses as dicts, per-request FID arrays,
        stats as a dict)."""
        n = len(requests)
        reqs = (GbRequest * max(1, n))()
        keep = []
        for r, q in enumerate(requests):
            arr, count = terms_array(q["terms"])
            keys = np.ascontiguousarray(q["keys"], dtype=np.uint64)
            vals = np.ascontiguousarray(q["values"], dtype=np.float64)
            keep += [arr, keys, vals]
            reqs[r] = GbRequest(float(q["arrival"]), int(q["n_spins"]), arr, count, float(q["dt"]),
                                int(q["steps"]), q["options"], _u64p(keys), _f64p(vals), len(vals))
        total = sum(int(q["steps"]) for q in requests)
        fids = np.zeros(max(1, total), np.float64)
        resp = (GbResponse * max(1, n))()
        slot_arr = (C.c_size_t * 3)(*slots)
        stats = GbServeStats()
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_serve(self.ptr, reqs, n, slot_arr, int(memory_budget),
                                    _f64p(fids) if record_fid else None, resp, C.byref(stats), err,
                                    len(err))
        if st:
            raise RuntimeError(f"serve failed ({STATUS_NAMES[st]}): {err.value.decode()}")
        out, per, off = [], [], 0
        for r, q in enumerate(requests):
            x = resp[r]
            out.append({name: getattr(x, name) for name, _ in GbResponse._fields_})
            per.append(fids[off:off + int(q["steps"])].copy())
            off += int(q["steps"])
        return out, per, {name: getattr(stats, name) for name, _ in GbServeStats._fields_}

    def close(self):
        if self.ptr:
            self.lib.tpgp_gb_destroy(self.ptr)
            self.ptr = None


class DeviceMap:
    """A tpgp_map kept in HBM between rotations (tpgp_gb_map)."""

    def __init__(self, engine: Engine, n_spins: int):
        self.engine = engine
        self.lib = engine.lib
        self.n_spins = n_spins
        self.n_words = (n_spins + 31) // 32
        ptr = C.c_void_p()
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_map_create(engine.ptr, n_spins, C.byref(ptr), err, len(err))
        if st:
            raise RuntimeError(f"tpgp_gb_map_create failed: {err.value.decode()}")
        self.ptr = ptr
        self._terms_cache = (None, None, 0)

    def __len__(self):
        return self.lib.tpgp_gb_map_len(self.ptr)

    def upload(self, keys, values):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        values = np.ascontiguousarray(values, dtype=np.float64)
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_map_upload(self.ptr, _u64p(keys), _f64p(values), len(values), err,
                                         len(err))
        return st, err.value.decode()

    def download(self):
        n = len(self)
        keys = np.zeros(max(1, n * self.n_words), np.uint64)
        values = np.zeros(max(1, n), np.float64)
        got = C.c_size_t()
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_map_download(self.ptr, _u64p(keys), _f64p(values), n, C.byref(got),
                                           err, len(err))
        if st:
            raise RuntimeError(f"download failed: {err.value.decode()}")
        return keys[:got.value * self.n_words], values[:got.value]

    def rotate(self, i, j, qi, qj, theta, opts=None, ledger=None):
        opts = opts if opts is not None else options()
        ledger = ledger if ledger is not None else GbLedger()
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_rotate(self.ptr, i, j, qi, qj, theta, C.byref(opts),
                                     C.byref(ledger), err, len(err))
        return st, ledger, err.value.decode()

    def _terms(self, terms):
        # the ctypes array is rebuilt only when a different term list is passed
        if self._terms_cache[0] is not terms:
            arr, count = terms_array(terms)
            self._terms_cache = (terms, arr, count)
        return self._terms_cache[1], self._terms_cache[2]

    def strang_step(self, terms, dt, opts=None, ledger=None):
        opts = opts if opts is not None else options()
        ledger = ledger if ledger is not None else GbLedger()
        arr, count = self._terms(terms)
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_strang_step(self.ptr, arr, count, dt, C.byref(opts),
                                          C.byref(ledger), err, len(err))
        return st, ledger, err.value.decode()

    def rotate_enclosed(self, rotations, opts=None, ledger=None):
        """Validated rotations (tpgp_gb_rotate_enclosed): rotations are
        (i, j, qi, qj, c, s, rc, rs) tuples.  Returns (status, ledger, message)."""
        opts = opts if opts is not None else options()
        ledger = ledger if ledger is not None else GbLedger()
        rots = list(rotations)
        arr = (native.GbRotation * max(1, len(rots)))()
        for k, r in enumerate(rots):
            arr[k] = native.GbRotation(*r)
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_rotate_enclosed(self.ptr, arr, len(rots), C.byref(opts),
                                              C.byref(ledger), err, len(err))
        return st, ledger, err.value.decode()

    def autotune(self, terms, dt, opts=None):
        """Times one step per candidate engine configuration from the current
        state (which is kept) and applies the fastest (tpgp_gb_map_autotune).
        Returns {"chosen", "before", "tried"} as dicts."""
        opts = opts if opts is not None else options()
        arr, count = self._terms(terms)
        tuning = native.GbTuning()
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_map_autotune(self.ptr, arr, count, dt, C.byref(opts), C.byref(tuning),
                                           err, len(err))
        if st:
            raise RuntimeError(f"autotune failed ({STATUS_NAMES[st]}): {err.value.decode()}")
        return {"chosen": tuning.chosen.as_dict(), "before": tuning.before.as_dict(),
                "tried": [tuning.tried[k].as_dict() for k in range(tuning.tried_count)]}

    def engine_config(self):
        c = native.GbEngineConfig()
        if self.lib.tpgp_gb_map_get_config(self.ptr, C.byref(c)):
            raise RuntimeError("tpgp_gb_map_get_config failed")
        return c.as_dict()

    def set_engine_config(self, **fields):
        c = native.GbEngineConfig()
        if self.lib.tpgp_gb_map_get_config(self.ptr, C.byref(c)):
            raise RuntimeError("tpgp_gb_map_get_config failed")
        for k, v in fields.items():
            setattr(c, k, v)
        if self.lib.tpgp_gb_map_set_config(self.ptr, C.byref(c)):
            raise ValueError(f"invalid engine configuration {fields}")

    def evolve(self, terms, dt, steps, opts=None, ledger=None, record_fid=True):
        opts = opts if opts is not None else options()
        ledger = ledger if ledger is not None else GbLedger()
        arr, count = self._terms(terms)
        fids = np.zeros(max(1, steps), np.float64)
        done = C.c_size_t()
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_evolve(self.ptr, arr, count, dt, steps, C.byref(opts),
                                     C.byref(ledger), _f64p(fids) if record_fid else None,
                                     C.byref(done), err, len(err))
        return st, fids[:done.value], ledger, err.value.decode()

    def liouvillian(self, terms, out=None):
        """out <- -i[H, self] (tpgp_gb_liouvillian); out defaults to a new map
        of the same spin count.  Returns (status, out map, message)."""
        out = out if out is not None else self.engine.map(self.n_spins)
        arr, count = terms_array(terms)
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_liouvillian(out.ptr, self.ptr, arr, count, err, len(err))
        return st, out, err.value.decode()

    def single_sum(self, pauli=1):
        out = C.c_double()
        st = self.lib.tpgp_gb_single_sum(self.ptr, pauli, C.byref(out))
        if st:
            raise RuntimeError(f"single_sum failed: {STATUS_NAMES[st]}")
        return out.value

    def last_elapsed_ms(self):
        return self.lib.tpgp_gb_last_elapsed_ms(self.ptr)

    def last_launches(self):
        return self.lib.tpgp_gb_last_launches(self.ptr)

    def last_terms(self):
        return self.lib.tpgp_gb_last_terms(self.ptr)

    KERNELS = ("k_classify", "k_flip_sort", "k_partition", "k_merge", "k_hash_rotate",
               "k_hash_build", "k_hash_chain_extract", "k_radix_sort", "k_hash_exact_ledger")

    def set_profiling(self, on=True):
        self.lib.tpgp_gb_set_profiling(self.ptr, int(bool(on)))

    def kernel_profile(self):
        ms = (C.c_double * len(self.KERNELS))()
        n = (C.c_size_t * len(self.KERNELS))()
        self.lib.tpgp_gb_kernel_profile(self.ptr, ms, n)
        return {k: (ms[i], n[i]) for i, k in enumerate(self.KERNELS) if n[i]}

    def close(self):
        if getattr(self, "ptr", None):
            self.lib.tpgp_gb_map_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent maps advanced together (tpgp_gb_batch)."""

    def __init__(self, engine: Engine, n_spins_list):
        self.engine = engine
        self.lib = engine.lib
        self.n_spins = [int(n) for n in n_spins_list]
        arr = (C.c_size_t * len(self.n_spins))(*self.n_spins)
        ptr = C.c_void_p()
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_batch_create(engine.ptr, len(self.n_spins), arr, C.byref(ptr), err,
                                           len(err))
        if st:
            raise RuntimeError(f"tpgp_gb_batch_create failed: {err.value.decode()}")
        self.ptr = ptr
        self._keep = {}

    def __len__(self):
        return len(self.n_spins)

    def upload(self, item, keys, values):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        values = np.ascontiguousarray(values, dtype=np.float64)
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_batch_upload(self.ptr, item, _u64p(keys), _f64p(values), len(values),
                                           err, len(err))
        if st:
            raise ValueError(f"batch upload failed: {err.value.decode()}")

    def set_terms(self, item, terms, dt, opts):
        arr, count = terms_array(terms)
        self._keep[item] = arr
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_batch_set_terms(self.ptr, item, arr, count, dt, C.byref(opts), err,
                                              len(err))
        if st:
            raise ValueError(f"batch set_terms failed ({STATUS_NAMES[st]}): {err.value.decode()}")

    def step(self, steps=1, record_fid=True):
        fids = np.zeros((max(1, steps), len(self)), np.float64)
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_batch_step(self.ptr, steps, _f64p(fids) if record_fid else None,
                                         err, len(err))
        if st:
            raise RuntimeError(f"batch step failed: {err.value.decode()}")
        return fids[:steps]

    def autotune(self):
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_batch_autotune(self.ptr, err, len(err))
        if st:
            raise RuntimeError(f"autotune failed: {err.value.decode()}")
        return {w: self.lib.tpgp_gb_batch_cluster(self.ptr, w) for w in (1, 2, 3, 4)}

    def tuning(self):
        """Per key width: base cluster size, terms per CTA of the size rule and
        CTA-local table slots per expected claim (tpgp_gb_batch_get_tuning)."""
        out = {}
        for w in (1, 2, 3, 4):
            c, p, f = C.c_int(), C.c_size_t(), C.c_double()
            st = self.lib.tpgp_gb_batch_get_tuning(self.ptr, w, C.byref(c), C.byref(p), C.byref(f))
            if st:
                raise ValueError(f"batch tuning query failed ({STATUS_NAMES[st]})")
            out[w] = {"cluster": c.value, "terms_per_cta": p.value, "table_slots_per_claim": f.value}
        return out

    def set_cluster(self, n_words, base, terms_per_cta=0):
        """Base cluster size and terms per CTA of the size rule for one key width."""
        err = C.create_string_buffer(256)
        st = self.lib.tpgp_gb_batch_set_cluster(self.ptr, n_words, base, terms_per_cta, err,
                                                len(err))
        if st:
            raise ValueError(err.value.decode())

    def max_cluster(self, n_words):
        return self.lib.tpgp_gb_batch_max_cluster(self.ptr, n_words)

    def item_status(self, item):
        return self.lib.tpgp_gb_batch_item_status(self.ptr, item)

    def item_len(self, item):
        return self.lib.tpgp_gb_batch_len(self.ptr, item)

    def ledger(self, item):
        led = GbLedger()
        self.lib.tpgp_gb_batch_ledger(self.ptr, item, C.byref(led))
        return led

    def download(self, item):
        n = self.item_len(item)
        words = (self.n_spins[item] + 31) // 32
        keys = np.zeros(max(1, n * words), np.uint64)
        values = np.zeros(max(1, n), np.float64)
        got = C.c_size_t()
        err = C.create_string_buffer(512)
        st = self.lib.tpgp_gb_batch_download(self.ptr, item, _u64p(keys), _f64p(values), n,
                                             C.byref(got), err, len(err))
        if st:
            raise RuntimeError(f"batch download failed: {err.value.decode()}")
        return keys[:got.value * words], values[:got.value]

    def last_elapsed_ms(self):
        return self.lib.tpgp_gb_batch_last_elapsed_ms(self.ptr)

    def last_terms(self):
        return self.lib.tpgp_gb_batch_last_terms(self.ptr)

    def last_launches(self):
        return self.lib.tpgp_gb_batch_last_launches(self.ptr)

    def close(self):
        if getattr(self, "ptr", None):
            self.lib.tpgp_gb_batch_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
