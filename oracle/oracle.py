"""ctypes front-end for the CPU oracle (test infrastructure only).

Two back-ends share one interface:

* ``Oracle`` loads ``oracle/_build/liborc.so`` -- the plain-C restatement in
  ``oracle/tpgp_oracle.c`` of the reference engine's rotation, Strang step and
  readout (DDevol engine/src/tpgp_rev.c:311-338, 432-809).
* ``Reference`` loads ``oracle/_ref/libtpgp_ref.so`` -- the reference engine
  itself, compiled from its own sources by ``oracle/Makefile``.  It exists
  only where the reference checkout exists; it pins the restatement
  (tests/golden/make_golden.py) and is never shipped.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the CUDA product path never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liborc.so")
REFERENCE_SO = os.path.join(HERE, "_ref", "libtpgp_ref.so")

STATUS_NAMES = ["ok", "einval", "enomem", "ecap", "enumeric", "ebackend", "ebudget"]


class MapStruct(C.Structure):
    """Field layout of tpgp_map (engine/include/tpgp_rev.h:25-29)."""

    _fields_ = [
        ("n_spins", C.c_size_t),
        ("n_words", C.c_size_t),
        ("len", C.c_size_t),
        ("capacity", C.c_size_t),
        ("keys", C.POINTER(C.c_uint64)),
        ("values", C.POINTER(C.c_double)),
    ]


class TermStruct(C.Structure):
    """Field layout of tpgp_term (engine/include/tpgp_rev.h:30-35)."""

    _fields_ = [
        ("i", C.c_size_t),
        ("j", C.c_size_t),
        ("qi", C.c_uint),
        ("qj", C.c_uint),
        ("h", C.c_double),
        ("layer", C.c_size_t),
    ]


class LedgerStruct(C.Structure):
    """Field layout of tpgp_ledger (engine/include/tpgp_rev.h:46-51)."""

    _fields_ = [
        ("dropped_l1", C.c_double),
        ("dropped_l2", C.c_double),
        ("dropped_l2_squared", C.c_double),
        ("arithmetic_l2", C.c_double),
        ("rotations", C.c_size_t),
        ("removal_events", C.c_size_t),
        ("peak_terms", C.c_size_t),
        ("arithmetic_enclosed", C.c_int),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class OptionsStruct(C.Structure):
    """Field layout of tpgp_options (engine/include/tpgp_rev.h:36-45)."""

    _fields_ = [
        ("threshold", C.c_double),
        ("max_terms", C.c_size_t),
        ("threads", C.c_uint),
        ("backend", C.c_int),
        ("validated", C.c_int),
        ("max_drop_l2", C.c_double),
        ("metal_context", C.c_void_p),
        ("cuda_context", C.c_void_p),
    ]


class RotationStruct(C.Structure):
    """orc_rotation: one rotation with explicit factors c, s and radii rc, rs."""

    _fields_ = [("i", C.c_size_t), ("j", C.c_size_t), ("qi", C.c_uint), ("qj", C.c_uint),
                ("c", C.c_double), ("s", C.c_double), ("rc", C.c_double), ("rs", C.c_double)]


def rotations_array(rots):
    """rots: iterable of (i, j, qi, qj, c, s, rc, rs) -> ctypes array of RotationStruct."""
    rots = list(rots)
    arr = (RotationStruct * max(1, len(rots)))()
    for k, r in enumerate(rots):
        arr[k] = RotationStruct(*r)
    return arr, len(rots)


def n_words_for(n_spins: int) -> int:
    return (n_spins + 31) // 32


def terms_array(terms):
    """terms: iterable of (i, j, qi, qj, h) -> ctypes array of TermStruct."""
    terms = list(terms)
    arr = (TermStruct * max(1, len(terms)))()
    for k, (i, j, qi, qj, h) in enumerate(terms):
        arr[k] = TermStruct(i, j, qi, qj, h, k)
    return arr, len(terms)


def _u64p(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


def _f64p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def build_oracle():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


class Oracle:
    """The C restatement (always available once ``make -C oracle`` ran)."""

    kind = "port"

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        lib = C.CDLL(path)
        lib.orc_map_from_arrays.argtypes = [
            C.POINTER(MapStruct), C.c_size_t, C.POINTER(C.c_uint64), C.POINTER(C.c_double),
            C.c_size_t]
        lib.orc_map_free.argtypes = [C.POINTER(MapStruct)]
        lib.orc_rotate.argtypes = [
            C.POINTER(MapStruct), C.c_size_t, C.c_size_t, C.c_uint, C.c_uint, C.c_double,
            C.c_double, C.c_double, C.c_size_t, C.c_double, C.c_uint, C.POINTER(LedgerStruct)]
        lib.orc_strang_step.argtypes = [
            C.POINTER(MapStruct), C.POINTER(TermStruct), C.c_size_t, C.c_double, C.c_double,
            C.c_size_t, C.c_double, C.c_uint, C.POINTER(LedgerStruct)]
        lib.orc_single_sum.argtypes = [C.POINTER(MapStruct), C.c_uint]
        lib.orc_single_sum.restype = C.c_double
        lib.orc_single_sum_arrays.argtypes = [
            C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.c_size_t, C.c_size_t, C.c_uint]
        lib.orc_single_sum_arrays.restype = C.c_double
        lib.orc_trig.argtypes = [C.c_double, C.c_double, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]
        lib.orc_branches.argtypes = [
            C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.c_size_t, C.c_size_t, C.c_size_t,
            C.c_size_t, C.c_size_t, C.c_uint, C.c_uint, C.c_double, C.c_double, C.c_double,
            C.c_double, C.c_int, C.POINTER(C.c_uint64), C.POINTER(C.c_double),
            C.POINTER(C.c_double)]
        lib.orc_rotations_enclosed.argtypes = [
            C.POINTER(MapStruct), C.POINTER(RotationStruct), C.c_size_t, C.c_double, C.c_size_t,
            C.c_double, C.POINTER(LedgerStruct)]
        lib.orc_max_threads.restype = C.c_int
        for name in ("orc_liouvillian", "orc_liouvillian_sorted"):
            getattr(lib, name).argtypes = [C.POINTER(MapStruct), C.POINTER(MapStruct),
                                           C.POINTER(TermStruct), C.c_size_t]
        for name in ("orc_strang_bound", "orc_strang_bound_taylor"):
            getattr(lib, name).argtypes = [C.POINTER(TermStruct), C.c_size_t, C.c_double]
            getattr(lib, name).restype = C.c_double
        self.lib = lib

    # -- maps -------------------------------------------------------------
    def _map(self, keys, values, n_spins):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        values = np.ascontiguousarray(values, dtype=np.float64)
        m = MapStruct()
        st = self.lib.orc_map_from_arrays(C.byref(m), n_spins, _u64p(keys), _f64p(values),
                                          len(values))
        if st:
            raise MemoryError("oracle map allocation failed")
        return m

    def _unmap(self, m):
        w = m.n_words
        keys = np.ctypeslib.as_array(m.keys, shape=(m.len * w,)).copy() if m.len else \
            np.zeros(0, np.uint64)
        values = np.ctypeslib.as_array(m.values, shape=(m.len,)).copy() if m.len else \
            np.zeros(0, np.float64)
        self.lib.orc_map_free(C.byref(m))
        return keys, values

    # -- the path ---------------------------------------------------------
    def trig(self, h, duration):
        c, s = C.c_double(), C.c_double()
        self.lib.orc_trig(h, duration, C.byref(c), C.byref(s))
        return c.value, s.value

    def branches(self, keys, values, n_spins, i, j, qi, qj, c, s, rc=0.0, rs=0.0, enclose=0):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        values = np.ascontiguousarray(values, dtype=np.float64)
        words = n_words_for(n_spins)
        count = len(values)
        ok = np.zeros(2 * count * words, np.uint64)
        ov = np.zeros(2 * count, np.float64)
        orad = np.zeros(2 * count, np.float64)
        st = self.lib.orc_branches(_u64p(keys), _f64p(values), count, words, n_spins, i, j, qi,
                                   qj, c, s, rc, rs, enclose, _u64p(ok), _f64p(ov), _f64p(orad))
        return st, ok, ov, orad

    def rotate(self, keys, values, n_spins, i, j, qi, qj, h, duration, threshold=0.0,
               max_terms=0, max_drop_l2=0.0, threads=1, ledger=None):
        m = self._map(keys, values, n_spins)
        led = ledger if ledger is not None else LedgerStruct()
        st = self.lib.orc_rotate(C.byref(m), i, j, qi, qj, h, duration, threshold, max_terms,
                                 max_drop_l2, threads, C.byref(led))
        k, v = self._unmap(m)
        return st, k, v, led

    def rotations_enclosed(self, keys, values, n_spins, rots, threshold=0.0, max_terms=0,
                           max_drop_l2=0.0, ledger=None):
        """Validated rotations with explicit (c, s, rc, rs), in order, transactional."""
        arr, count = rotations_array(rots)
        m = self._map(keys, values, n_spins)
        led = ledger if ledger is not None else LedgerStruct()
        st = self.lib.orc_rotations_enclosed(C.byref(m), arr, count, threshold, max_terms,
                                             max_drop_l2, C.byref(led))
        k, v = self._unmap(m)
        return st, k, v, led

    def strang_step(self, keys, values, n_spins, terms, dt, threshold=0.0, max_terms=0,
                    max_drop_l2=0.0, threads=1, ledger=None, steps=1, on_step=None):
        arr, count = terms_array(terms)
        m = self._map(keys, values, n_spins)
        led = ledger if ledger is not None else LedgerStruct()
        st = 0
        for step in range(steps):
            st = self.lib.orc_strang_step(C.byref(m), arr, count, dt, threshold, max_terms,
                                          max_drop_l2, threads, C.byref(led))
            if st:
                break
            if on_step is not None:
                on_step(step, self.lib.orc_single_sum(C.byref(m), 1), m.len)
        k, v = self._unmap(m)
        return st, k, v, led

    def single_sum(self, keys, values, n_spins, pauli=1):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        values = np.ascontiguousarray(values, dtype=np.float64)
        return self.lib.orc_single_sum_arrays(_u64p(keys), _f64p(values), len(values), n_spins,
                                              pauli)

    def max_threads(self):
        return self.lib.orc_max_threads()

    def rotate_timed(self, keys, values, n_spins, i, j, qi, qj, h, duration, threshold=0.0,
                     threads=1):
        """One rotation from (keys, values); returns (status, output terms,
        seconds spent in the C rotation call alone)."""
        m = self._map(keys, values, n_spins)
        led = LedgerStruct()
        t0 = time.perf_counter()
        st = self.lib.orc_rotate(C.byref(m), i, j, qi, qj, h, duration, threshold, 0, 0.0,
                                 threads, C.byref(led))
        secs = time.perf_counter() - t0
        n_out = m.len
        self.lib.orc_map_free(C.byref(m))
        return st, n_out, secs

    def liouvillian(self, keys, values, n_spins, terms, sorted_sums=False):
        """-i[H, A] (tpgp_liouvillian, tpgp_rev.c:810-857): (status, keys, values).
        sorted_sums: the sort-then-sum restatement (for large maps) instead of
        sorted insertion."""
        arr, count = terms_array(terms)
        src = self._map(keys, values, n_spins)
        out = self._map(np.zeros(0, np.uint64), np.zeros(0), n_spins)
        f = self.lib.orc_liouvillian_sorted if sorted_sums else self.lib.orc_liouvillian
        st = f(C.byref(out), C.byref(src), arr, count)
        self.lib.orc_map_free(C.byref(src))
        k, v = self._unmap(out)
        return st, k, v

    def strang_bound(self, terms, dt, taylor_only=False):
        """Upward-rounded Strang splitting bound per step (tpgp_rev.c:875-961)."""
        arr, count = terms_array(terms)
        f = self.lib.orc_strang_bound_taylor if taylor_only else self.lib.orc_strang_bound
        return f(arr, count, dt)


class Reference:
    """The reference engine compiled from its own sources (this container only)."""

    kind = "reference"

    def __init__(self, path: str = REFERENCE_SO):
        lib = C.CDLL(path)
        lib.tpgp_default_options.restype = OptionsStruct
        lib.tpgp_map_init.argtypes = [C.POINTER(MapStruct), C.c_size_t]
        lib.tpgp_map_add.argtypes = [C.POINTER(MapStruct), C.POINTER(C.c_uint64), C.c_double]
        lib.tpgp_map_free.argtypes = [C.POINTER(MapStruct)]
        lib.tpgp_rotate.argtypes = [
            C.POINTER(MapStruct), C.c_size_t, C.c_size_t, C.c_uint, C.c_uint, C.c_double,
            C.POINTER(OptionsStruct), C.POINTER(LedgerStruct)]
        lib.tpgp_strang_step.argtypes = [
            C.POINTER(MapStruct), C.POINTER(TermStruct), C.c_size_t, C.c_double,
            C.POINTER(OptionsStruct), C.POINTER(LedgerStruct)]
        lib.tpgp_map_single_sum.argtypes = [C.POINTER(MapStruct), C.c_uint]
        lib.tpgp_map_single_sum.restype = C.c_double
        lib.tpgp_ledger_init.argtypes = [C.POINTER(LedgerStruct), C.c_int]
        for name in ("tpgp_strang_bound", "tpgp_strang_bound_taylor"):
            getattr(lib, name).argtypes = [C.POINTER(TermStruct), C.c_size_t, C.c_double]
            getattr(lib, name).restype = C.c_double
        lib.tpgp_liouvillian.argtypes = [C.POINTER(MapStruct), C.POINTER(MapStruct),
                                         C.POINTER(TermStruct), C.c_size_t]
        self.lib = lib

    def liouvillian(self, keys, values, n_spins, terms):
        """The reference's own tpgp_liouvillian: (status, keys, values)."""
        arr, count = terms_array(terms)
        src = self._map(keys, values, n_spins)
        out = MapStruct()
        if self.lib.tpgp_map_init(C.byref(out), n_spins):
            raise ValueError("tpgp_map_init failed")
        st = self.lib.tpgp_liouvillian(C.byref(out), C.byref(src), arr, count)
        self.lib.tpgp_map_free(C.byref(src))
        k, v = self._unmap(out)
        return st, k, v

    def strang_bound(self, terms, dt, taylor_only=False):
        arr, count = terms_array(terms)
        f = self.lib.tpgp_strang_bound_taylor if taylor_only else self.lib.tpgp_strang_bound
        return f(arr, count, dt)

    def rotate_timed(self, keys, values, n_spins, i, j, qi, qj, h, duration, threshold=0.0,
                     threads=1):
        """tpgp_rotate of h * duration (OpenMP backend with `threads`) from
        (keys, values); returns (status, output terms, seconds of the call)."""
        m = self._map(keys, values, n_spins)
        o = self.options(threshold, 0, 0.0, threads, 2 if threads > 1 else 0)
        led = LedgerStruct()
        t0 = time.perf_counter()
        st = self.lib.tpgp_rotate(C.byref(m), i, j, qi, qj, h * duration, C.byref(o),
                                  C.byref(led))
        secs = time.perf_counter() - t0
        n_out = m.len
        self.lib.tpgp_map_free(C.byref(m))
        return st, n_out, secs

    def options(self, threshold=0.0, max_terms=0, max_drop_l2=0.0, threads=1, backend=0):
        o = self.lib.tpgp_default_options()
        o.threshold = threshold
        o.max_terms = max_terms
        o.max_drop_l2 = max_drop_l2
        o.threads = threads
        o.backend = backend
        return o

    def _map(self, keys, values, n_spins):
        """Fills a tpgp_map's storage directly (libc malloc, released by
        tpgp_map_free), so callers can also state invalid contents such as a
        nonfinite coefficient."""
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        values = np.ascontiguousarray(values, dtype=np.float64)
        m = MapStruct()
        if self.lib.tpgp_map_init(C.byref(m), n_spins):
            raise ValueError("tpgp_map_init failed")
        n = len(values)
        if n:
            libc = C.CDLL(None)
            libc.malloc.restype = C.c_void_p
            libc.malloc.argtypes = [C.c_size_t]
            kp = libc.malloc(max(1, keys.nbytes))
            vp = libc.malloc(max(1, values.nbytes))
            C.memmove(kp, keys.ctypes.data, keys.nbytes)
            C.memmove(vp, values.ctypes.data, values.nbytes)
            m.keys = C.cast(kp, C.POINTER(C.c_uint64))
            m.values = C.cast(vp, C.POINTER(C.c_double))
            m.len = n
            m.capacity = n
        return m

    def _unmap(self, m):
        w = m.n_words
        keys = np.ctypeslib.as_array(m.keys, shape=(m.len * w,)).copy() if m.len else \
            np.zeros(0, np.uint64)
        values = np.ctypeslib.as_array(m.values, shape=(m.len,)).copy() if m.len else \
            np.zeros(0, np.float64)
        self.lib.tpgp_map_free(C.byref(m))
        return keys, values

    def rotate(self, keys, values, n_spins, i, j, qi, qj, theta, threshold=0.0, max_terms=0,
               max_drop_l2=0.0, threads=1, backend=0, ledger=None):
        m = self._map(keys, values, n_spins)
        o = self.options(threshold, max_terms, max_drop_l2, threads, backend)
        led = ledger if ledger is not None else LedgerStruct()
        st = self.lib.tpgp_rotate(C.byref(m), i, j, qi, qj, theta, C.byref(o), C.byref(led))
        k, v = self._unmap(m)
        return st, k, v, led

    def strang_step(self, keys, values, n_spins, terms, dt, threshold=0.0, max_terms=0,
                    max_drop_l2=0.0, threads=1, backend=0, ledger=None, steps=1,
                    on_step=None):
        arr, count = terms_array(terms)
        m = self._map(keys, values, n_spins)
        o = self.options(threshold, max_terms, max_drop_l2, threads, backend)
        led = ledger if ledger is not None else LedgerStruct()
        st = 0
        for step in range(steps):
            st = self.lib.tpgp_strang_step(C.byref(m), arr, count, dt, C.byref(o),
                                           C.byref(led))
            if st:
                break
            if on_step is not None:
                on_step(step, self.lib.tpgp_map_single_sum(C.byref(m), 1), m.len)
        k, v = self._unmap(m)
        return st, k, v, led
