"""ctypes bindings of ``libtpgp_gb300.so`` (include/tpgp_cuda_rev.h, include/tpgp_gb300.h).

The library is the product: every call here goes straight to the sm_103a
kernels.  There is no CPU fallback -- if the library cannot be loaded or no
GB300 is visible, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

STATUS_NAMES = ["ok", "einval", "enomem", "ecap", "enumeric", "ebackend", "ebudget"]
CUDA_STATUS_NAMES = ["ok", "einval", "enomem", "edevice", "enumeric"]

_lock = threading.Lock()
_lib = None


class GbTerm(C.Structure):
    """tpgp_gb_term: layout of tpgp_term (engine/include/tpgp_rev.h:30-35)."""

    _fields_ = [("i", C.c_size_t), ("j", C.c_size_t), ("qi", C.c_uint), ("qj", C.c_uint),
                ("h", C.c_double), ("layer", C.c_size_t)]


class GbLedger(C.Structure):
    """tpgp_gb_ledger: layout of tpgp_ledger (engine/include/tpgp_rev.h:46-51)."""

    _fields_ = [("dropped_l1", C.c_double), ("dropped_l2", C.c_double),
                ("dropped_l2_squared", C.c_double), ("arithmetic_l2", C.c_double),
                ("rotations", C.c_size_t), ("removal_events", C.c_size_t),
                ("peak_terms", C.c_size_t), ("arithmetic_enclosed", C.c_int)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class GbCheckpoint(C.Structure):
    """tpgp_gb_checkpoint (include/tpgp_gb300.h): a restart record in host memory."""

    _fields_ = [("n_spins", C.c_size_t), ("len", C.c_size_t), ("keys", C.POINTER(C.c_uint64)),
                ("values", C.POINTER(C.c_double)), ("terms", C.POINTER(GbTerm)),
                ("term_count", C.c_size_t), ("threshold", C.c_double), ("max_terms", C.c_size_t),
                ("threads", C.c_uint), ("backend", C.c_int), ("validated", C.c_int),
                ("max_drop_l2", C.c_double), ("ledger", GbLedger), ("dt", C.c_double),
                ("pf_bound", C.c_double), ("residual_bound", C.c_double),
                ("max_fid_bound", C.c_double), ("step", C.c_size_t), ("total_steps", C.c_size_t),
                ("residual_depth", C.c_int), ("initial_global", C.c_int), ("model", C.c_char * 32),
                ("j2", C.c_double), ("linear_size", C.c_size_t), ("resumed_from_step", C.c_size_t),
                ("prior_total_steps", C.c_size_t), ("prior_max_terms", C.c_size_t),
                ("stop_reason", C.c_int), ("last_status", C.c_int)]


class GbRotation(C.Structure):
    """tpgp_gb_rotation: one rotation with the caller's factors c, s and radii rc, rs."""

    _fields_ = [("i", C.c_size_t), ("j", C.c_size_t), ("qi", C.c_uint), ("qj", C.c_uint),
                ("c", C.c_double), ("s", C.c_double), ("rc", C.c_double), ("rs", C.c_double)]


class GbEngineConfig(C.Structure):
    """tpgp_gb_engine_config (include/tpgp_gb300.h): a map's step-engine launch configuration."""

    _fields_ = [("hash_step", C.c_int), ("hash_ctas", C.c_int), ("hash_pdl", C.c_int),
                ("hash_fuse", C.c_int), ("sorted_pdl", C.c_int), ("step_ms", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class GbTuning(C.Structure):
    """tpgp_gb_tuning: the autotuner's choice, the entry configuration and every trial."""

    _fields_ = [("chosen", GbEngineConfig), ("before", GbEngineConfig), ("tried_count", C.c_size_t),
                ("tried", GbEngineConfig * 16)]


class GbOptions(C.Structure):
    _fields_ = [("threshold", C.c_double), ("max_terms", C.c_size_t),
                ("max_drop_l2", C.c_double), ("exact_ledger", C.c_int), ("use_graphs", C.c_int),
                ("wait_polls", C.c_uint)]


class GbRequest(C.Structure):
    """tpgp_gb_request (include/tpgp_gb300.h)."""

    _fields_ = [("arrival", C.c_double), ("n_spins", C.c_size_t), ("terms", C.POINTER(GbTerm)),
                ("count", C.c_size_t), ("dt", C.c_double), ("steps", C.c_size_t),
                ("options", GbOptions), ("keys", C.POINTER(C.c_uint64)),
                ("values", C.POINTER(C.c_double)), ("len", C.c_size_t)]


class GbResponse(C.Structure):
    """tpgp_gb_response (include/tpgp_gb300.h)."""

    _fields_ = [("admitted", C.c_double), ("finished", C.c_double), ("status", C.c_int),
                ("slot", C.c_size_t), ("slot_spins", C.c_size_t), ("peak_terms", C.c_size_t),
                ("fid_last", C.c_double)]


class GbServeStats(C.Structure):
    """tpgp_gb_serve_stats (include/tpgp_gb300.h)."""

    _fields_ = [("busy_seconds", C.c_double), ("wall_seconds", C.c_double),
                ("ticks", C.c_ulonglong), ("terms", C.c_ulonglong), ("launches", C.c_ulonglong),
                ("max_active", C.c_size_t)]


def _bind(lib):
    P = C.POINTER
    u64p, f64p, charp = P(C.c_uint64), P(C.c_double), C.c_char_p
    sz = C.c_size_t
    # reference-compatible branch ABI
    lib.tpgp_cuda_compiled.restype = C.c_int
    lib.tpgp_cuda_create.restype = C.c_void_p
    lib.tpgp_cuda_create.argtypes = [C.c_int, charp, sz]
    lib.tpgp_cuda_destroy.argtypes = [C.c_void_p]
    lib.tpgp_cuda_device_name.restype = C.c_char_p
    lib.tpgp_cuda_device_name.argtypes = [C.c_void_p]
    lib.tpgp_cuda_branches.restype = C.c_int
    lib.tpgp_cuda_branches.argtypes = [
        C.c_void_p, u64p, f64p, sz, sz, sz, sz, sz, C.c_uint, C.c_uint, C.c_double, C.c_double,
        C.c_double, C.c_double, C.c_int, u64p, f64p, f64p, charp, sz]
    lib.tpgp_cuda_branches_static.restype = C.c_int
    lib.tpgp_cuda_branches_static.argtypes = [
        C.c_int, u64p, f64p, sz, sz, sz, sz, sz, C.c_uint, C.c_uint, C.c_double, C.c_double,
        C.c_double, C.c_double, C.c_int, u64p, f64p, f64p, charp, sz]
    # device-resident ABI
    lib.tpgp_gb_compiled.restype = C.c_int
    lib.tpgp_gb_default_options.restype = GbOptions
    lib.tpgp_gb_create.restype = C.c_void_p
    lib.tpgp_gb_create.argtypes = [C.c_int, charp, sz]
    lib.tpgp_gb_destroy.argtypes = [C.c_void_p]
    lib.tpgp_gb_device_name.restype = C.c_char_p
    lib.tpgp_gb_device_name.argtypes = [C.c_void_p]
    lib.tpgp_gb_map_create.restype = C.c_int
    lib.tpgp_gb_map_create.argtypes = [C.c_void_p, sz, P(C.c_void_p), charp, sz]
    lib.tpgp_gb_map_destroy.argtypes = [C.c_void_p]
    lib.tpgp_gb_map_len.restype = sz
    lib.tpgp_gb_map_len.argtypes = [C.c_void_p]
    lib.tpgp_gb_map_spins.restype = sz
    lib.tpgp_gb_map_spins.argtypes = [C.c_void_p]
    lib.tpgp_gb_map_upload.restype = C.c_int
    lib.tpgp_gb_map_upload.argtypes = [C.c_void_p, u64p, f64p, sz, charp, sz]
    lib.tpgp_gb_map_download.restype = C.c_int
    lib.tpgp_gb_map_download.argtypes = [C.c_void_p, u64p, f64p, sz, P(sz), charp, sz]
    lib.tpgp_gb_rotate.restype = C.c_int
    lib.tpgp_gb_rotate.argtypes = [C.c_void_p, sz, sz, C.c_uint, C.c_uint, C.c_double,
                                   P(GbOptions), P(GbLedger), charp, sz]
    lib.tpgp_gb_strang_step.restype = C.c_int
    lib.tpgp_gb_strang_step.argtypes = [C.c_void_p, P(GbTerm), sz, C.c_double, P(GbOptions),
                                        P(GbLedger), charp, sz]
    lib.tpgp_gb_rotate_enclosed.restype = C.c_int
    lib.tpgp_gb_rotate_enclosed.argtypes = [C.c_void_p, P(GbRotation), sz, P(GbOptions),
                                            P(GbLedger), charp, sz]
    lib.tpgp_gb_map_autotune.restype = C.c_int
    lib.tpgp_gb_map_autotune.argtypes = [C.c_void_p, P(GbTerm), sz, C.c_double, P(GbOptions),
                                         P(GbTuning), charp, sz]
    lib.tpgp_gb_map_get_config.restype = C.c_int
    lib.tpgp_gb_map_get_config.argtypes = [C.c_void_p, P(GbEngineConfig)]
    lib.tpgp_gb_map_set_config.restype = C.c_int
    lib.tpgp_gb_map_set_config.argtypes = [C.c_void_p, P(GbEngineConfig)]
    lib.tpgp_gb_evolve.restype = C.c_int
    lib.tpgp_gb_evolve.argtypes = [C.c_void_p, P(GbTerm), sz, C.c_double, sz, P(GbOptions),
                                   P(GbLedger), f64p, P(sz), charp, sz]
    lib.tpgp_gb_single_sum.restype = C.c_int
    lib.tpgp_gb_single_sum.argtypes = [C.c_void_p, C.c_uint, f64p]
    lib.tpgp_gb_checkpoint_write.restype = C.c_int
    lib.tpgp_gb_checkpoint_write.argtypes = [charp, P(GbCheckpoint), charp, sz]
    lib.tpgp_gb_checkpoint_load.restype = C.c_int
    lib.tpgp_gb_checkpoint_load.argtypes = [charp, P(GbCheckpoint), charp, sz]
    lib.tpgp_gb_checkpoint_free.argtypes = [P(GbCheckpoint)]
    lib.tpgp_gb_map_l2.restype = C.c_int
    lib.tpgp_gb_map_l2.argtypes = [C.c_void_p, f64p]
    lib.tpgp_gb_upward_sums.restype = C.c_int
    lib.tpgp_gb_upward_sums.argtypes = [C.c_void_p, f64p, C.c_size_t, C.c_size_t, f64p]
    lib.tpgp_gb_strang_bound.restype = C.c_double
    lib.tpgp_gb_strang_bound.argtypes = [P(GbTerm), sz, C.c_double]
    lib.tpgp_gb_liouvillian.restype = C.c_int
    lib.tpgp_gb_liouvillian.argtypes = [C.c_void_p, C.c_void_p, P(GbTerm), sz, charp, sz]
    lib.tpgp_gb_last_elapsed_ms.restype = C.c_double
    lib.tpgp_gb_last_elapsed_ms.argtypes = [C.c_void_p]
    lib.tpgp_gb_last_launches.restype = sz
    lib.tpgp_gb_last_launches.argtypes = [C.c_void_p]
    lib.tpgp_gb_last_terms.restype = sz
    lib.tpgp_gb_last_terms.argtypes = [C.c_void_p]
    lib.tpgp_gb_batch_create.restype = C.c_int
    lib.tpgp_gb_batch_create.argtypes = [C.c_void_p, sz, P(sz), P(C.c_void_p), charp, sz]
    lib.tpgp_gb_batch_destroy.argtypes = [C.c_void_p]
    lib.tpgp_gb_batch_upload.restype = C.c_int
    lib.tpgp_gb_batch_upload.argtypes = [C.c_void_p, sz, u64p, f64p, sz, charp, sz]
    lib.tpgp_gb_batch_set_terms.restype = C.c_int
    lib.tpgp_gb_batch_set_terms.argtypes = [C.c_void_p, sz, P(GbTerm), sz, C.c_double,
                                            P(GbOptions), charp, sz]
    lib.tpgp_gb_batch_step.restype = C.c_int
    lib.tpgp_gb_batch_step.argtypes = [C.c_void_p, sz, f64p, charp, sz]
    lib.tpgp_gb_batch_autotune.restype = C.c_int
    lib.tpgp_gb_batch_autotune.argtypes = [C.c_void_p, charp, sz]
    lib.tpgp_gb_batch_cluster.restype = C.c_int
    lib.tpgp_gb_batch_cluster.argtypes = [C.c_void_p, sz]
    lib.tpgp_gb_batch_set_cluster.restype = C.c_int
    lib.tpgp_gb_batch_set_cluster.argtypes = [C.c_void_p, sz, C.c_int, sz, charp, sz]
    lib.tpgp_gb_batch_uses_tables.restype = C.c_int
    lib.tpgp_gb_batch_uses_tables.argtypes = [C.c_void_p]
    lib.tpgp_gb_batch_get_tuning.restype = C.c_int
    lib.tpgp_gb_batch_get_tuning.argtypes = [C.c_void_p, sz, C.POINTER(C.c_int),
                                             C.POINTER(C.c_size_t), C.POINTER(C.c_double)]
    lib.tpgp_gb_batch_max_cluster.restype = C.c_int
    lib.tpgp_gb_batch_max_cluster.argtypes = [C.c_void_p, sz]
    lib.tpgp_gb_batch_item_status.restype = C.c_int
    lib.tpgp_gb_batch_item_status.argtypes = [C.c_void_p, sz]
    lib.tpgp_gb_batch_len.restype = sz
    lib.tpgp_gb_batch_len.argtypes = [C.c_void_p, sz]
    lib.tpgp_gb_batch_ledger.restype = C.c_int
    lib.tpgp_gb_batch_ledger.argtypes = [C.c_void_p, sz, P(GbLedger)]
    lib.tpgp_gb_batch_download.restype = C.c_int
    lib.tpgp_gb_batch_download.argtypes = [C.c_void_p, sz, u64p, f64p, sz, P(sz), charp, sz]
    lib.tpgp_gb_batch_last_elapsed_ms.restype = C.c_double
    lib.tpgp_gb_batch_last_elapsed_ms.argtypes = [C.c_void_p]
    lib.tpgp_gb_batch_last_terms.restype = sz
    lib.tpgp_gb_batch_last_terms.argtypes = [C.c_void_p]
    lib.tpgp_gb_batch_last_launches.restype = sz
    lib.tpgp_gb_batch_last_launches.argtypes = [C.c_void_p]
    lib.tpgp_gb_serve.restype = C.c_int
    lib.tpgp_gb_serve.argtypes = [C.c_void_p, P(GbRequest), sz, P(sz), sz, f64p, P(GbResponse),
                                  P(GbServeStats), charp, sz]
    lib.tpgp_gb_set_profiling.argtypes = [C.c_void_p, C.c_int]
    lib.tpgp_gb_kernel_profile.argtypes = [C.c_void_p, f64p, P(sz)]
    return lib


def load(build_if_needed: bool = True):
    """Loads (building first if needed) the native library; raises on failure."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_needed:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"native library missing: {path} (run ddevol_gb300.build)")
        _lib = _bind(C.CDLL(path))
        return _lib


def library_path() -> str:
    return _build.LIB
