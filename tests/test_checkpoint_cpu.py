"""Restart records in the reference's version-2 checkpoint format, host
side (no GPU): a record written by the reference CLI loads here and is
written back byte for byte; a record written here loads in the reference
engine's own loader (engine/src/checkpoint_rev.c, compiled from its sources
into oracle/_ref where the checkout was present); a damaged record is
rejected and leaves the destination untouched."""
import ctypes as C
import os

import numpy as np
import pytest

from ddevol_gb300 import native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "cli_ring16.tpgpck")
REFCK = os.path.join(ROOT, "oracle", "_ref", "libtpgp_refck.so")


def load(lib, path):
    rec = native.GbCheckpoint()
    err = C.create_string_buffer(256)
    st = lib.tpgp_gb_checkpoint_load(path.encode(), C.byref(rec), err, 256)
    return st, rec, err.value.decode()


def test_reference_record_loads_and_is_rewritten_byte_for_byte(tmp_path):
    lib = native.load()
    st, rec, msg = load(lib, GOLDEN)
    assert st == 0, msg
    assert rec.n_spins == 16 and rec.step == 20 and rec.total_steps == 20
    assert rec.term_count == 96 and rec.len == 1991 and rec.model == b"edges"
    assert rec.stop_reason == 1 and rec.residual_depth == -1 and np.isnan(rec.residual_bound)
    assert rec.ledger.rotations == 3840
    out = str(tmp_path / "again.tpgpck")
    err = C.create_string_buffer(256)
    assert lib.tpgp_gb_checkpoint_write(out.encode(), C.byref(rec), err, 256) == 0, err.value
    assert open(out, "rb").read() == open(GOLDEN, "rb").read()
    assert os.path.exists(out + ".manifest.json")
    lib.tpgp_gb_checkpoint_free(C.byref(rec))


def test_damaged_record_is_rejected(tmp_path):
    lib = native.load()
    bad = tmp_path / "bad.tpgpck"
    data = bytearray(open(GOLDEN, "rb").read())
    data[500] ^= 1
    bad.write_bytes(bytes(data))
    st, rec0, _ = load(lib, GOLDEN)
    assert st == 0
    before = (rec0.len, rec0.step)
    err = C.create_string_buffer(256)
    assert lib.tpgp_gb_checkpoint_load(str(bad).encode(), C.byref(rec0), err, 256) == 1
    assert b"checksum" in err.value
    assert (rec0.len, rec0.step) == before  # destination untouched
    short = tmp_path / "short.tpgpck"
    short.write_bytes(bytes(data[:200]))
    assert lib.tpgp_gb_checkpoint_load(str(short).encode(), C.byref(rec0), err, 256) == 1
    lib.tpgp_gb_checkpoint_free(C.byref(rec0))


class RefMap(C.Structure):
    _fields_ = [("n_spins", C.c_size_t), ("n_words", C.c_size_t), ("len", C.c_size_t),
                ("capacity", C.c_size_t), ("keys", C.POINTER(C.c_uint64)),
                ("values", C.POINTER(C.c_double))]


class RefOptions(C.Structure):
    _fields_ = [("threshold", C.c_double), ("max_terms", C.c_size_t), ("threads", C.c_uint),
                ("backend", C.c_int), ("validated", C.c_int), ("max_drop_l2", C.c_double),
                ("metal_context", C.c_void_p), ("cuda_context", C.c_void_p)]


class RefCheckpoint(C.Structure):
    """tpgp_checkpoint (engine/include/checkpoint_rev.h:6-22)."""
    _fields_ = [("map", RefMap), ("terms", C.POINTER(native.GbTerm)), ("term_count", C.c_size_t),
                ("options", RefOptions), ("ledger", native.GbLedger), ("dt", C.c_double),
                ("pf_bound", C.c_double), ("residual_bound", C.c_double),
                ("max_fid_bound", C.c_double), ("step", C.c_size_t), ("total_steps", C.c_size_t),
                ("residual_depth", C.c_int), ("initial_global", C.c_int), ("model", C.c_char * 32),
                ("j2", C.c_double), ("linear_size", C.c_size_t), ("resumed_from_step", C.c_size_t),
                ("prior_total_steps", C.c_size_t), ("prior_max_terms", C.c_size_t),
                ("stop_reason", C.c_int), ("last_status", C.c_int)]


@pytest.mark.skipif(not os.path.exists(REFCK), reason="reference engine not built here")
def test_record_written_here_loads_in_the_reference(tmp_path):
    lib = native.load()
    st, rec, msg = load(lib, GOLDEN)
    assert st == 0, msg
    # a different run state: a GPU-backend record at step 20 of 40
    rec.backend = 4
    rec.total_steps = 40
    rec.stop_reason = 0
    rec.pf_bound = 1.25e-9
    out = str(tmp_path / "ours.tpgpck")
    err = C.create_string_buffer(256)
    assert lib.tpgp_gb_checkpoint_write(out.encode(), C.byref(rec), err, 256) == 0, err.value
    ref = C.CDLL(REFCK)
    ref.tpgp_checkpoint_load.argtypes = [C.c_char_p, C.POINTER(RefCheckpoint), C.c_char_p, C.c_size_t]
    ref.tpgp_checkpoint_free.argtypes = [C.POINTER(RefCheckpoint)]
    got = RefCheckpoint()
    assert ref.tpgp_checkpoint_load(out.encode(), C.byref(got), err, 256) == 0, err.value
    assert got.map.n_spins == 16 and got.map.len == rec.len and got.step == 20
    assert got.total_steps == 40 and got.options.backend == 4 and got.pf_bound == 1.25e-9
    n = rec.len
    assert np.array_equal(np.ctypeslib.as_array(got.map.keys, (n,)),
                          np.ctypeslib.as_array(rec.keys, (n,)))
    assert np.array_equal(np.ctypeslib.as_array(got.map.values, (n,)).view(np.uint64),
                          np.ctypeslib.as_array(rec.values, (n,)).view(np.uint64))
    ref.tpgp_checkpoint_free(C.byref(got))
    lib.tpgp_gb_checkpoint_free(C.byref(rec))
