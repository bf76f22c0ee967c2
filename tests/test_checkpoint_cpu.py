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


def as_reference(rec):
    """The same record as the reference's tpgp_checkpoint (arrays shared)."""
    r = RefCheckpoint()
    r.map = RefMap(rec.n_spins, (rec.n_spins + 31) // 32, rec.len, rec.len, rec.keys, rec.values)
    r.terms, r.term_count = rec.terms, rec.term_count
    r.options = RefOptions(rec.threshold, rec.max_terms, rec.threads, rec.backend, rec.validated,
                           rec.max_drop_l2, None, None)
    for name in ("ledger", "dt", "pf_bound", "residual_bound", "max_fid_bound", "step",
                 "total_steps", "residual_depth", "initial_global", "model", "j2", "linear_size",
                 "resumed_from_step", "prior_total_steps", "prior_max_terms", "stop_reason",
                 "last_status"):
        setattr(r, name, getattr(rec, name))
    return r


def _mutations():
    """(name, change, valid): one field of the reference CLI's record changed."""
    nan, inf = float("nan"), float("inf")

    def field(name, value):
        return lambda r: setattr(r, name, value)

    def ledger(name, value):
        return lambda r: setattr(r.ledger, name, value)

    def value0(v):
        return lambda r: r.values.__setitem__(0, v)

    def term0(name, value):
        return lambda r: setattr(r.terms[0], name, value)

    return [
        ("dt zero", field("dt", 0.0), False), ("dt inf", field("dt", inf), False),
        ("step past total", field("step", 21), False),
        ("resumed past step", field("resumed_from_step", 21), False),
        ("residual depth 11", field("residual_depth", 11), False),
        ("initial 2", field("initial_global", 2), False),
        ("model empty", field("model", b""), False), ("model upper", field("model", b"Ring"), False),
        ("model ok", field("model", b"ring_2"), True), ("j2 nan", field("j2", nan), False),
        ("stop 7", field("stop_reason", 7), False),
        ("complete early", lambda r: (setattr(r, "total_steps", 40)), False),
        ("running early", lambda r: (setattr(r, "total_steps", 40), setattr(r, "stop_reason", 0)),
         True),
        ("status 7", field("last_status", 7), False), ("threshold -1", field("threshold", -1.0), False),
        ("threads 0", field("threads", 0), False), ("threads big", field("threads", 70000), False),
        ("backend 5", field("backend", 5), False), ("validated 2", field("validated", 2), False),
        ("budget -1", field("max_drop_l2", -1.0), False),
        ("cap below len", field("max_terms", 100), False), ("no cap", field("max_terms", 0), True),
        ("fid stop unbounded", field("max_fid_bound", 0.5), False),
        ("dropped nan", ledger("dropped_l2", nan), False), ("dropped inf", ledger("dropped_l2", inf), True),
        ("dropped -1", ledger("dropped_l1", -1.0), False), ("pf nan", field("pf_bound", nan), False),
        ("enclosed unvalidated", ledger("arithmetic_enclosed", 1), False),
        ("peak below len", ledger("peak_terms", 10), False),
        ("residual without depth", field("residual_bound", 0.1), False),
        ("depth without residual", field("residual_depth", 2), False),
        ("depth with residual",
         lambda r: (setattr(r, "residual_depth", 2), setattr(r, "residual_bound", 0.1)), True),
        ("zero value", value0(0.0), False), ("inf value", value0(inf), False),
        ("keys out of order", lambda r: r.keys.__setitem__(0, r.keys[1] + 1), False),
        ("padding bits", lambda r: r.keys.__setitem__(0, 1 << 40), False),
        ("term same site", term0("j", 0), False), ("term label 4", term0("qi", 4), False),
        ("term h inf", term0("h", inf), False),
    ]


@pytest.mark.parametrize("name,change,valid", _mutations(), ids=[m[0] for m in _mutations()])
def test_record_invariants(tmp_path, name, change, valid):
    """Each of the reference's record invariants (checkpoint_rev.c:116-195),
    one field at a time on the reference CLI's record: the writer refuses an
    invalid record (and writes nothing) and accepts a valid one; where the
    reference engine was built here, its own writer decides the same way."""
    lib = native.load()
    st, rec, msg = load(lib, GOLDEN)
    assert st == 0, msg
    change(rec)
    out = str(tmp_path / "r.tpgpck")
    err = C.create_string_buffer(256)
    ours = lib.tpgp_gb_checkpoint_write(out.encode(), C.byref(rec), err, 256)
    assert (ours == 0) == valid, (name, err.value)
    assert os.path.exists(out) == valid
    if os.path.exists(REFCK):
        ref = C.CDLL(REFCK)
        ref.tpgp_checkpoint_save.argtypes = [C.c_char_p, C.POINTER(RefCheckpoint), C.c_char_p,
                                             C.c_size_t]
        ref_out = str(tmp_path / "ref.tpgpck")
        theirs = ref.tpgp_checkpoint_save(ref_out.encode(), C.byref(as_reference(rec)), err, 256)
        assert (theirs == 0) == valid, (name, err.value)
    lib.tpgp_gb_checkpoint_free(C.byref(rec))
