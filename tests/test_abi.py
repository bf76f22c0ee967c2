"""The C-ABI library builds for sm_103a, loads, and exports every declared symbol.

No compute call is made here (this runs without a GPU); on a machine with no
device the context constructors must fail loudly rather than fall back.
"""
import ctypes as C
import os
import re

import pytest

from ddevol_gb300 import build as gbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for header in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not header.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", header)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(tpgp_\w+)\s*\(", text):
            names.append(m.group(1))
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    path = gbuild.build()
    return C.CDLL(path)


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert "tpgp_cuda_branches" in names and "tpgp_gb_strang_step" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_compiled_flags(lib):
    assert lib.tpgp_cuda_compiled() == 1
    assert lib.tpgp_gb_compiled() == 1


def test_argument_checks_need_no_device(lib):
    f = lib.tpgp_cuda_branches
    f.restype = C.c_int
    err = C.create_string_buffer(256)
    # NULL context -> EINVAL before any CUDA call (the status of engine/src/cuda_rev.cu:180-186)
    st = f(None, None, None, C.c_size_t(0), C.c_size_t(1), C.c_size_t(2), C.c_size_t(0),
           C.c_size_t(1), C.c_uint(3), C.c_uint(3), C.c_double(.6), C.c_double(.8),
           C.c_double(0), C.c_double(0), C.c_int(1), None, None, None, err, C.c_size_t(256))
    assert st == 1
    assert b"NULL context" in err.value


def test_sm103a_code_in_library():
    # the fatbin carries sm_103a SASS (checked by the build flags, not by decoding it)
    assert "arch=compute_103a,code=sm_103a" in " ".join(gbuild.NVCC_FLAGS)
