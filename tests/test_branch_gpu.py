"""The reference-compatible branch ABI on the GPU, bitwise against the oracle.

Restates the case matrix of the reference's own test (DDevol
engine/tests/test_cuda_rev.c): the 8192 two-site cases crossing every Pauli key
with 16 edge coefficients (signed zeros, subnormals, DBL_MAX/4), the 20,560
N=1000 cases at word boundaries, the exact-angle factors, every invalid-input
status, and two threads sharing one context.
"""
import ctypes as C
import math
import sys
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DBL_MAX = sys.float_info.max
EDGE = [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, -2.2250738585072014e-308, 1.0, -1.0,
        DBL_MAX * 0.25, -DBL_MAX * 0.25, float.fromhex("0x1.fffffffffffffp-1"),
        -float.fromhex("0x1.fffffffffffffp-1"), 2.0 ** -1000, -(2.0 ** -1000), 2.0 ** 1000,
        -(2.0 ** 1000)]
M64 = (1 << 64) - 1


def xorshift(state):
    state ^= (state << 13) & M64
    state ^= state >> 7
    state ^= (state << 17) & M64
    return state & M64


def compare(ctx, oracle, keys, values, spins, i, j, qi, qj, c, s, rc, rs, enclose):
    st, k, v, r, err = ctx.branches(keys, values, spins, i, j, qi, qj, c, s, rc, rs, enclose)
    ost, ok, ov, orad = oracle.branches(keys, values, spins, i, j, qi, qj, c, s, rc, rs, enclose)
    assert ost == 0
    assert st == 0, err
    assert np.array_equal(k, ok)
    assert np.array_equal(v.view(np.uint64), ov.view(np.uint64))
    assert np.array_equal(r.view(np.uint64), orad.view(np.uint64))


def test_two_site_cross_product(branch_ctx, oracle):
    keys = np.array([p for p in range(16) for _ in range(16)], np.uint64)
    values = np.array([EDGE[v] for _ in range(16) for v in range(16)], np.float64)
    cases = 0
    for qi in range(4):
        for qj in range(4):
            for enclose in (0, 1):
                compare(branch_ctx, oracle, keys, values, 2, 0, 1, qi, qj, 0.6, -0.8,
                        2.0 ** -54, 2.0 ** -1050, enclose)
                cases += len(values)
    assert cases == 8192


def test_n1000_word_boundaries(branch_ctx, oracle):
    count, words = 257, 32
    seed = 0x9E3779B97F4A7C15
    keys = np.zeros(count * words, np.uint64)
    coeff = np.zeros(count, np.float64)
    for k in range(count):
        for w in range(words):
            seed = xorshift(seed)
            keys[k * words + w] = seed
        keys[k * words + words - 1] &= np.uint64(0xFFFF)
        if k < 16:
            coeff[k] = EDGE[k]
        else:
            seed = xorshift(seed)
            coeff[k] = math.ldexp((seed >> 11) * 2.0 ** -53, (k % 1800) - 900)
    cases = 0
    for a, b in ((0, 15), (15, 16), (31, 32), (511, 999), (999, 0)):
        for qi in range(4):
            for qj in range(4):
                compare(branch_ctx, oracle, keys, coeff, 1000, a, b, qi, qj, -0.8, 0.6,
                        2.0 ** -54, 2.0 ** -54, 1)
                cases += count
    assert cases == 20560
    compare(branch_ctx, oracle, keys, coeff, 1000, 0, 999, 3, 3, 1.0, -0.0, 0.0, 0.0, 1)
    compare(branch_ctx, oracle, keys, coeff, 1000, 0, 999, 3, 3, 0.0, -1.0, 0.0, 0.0, 1)


def test_invalid_inputs(branch_ctx):
    lib, ctx = branch_ctx.lib, branch_ctx.ptr
    err = C.create_string_buffer(512)
    key = (C.c_uint64 * 1)(1)
    val = (C.c_double * 1)(1.0)
    ok_, ov, orad = (C.c_uint64 * 2)(), (C.c_double * 2)(), (C.c_double * 2)()

    def call(c=ctx, k=key, v=val, n=1, w=1, sp=2, i=0, j=1, qi=3, qj=3, cc=.6, s=.8, rc=0.0,
             rs=0.0, en=1, outk=ok_, outv=ov, outr=orad):
        return lib.tpgp_cuda_branches(c, k, v, n, w, sp, i, j, qi, qj, cc, s, rc, rs, en, outk,
                                      outv, outr, err, len(err))
    assert call(c=None) == 1
    assert call(k=None) == 1
    assert call(n=(1 << 64) - 1) == 1
    assert call(w=2) == 1
    assert call(j=0) == 1
    assert call(qi=4) == 1
    assert call(cc=float("nan")) == 1
    assert call(rc=float("inf")) == 1
    assert call(rc=-1.0) == 1
    assert call(en=2) == 1
    assert call(outk=C.cast(key, C.POINTER(C.c_uint64))) == 1  # overlaps the input
    assert call(k=None, v=None, n=0, outk=None, outv=None, outr=None) == 0
    key[0] = 16  # a padding bit above two spins
    assert call() == 1
    key[0] = 1
    val[0] = float("nan")
    assert call() == 4
    val[0] = float("inf")
    assert call() == 4
    key[0] = 0  # commuting input must not bypass the check
    assert call() == 4
    key[0] = 1
    val[0] = DBL_MAX
    assert call(cc=2.0) == 4
    val[0] = 1.0
    assert call() == 0  # reuse after failures
    assert not lib.tpgp_cuda_create(-1, err, len(err))
    assert not lib.tpgp_cuda_create(2 ** 31 - 1, err, len(err))
    assert "sm_" in branch_ctx.name


def test_two_concurrent_callers(branch_ctx, oracle):
    failures = []

    def worker(seed):
        try:
            keys = np.zeros(64 * 32, np.uint64)
            for k in range(64):
                for w in range(32):
                    seed = xorshift(seed)
                    keys[k * 32 + w] = seed
                keys[k * 32 + 31] &= np.uint64(0xFFFF)
            values = np.array([(k + 1) / 64 for k in range(64)])
            for q in (1, 2, 3):
                compare(branch_ctx, oracle, keys, values, 1000, 511, 999, q, q, .6, -.8,
                        2.0 ** -54, 2.0 ** -54, 1)
        except AssertionError as e:  # pragma: no cover - reported below
            failures.append(e)

    threads = [threading.Thread(target=worker, args=(s,)) for s in (0x431217, 0x187721)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not failures
