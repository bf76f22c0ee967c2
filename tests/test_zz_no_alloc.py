"""The allocation-free branch entry point against the ordinary one.

tpgp_cuda_branches_static is for callers that cannot call cudaMalloc (code
inside a host allocator or a real-time section, plugins whose host
application owns all device memory): its staging buffers live in a static
16 MiB device array instead of memory the library allocates.  Its outputs
must equal tpgp_cuda_branches' bit for bit, on consecutive calls that share
the array (so leftovers from one call must not leak into the next), and a
run of calls must leave the device's free memory unchanged.  This file is
collected last so a failure here never hides the other GPU tests.
"""
import ctypes as C

import numpy as np
import pytest

from ddevol_gb300 import native

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


def _u64(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


def _f64(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def random_batch(seed, count, spins):
    rng = np.random.default_rng(seed)
    words = (spins + 31) // 32
    keys = rng.integers(0, 2 ** 63, size=count * words, dtype=np.int64).astype(np.uint64)
    keys ^= rng.integers(0, 2, size=count * words, dtype=np.int64).astype(np.uint64) << np.uint64(63)
    rem = spins % 32
    if rem:
        keys[words - 1::words] &= np.uint64((1 << (2 * rem)) - 1)
    values = rng.standard_normal(count) * 10.0 ** rng.uniform(-300, 300, count)
    return keys, values, words


def call(lib, static, ctx, keys, values, count, words, spins, i, j, qi, qj, c, s, rc, rs, enc):
    ok = np.zeros(max(1, 2 * count * words), np.uint64)
    ov = np.zeros(max(1, 2 * count), np.float64)
    orad = np.zeros(max(1, 2 * count), np.float64)
    err = C.create_string_buffer(512)
    if static:
        st = lib.tpgp_cuda_branches_static(0, _u64(keys), _f64(values), count, words, spins, i, j,
                                           qi, qj, c, s, rc, rs, enc, _u64(ok), _f64(ov),
                                           _f64(orad), err, len(err))
    else:
        st = lib.tpgp_cuda_branches(ctx, _u64(keys), _f64(values), count, words, spins, i, j, qi,
                                    qj, c, s, rc, rs, enc, _u64(ok), _f64(ov), _f64(orad), err,
                                    len(err))
    return st, ok, ov, orad, err.value.decode()


@pytest.fixture(scope="module")
def lib_ctx():
    lib = native.load()
    err = C.create_string_buffer(256)
    ctx = lib.tpgp_cuda_create(0, err, len(err))
    assert ctx, err.value
    yield lib, ctx
    lib.tpgp_cuda_destroy(ctx)


CASES = [
    # seed, count, spins, i, j, qi, qj, c, s, rc, rs, enclose
    (11, 5000, 1000, 511, 999, 3, 1, 0.6, -0.8, 2.0 ** -54, 2.0 ** -54, 1),
    (12, 40000, 64, 63, 0, 2, 2, -0.8, 0.6, 0.0, 0.0, 0),
    (13, 70000, 16, 3, 12, 1, 3, 0.28, 0.96, 2.0 ** -60, 2.0 ** -60, 1),
]


def test_static_equals_ordinary_on_consecutive_calls(lib_ctx):
    lib, ctx = lib_ctx
    for repeat in range(2):  # two passes: every call reuses the array left by the one before
        for seed, count, spins, i, j, qi, qj, c, s, rc, rs, enc in CASES:
            keys, values, words = random_batch(seed + repeat, count, spins)
            a = call(lib, True, ctx, keys, values, count, words, spins, i, j, qi, qj, c, s, rc, rs,
                     enc)
            b = call(lib, False, ctx, keys, values, count, words, spins, i, j, qi, qj, c, s, rc, rs,
                     enc)
            assert a[0] == b[0] == 0, (a[4], b[4])
            assert np.array_equal(a[1], b[1])
            assert np.array_equal(a[2].view(np.uint64), b[2].view(np.uint64))
            assert np.array_equal(a[3].view(np.uint64), b[3].view(np.uint64))


def test_failure_flag_does_not_leak_and_limit_is_enforced(lib_ctx):
    lib, ctx = lib_ctx
    keys, values, words = random_batch(21, 1000, 64)
    bad = values.copy()
    bad[17] = np.nan
    a = call(lib, True, ctx, keys, bad, 1000, words, 64, 0, 1, 3, 3, .6, .8, 0, 0, 0)
    assert a[0] == 4  # ENUMERIC, like the ordinary entry point
    b = call(lib, True, ctx, keys, values, 1000, words, 64, 0, 1, 3, 3, .6, .8, 0, 0, 0)
    c = call(lib, False, ctx, keys, values, 1000, words, 64, 0, 1, 3, 3, .6, .8, 0, 0, 0)
    assert b[0] == c[0] == 0
    assert np.array_equal(b[2].view(np.uint64), c[2].view(np.uint64))
    # beyond the static array: a clear EINVAL, nothing touched
    big = 16 * 2 ** 20 // 64 + 1024
    keys, values, words = random_batch(22, big, 16)
    d = call(lib, True, ctx, keys, values, big, words, 16, 0, 1, 3, 3, .6, .8, 0, 0, 0)
    assert d[0] == 1 and "at most" in d[4]


def test_static_calls_leave_free_memory_unchanged(lib_ctx):
    """After a warm-up call (which loads the module and its array), a run of
    allocation-free calls of several sizes changes the device's free memory
    by nothing.  The ordinary entry point is kept out of the window."""
    torch = pytest.importorskip("torch")
    lib, _ = lib_ctx
    keys, values, words = random_batch(31, 2000, 64)
    assert call(lib, True, None, keys, values, 2000, words, 64, 0, 5, 1, 2, .6, .8, 0, 0, 0)[0] == 0
    torch.cuda.synchronize(0)
    free_before, _ = torch.cuda.mem_get_info(0)
    for seed, count, spins in ((32, 100, 16), (33, 60000, 64), (34, 3000, 1000), (35, 1, 2)):
        keys, values, words = random_batch(seed, count, spins)
        st = call(lib, True, None, keys, values, count, words, spins, 0, 1, 3, 1, .28, .96, 0, 0,
                  0)
        assert st[0] == 0, st[4]
    free_after, _ = torch.cuda.mem_get_info(0)
    assert free_after == free_before
