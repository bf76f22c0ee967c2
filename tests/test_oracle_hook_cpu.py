"""The oracle's branch hook (oracle/tpgp_oracle.h, orc_set_branch_backend).

tests/c/branch_backend.c runs the oracle's Strang step with its raw children
taken from the GPU through this hook, the way the reference engine takes them
from its CUDA backend (engine/src/tpgp_rev.c:622-640).  Here, on the CPU, the
hook itself is checked: children from a hook that computes them with the
oracle's own branch give the same trajectory bit for bit as the built-in
loop, and a hook's failure status stops the step with the map and ledger
untouched (the step is transactional, tpgp_rev.c:776-809).
"""
import ctypes as C

import numpy as np

from ddevol_gb300 import hamiltonians as H
from oracle.oracle import LedgerStruct, terms_array

HOOK = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.c_size_t,
                   C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t, C.c_uint, C.c_uint,
                   C.c_double, C.c_double, C.POINTER(C.c_uint64), C.POINTER(C.c_double))


def run(oracle, keys, values, n_spins, terms, dt, threshold, steps, hook=None):
    lib = oracle.lib
    lib.orc_set_branch_backend.argtypes = [HOOK, C.c_void_p]
    arr, count = terms_array(terms)
    m = oracle._map(keys, values, n_spins)
    led = LedgerStruct()
    statuses = []
    try:
        lib.orc_set_branch_backend(hook if hook is not None else HOOK(), None)
        for _ in range(steps):
            statuses.append(lib.orc_strang_step(C.byref(m), arr, count, dt, threshold, 0, 0.0, 1,
                                                C.byref(led)))
    finally:
        lib.orc_set_branch_backend(HOOK(), None)
    k, v = oracle._unmap(m)
    return statuses, k, v, led


def test_hook_children_give_the_builtin_trajectory(oracle):
    calls = []

    @HOOK
    def branch(user, keys, values, count, words, spins, i, j, qi, qj, c, s, out_keys, out_values):
        radii = (C.c_double * (2 * count))()
        calls.append(count)
        st = oracle.lib.orc_branches(keys, values, count, words, spins, i, j, qi, qj, c, s, 0.0,
                                     0.0, 0, out_keys, out_values, radii)
        return 0 if st == 0 else 5

    terms = H.ring_j1j2(10)
    k0, v0 = H.global_x_operator(10)
    a = run(oracle, k0, v0, 10, terms, 0.01, 1e-6, 4)
    b = run(oracle, k0, v0, 10, terms, 0.01, 1e-6, 4, hook=branch)
    assert a[0] == b[0] == [0, 0, 0, 0]
    assert len(calls) == b[3].rotations == 4 * 2 * len(terms)
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[2].view(np.uint64), b[2].view(np.uint64))
    assert a[3].as_dict() == b[3].as_dict()


def test_hook_failure_leaves_the_map_and_ledger(oracle):
    for code in (5, 4, 2):  # EBACKEND, ENUMERIC, ENOMEM pass through as the step's status
        seen = []

        @HOOK
        def failing(user, keys, values, count, *rest):
            seen.append(count)
            return code if len(seen) == 7 else oracle.lib.orc_branches(
                keys, values, count, *rest[:8], 0.0, 0.0, 0, rest[8], rest[9],
                (C.c_double * (2 * count))())

        terms = H.ring_j1j2(8)
        k0, v0 = H.single_site_operator(8)
        good = run(oracle, k0, v0, 8, terms, 0.01, 1e-6, 1)
        statuses, k, v, led = run(oracle, k0, v0, 8, terms, 0.01, 1e-6, 2, hook=failing)
        # the first step's 7th rotation fails; the second step runs in full
        assert statuses[0] == code and statuses[1] == 0
        assert np.array_equal(k, good[1]) and np.array_equal(v.view(np.uint64),
                                                             good[2].view(np.uint64))
        assert led.as_dict() == good[3].as_dict()
