"""Known answers from the reference's own test (test_core_rev.c:36-79, local_dense).

Every two-site conjugation exp(-i t Q) P exp(+i t Q), Q, P in {I,X,Y,Z}^2, is
compared with independent 4x4 complex matrices at tolerance 8e-16.  Runs the
CPU oracle here; the GPU variant lives in test_rotate_gpu.py.
"""
import numpy as np

PAULI = [np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]),
         np.array([[1, 0], [0, -1]])]


def two_site(a, b):
    # site 0 is the low bit of the basis index, as in test_core_rev.c:21-27
    return np.kron(PAULI[b], PAULI[a])


def dense_conjugation(qa, qb, pa, pb, theta):
    q = two_site(qa, qb)
    u = np.cos(theta) * np.eye(4) - 1j * np.sin(theta) * q
    ud = np.cos(theta) * np.eye(4) + 1j * np.sin(theta) * q
    r = u @ two_site(pa, pb) @ ud
    out = {}
    for a in range(4):
        for b in range(4):
            coef = np.trace(two_site(a, b).conj().T @ r) / 4
            out[a | (b << 2)] = coef
    return out


def local_dense_cases():
    for qa in range(4):
        for qb in range(4):
            for pa in range(4):
                for pb in range(4):
                    yield qa, qb, pa, pb


def check_local_dense(rotate):
    """rotate(key, value, qa, qb, theta) -> dict key -> value"""
    theta = 0.371
    n = 0
    for qa, qb, pa, pb in local_dense_cases():
        got = rotate(np.array([pa | (pb << 2)], np.uint64), np.array([1.0]), qa, qb, theta)
        want = dense_conjugation(qa, qb, pa, pb, theta)
        for key, coef in want.items():
            assert abs(got.get(key, 0.0) - coef.real) < 8e-16
            assert abs(coef.imag) < 1e-15
        assert abs(np.sqrt(sum(v * v for v in got.values())) - 1) < 5e-16
        n += 1
    assert n == 256


def test_local_dense_oracle(oracle):
    def rotate(keys, values, qa, qb, theta):
        st, k, v, _ = oracle.rotate(keys, values, 2, 0, 1, qa, qb, theta, 1.0)
        assert st == 0
        return {int(a): float(b) for a, b in zip(k, v)}
    check_local_dense(rotate)
