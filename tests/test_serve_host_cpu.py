"""The continuous-batching loop's host logic on the CPU (no GPU).

tpgp_gb_serve (ddevol_gb300/csrc/serve.cu) is host code over the batch ABI.
Here it is linked against tests/c/oracle_engine.cpp, the batch calls
restated on the CPU oracle (test infrastructure; the device batch is bitwise
the oracle, which the GPU suite checks), so its scheduling runs without a
GPU: requests arriving staggered and outnumbering the slots queue, take
slots of a sufficient width as earlier solves finish, and run interleaved;
each request's per-step FIDs must be bitwise the oracle's on the request
alone at its own spin count, however it was scheduled; a memory budget that
fits one projected solve admits one at a time; a failing request fails
alone.
"""
import ctypes as C
import os
import subprocess
import types

import numpy as np
import pytest

from ddevol_gb300 import hamiltonians as H
from ddevol_gb300 import native
from ddevol_gb300.engine import Engine, options

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def server(tmp_path_factory):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    out = tmp_path_factory.mktemp("serve_host")
    orc = os.path.join(ROOT, "oracle", "_build")
    lib = str(out / "libserve_host.so")
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-x", "c++",
                    os.path.join(ROOT, "ddevol_gb300", "csrc", "serve.cu"),
                    os.path.join(ROOT, "tests", "c", "oracle_engine.cpp"), "-o", lib,
                    "-L", orc, "-lorc", f"-Wl,-rpath,{orc}"], check=True)
    host = C.CDLL(lib)
    P, sz = C.POINTER, C.c_size_t
    host.tpgp_gb_create.restype = C.c_void_p
    host.tpgp_gb_create.argtypes = [C.c_int, C.c_char_p, sz]
    host.tpgp_gb_destroy.argtypes = [C.c_void_p]
    host.tpgp_gb_serve.restype = C.c_int
    host.tpgp_gb_serve.argtypes = [C.c_void_p, P(native.GbRequest), sz, P(sz), sz,
                                   P(C.c_double), P(native.GbResponse), P(native.GbServeStats),
                                   C.c_char_p, sz]
    ctx = host.tpgp_gb_create(0, None, 0)
    yield types.SimpleNamespace(lib=host, ptr=ctx, serve=lambda *a, **k: Engine.serve(
        types.SimpleNamespace(lib=host, ptr=ctx), *a, **k))
    host.tpgp_gb_destroy(ctx)


def make_requests(count, seed, gap):
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(count):
        n, terms, thr, steps, dt = H.serving_request(rng, steps_range=(3, 8))
        keys, vals = H.single_site_operator(n, 0)
        reqs.append(dict(arrival=k * gap, n_spins=n, terms=terms, dt=dt, steps=steps,
                         options=options(thr, exact_ledger=False), keys=keys, values=vals))
    return reqs


def oracle_fids(oracle, q):
    fo = []
    st, _, _, _ = oracle.strang_step(q["keys"], q["values"], q["n_spins"], q["terms"], q["dt"],
                                     threshold=q["options"].threshold, steps=q["steps"],
                                     on_step=lambda s, f, n: fo.append(f))
    assert st == 0
    return np.array(fo)


def test_mixed_stream_matches_the_oracle_per_request(server, oracle):
    reqs = make_requests(12, seed=21, gap=0.002)
    assert {(q["n_spins"] + 31) // 32 for q in reqs} == {1, 2, 3}
    resp, fids, stats = server.serve(reqs, slots=(2, 2, 2))
    assert stats["ticks"] >= max(q["steps"] for q in reqs) and 1 <= stats["max_active"] <= 6
    for r, q in enumerate(reqs):
        x = resp[r]
        assert x["status"] == 0
        assert x["slot_spins"] >= q["n_spins"] and x["slot_spins"] % 32 == 0
        assert x["admitted"] >= q["arrival"] - 1e-9 and x["finished"] >= x["admitted"]
        assert np.array_equal(fids[r].view(np.uint64), oracle_fids(oracle, q).view(np.uint64)), r


def test_queueing_reuses_slots_and_memory_budget_admits_one(server, oracle):
    reqs = make_requests(7, seed=22, gap=0.0)
    resp, fids, stats = server.serve(reqs, slots=(1, 1, 1))
    assert all(x["status"] == 0 for x in resp)
    assert max(x["admitted"] - q["arrival"] for x, q in zip(resp, reqs)) > 0
    # a budget below one projected solve: the server still admits a request
    # when nothing is running, and only then
    resp1, fids1, stats1 = server.serve(reqs, slots=(3, 3, 3), memory_budget=1)
    assert stats1["max_active"] == 1 and all(x["status"] == 0 for x in resp1)
    spans = sorted((x["admitted"], x["finished"]) for x in resp1)
    assert all(b[0] >= a[1] for a, b in zip(spans, spans[1:]))  # one at a time
    for r in range(len(reqs)):
        assert np.array_equal(fids1[r].view(np.uint64), fids[r].view(np.uint64)), r


def test_failing_requests_do_not_disturb_the_others(server, oracle):
    """A request that hits its term cap fails on its own (ECAP, its slot
    freed for the next request), one with an unusable time step is refused at
    admission (ENUMERIC: dt/2 inexact, as tpgp_strang_step refuses it); every
    other request's FIDs stay bitwise the oracle's."""
    reqs = make_requests(8, seed=23, gap=0.001)
    reqs[2]["options"] = options(reqs[2]["options"].threshold, max_terms=3, exact_ledger=False)
    reqs[5]["dt"] = 5e-324
    resp, fids, stats = server.serve(reqs, slots=(1, 1, 1))
    assert resp[2]["status"] == 3 and resp[5]["status"] == 4
    for r, q in enumerate(reqs):
        if r in (2, 5):
            continue
        assert resp[r]["status"] == 0
        assert np.array_equal(fids[r].view(np.uint64), oracle_fids(oracle, q).view(np.uint64)), r
