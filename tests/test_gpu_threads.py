"""Host threads sharing the library: tables created, set (solved) and
evaluated concurrently from several threads give the same bits as the same
work done one table at a time; threads evaluating one shared table on their
own streams do too; and the error status is per thread (a thread whose calls
fail does not change what another thread's error query returns).  The
reference's GPU path is not re-entrant (one global basis constant, the
default stream, a blocking sync per call); these are the library's
replacements for that."""
import ctypes as C
import threading

import numpy as np
import pytest

from einspline_gb300 import _lib as L
from einspline_gb300 import api, synth

GRID = [(0.0, 1.0, 16), (0.0, 1.0, 14), (0.0, 1.0, 15)]
PER = [(api.PERIODIC, api.PERIODIC)] * 3


def _build_and_eval(kind, seed, npts, storage=api.STORE_NATIVE):
    import torch
    N = 24
    G = api.MultiUBspline3D(kind, GRID, PER, N, storage=storage)
    dt = np.float32 if kind == "s" else np.float64
    data = synth.grid_data_uniform(seed, (16, 14, 15), N, dt)
    for i in range(N):
        G.set(i, data[i])
    G.flush()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        pos = torch.from_numpy(synth.points_uniform(seed + 1, npts)).cuda()
        out = G.eval(pos, rule=0, layout=0, stream=s)
    s.synchronize()
    return [x.cpu().numpy() for x in out]


def _run_threads(fns):
    barrier = threading.Barrier(len(fns))
    results, errors = [None] * len(fns), []

    def wrap(i, fn):
        try:
            barrier.wait()
            results[i] = fn()
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(repr(e))

    ts = [threading.Thread(target=wrap, args=(i, f)) for i, f in enumerate(fns)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=300)
    assert not any(t.is_alive() for t in ts), "a thread did not finish"
    assert not errors, errors
    return results


@pytest.mark.gpu
def test_tables_built_and_evaluated_concurrently():
    jobs = [("s", 301, 3000, api.STORE_NATIVE), ("d", 302, 2000, api.STORE_NATIVE), ("s", 303, 4000, api.STORE_F16),
            ("s", 304, 2500, api.STORE_NATIVE), ("d", 305, 1500, api.STORE_NATIVE), ("s", 306, 3500, api.STORE_I16)]
    ref = [_build_and_eval(*j) for j in jobs]
    for _ in range(2):
        got = _run_threads([lambda j=j: _build_and_eval(*j) for j in jobs])
        for r, g, j in zip(ref, got, jobs):
            for a, b in zip(g, r):
                assert np.array_equal(a, b), j


@pytest.mark.gpu
def test_threads_share_one_table():
    import torch
    N = 40
    G = api.MultiUBspline3D("s", GRID, PER, N, storage=api.STORE_F16)
    G.set_device(0, torch.from_numpy(synth.grid_data_uniform(311, (16, 14, 15), N, np.float32)).cuda())
    G.flush()
    pos = [torch.from_numpy(synth.points_uniform(312 + k, 2000 + 300 * k)).cuda() for k in range(6)]
    ref = [[x.cpu().numpy() for x in G.eval(p, rule=1, layout=1)] for p in pos]

    def work(k):
        s = torch.cuda.Stream()
        outs = []
        for _ in range(5):
            with torch.cuda.stream(s):
                outs.append(G.eval(pos[k], rule=1, layout=1, stream=s))
        s.synchronize()
        return [[x.cpu().numpy() for x in o] for o in outs]

    got = _run_threads([lambda k=k: work(k) for k in range(6)])
    for k in range(6):
        for rep in got[k]:
            for a, b in zip(rep, ref[k]):
                assert np.array_equal(a, b), k


@pytest.mark.gpu
def test_error_status_is_per_thread():
    import torch
    lib = L.load()
    G = api.MultiUBspline3D("s", GRID, PER, 8)
    G.set_device(0, torch.from_numpy(synth.grid_data_uniform(321, (16, 14, 15), 8, np.float32)).cuda())
    G.flush()
    pos = torch.from_numpy(synth.points_uniform(322, 500)).cuda()
    stop = threading.Event()
    seen = {"bad": 0, "good": 0, "good_nonzero": 0}

    def failing():
        while not stop.is_set():
            # an invalid tile: the call fails and sets this thread's status
            if lib.einspline_gb300_set_tile(G.table, 48, 1, 1) != 0 and lib.einspline_gb300_last_error() != 0:
                seen["bad"] += 1
            lib.einspline_gb300_clear_error()

    def good():
        s = torch.cuda.Stream()
        out = (torch.empty((500, 8), device="cuda"), torch.empty((500, 8, 3), device="cuda"),
               torch.empty((500, 8, 6), device="cuda"))
        o = G.opts(True, True, 0, 0, False)
        for _ in range(300):
            rc = lib.einspline_gb300_eval_3d(G.table, C.byref(o), 500, C.c_void_p(pos.data_ptr()),
                                             C.c_void_p(out[0].data_ptr()), C.c_void_p(out[1].data_ptr()),
                                             C.c_void_p(out[2].data_ptr()), C.c_void_p(s.cuda_stream))
            if rc != 0 or lib.einspline_gb300_last_error() != 0:
                seen["good_nonzero"] += 1
            seen["good"] += 1
        s.synchronize()

    t = threading.Thread(target=failing)
    t.start()
    try:
        good()
    finally:
        stop.set()
        t.join(timeout=60)
    assert seen["bad"] > 0 and seen["good"] == 300
    assert seen["good_nonzero"] == 0
