"""The allocation-free sorted evaluation (einspline_gb300_eval_3d_sorted_noalloc).

It exists for callers that cannot let a library call cudaMalloc while they
run (their own pool allocator owns the device memory, or an allocation's
implicit synchronisation would break their timing or capture).  It must give
the same results as the allocating entry, einspline_gb300_eval_3d with
sorting, through the C-ABI, on consecutive calls that share its fixed
scratch array; after its set-up (an empty warm-up call) no call may take
device memory, up to the largest batch it accepts.  This file is collected
last on purpose."""
import ctypes as C

import numpy as np
import pytest

from einspline_gb300 import _lib as L
from einspline_gb300 import api, synth

from helpers import TOL

MAX_POINTS = 262144  # the entry's fixed limit


def _call(lib, G, opts, npts, pos, out):
    ptr = lambda t: C.c_void_p(t.data_ptr() if t is not None else 0)  # noqa: E731
    return lib.einspline_gb300_eval_3d_sorted_noalloc(G.table, C.byref(opts), npts, ptr(pos), ptr(out[0]),
                                                      ptr(out[1]), ptr(out[2]), None)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,storage", [("s", api.STORE_NATIVE), ("d", api.STORE_NATIVE), ("s", api.STORE_F16)])
def test_noalloc_sorted_matches_allocating_entry(kind, storage):
    """FP32 and FP64 tables, and an F16 table, which evaluates on the tensor
    cores (their tensor memory is on-chip, not device memory)."""
    import torch
    lib = L.load()
    M, N = 24, 96
    grids = [(0.0, 1.0, M)] * 3
    G = api.MultiUBspline3D(kind, grids, [(api.PERIODIC, api.PERIODIC)] * 3, N, storage=storage)
    data = synth.grid_data_uniform(7, (M, M, M), N, np.float32 if kind == "s" else np.float64)
    for i in range(N):
        G.set(i, data[i])
    G.flush()
    dt = torch.float32 if kind == "s" else torch.float64
    opts = L.EvalOpts(1, 1, 0, 0, 1, 0, 0, 0)
    # two calls in a row share the scratch (counting sort), then batches
    # large enough for the radix sort in the same scratch, the last one at
    # the entry's limit (the sort's largest work space)
    cases = ((11, 5000), (12, 5037), (13, 140000), (14, MAX_POINTS))
    pos, ref, out = [], [], []
    for seed, n in cases:
        p = torch.from_numpy(synth.points_uniform(seed, n)).cuda()
        pos.append(p)
        ref.append(G.eval(p, vgh=True, rule=0, layout=0, sort=True))
        out.append((torch.full((n, N), -1.0, dtype=dt, device="cuda"),
                    torch.full((n, N, 3), -1.0, dtype=dt, device="cuda"),
                    torch.full((n, N, 6), -1.0, dtype=dt, device="cuda")))
    torch.cuda.synchronize()
    # set-up: an empty call with the options of the calls below
    assert _call(lib, G, opts, 0, None, (None, None, None)) == 0, lib.einspline_gb300_last_error_message()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for (seed, n), p, o in zip(cases, pos, out):
        rc = _call(lib, G, opts, n, p, o)
        torch.cuda.synchronize()
        assert rc == 0, lib.einspline_gb300_last_error_message()
        assert torch.cuda.mem_get_info()[0] == free0, f"call with {n} points took device memory"
    for (seed, n), o, r in zip(cases, out, ref):
        for a, b in zip(o, r):
            den = float(b.abs().max())
            assert float((a - b).abs().max()) / den <= TOL[kind]
            assert torch.equal(a, b), f"{n} points: not bit-identical to the allocating entry"


@pytest.mark.gpu
def test_noalloc_refuses_batches_beyond_its_scratch():
    import torch
    lib = L.load()
    G = api.MultiUBspline3D("s", [(0.0, 1.0, 8)] * 3, [(api.PERIODIC, api.PERIODIC)] * 3, 4)
    G.set(0, np.zeros((8, 8, 8), np.float32))
    opts = L.EvalOpts(0, 1, 0, 0, 1, 0, 0, 0)
    n = MAX_POINTS + 1
    pos = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    v = torch.empty((n, 4), device="cuda")
    rc = lib.einspline_gb300_eval_3d_sorted_noalloc(G.table, C.byref(opts), n, C.c_void_p(pos.data_ptr()),
                                                    C.c_void_p(v.data_ptr()), None, None, None)
    assert rc == 4  # EINSPLINE_GB300_ESIZE
    assert b"262144" in lib.einspline_gb300_last_error_message()
    lib.einspline_gb300_clear_error()
