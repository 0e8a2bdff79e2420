"""The allocation-free sorted evaluation (einspline_gb300_eval_3d_sorted_noalloc).

It exists for callers that cannot let a library call cudaMalloc while they
run (their own pool allocator owns the device memory, or an allocation's
implicit synchronisation would break their timing or capture).  It must give
the same results as the allocating entry, einspline_gb300_eval_3d with
sorting, through the C-ABI, on consecutive calls that share its fixed
scratch array.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

from einspline_gb300 import _lib as L
from einspline_gb300 import api, synth

from helpers import TOL, rel_err


def _call(lib, G, opts, pos, out):
    ptr = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
    return lib.einspline_gb300_eval_3d_sorted_noalloc(G.table, C.byref(opts), pos.shape[0], ptr(pos), ptr(out[0]),
                                                      ptr(out[1]), ptr(out[2]), None)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sd")
def test_noalloc_sorted_matches_allocating_entry(kind):
    import torch
    lib = L.load()
    M, N = 24, 96
    grids = [(0.0, 1.0, M)] * 3
    G = api.MultiUBspline3D(kind, grids, [(api.PERIODIC, api.PERIODIC)] * 3, N)
    data = synth.grid_data_uniform(7, (M, M, M), N, np.float32 if kind == "s" else np.float64)
    for i in range(N):
        G.set(i, data[i])
    G.flush()
    dt = torch.float32 if kind == "s" else torch.float64
    opts = L.EvalOpts(1, 1, 0, 0, 1, 0, 0, 0)
    # two calls in a row share the scratch (counting sort), then a batch large
    # enough for the radix sort in the same scratch
    for call, (seed, n) in enumerate(((11, 5000), (12, 5037), (13, 140000))):
        pos = torch.from_numpy(synth.points_uniform(seed, n)).cuda()
        P = pos.shape[0]
        ref = G.eval(pos, vgh=True, rule=0, layout=0, sort=True)
        out = (torch.full((P, N), -1.0, dtype=dt, device="cuda"), torch.full((P, N, 3), -1.0, dtype=dt, device="cuda"),
               torch.full((P, N, 6), -1.0, dtype=dt, device="cuda"))
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = _call(lib, G, opts, pos, out)
        torch.cuda.synchronize()
        assert rc == 0, lib.einspline_gb300_last_error_message()
        if call == 1:  # set-up is done: the second call must not take device memory
            assert torch.cuda.mem_get_info()[0] == free0
        for a, b in zip(out, ref):
            a, b = a.cpu().numpy(), b.cpu().numpy()
            assert rel_err(a, b) <= TOL[kind]
            assert np.array_equal(a, b)


@pytest.mark.gpu
def test_noalloc_refuses_batches_beyond_its_scratch():
    import torch
    lib = L.load()
    G = api.MultiUBspline3D("s", [(0.0, 1.0, 8)] * 3, [(api.PERIODIC, api.PERIODIC)] * 3, 4)
    G.set(0, np.zeros((8, 8, 8), np.float32))
    opts = L.EvalOpts(0, 1, 0, 0, 1, 0, 0, 0)
    n = 262145
    pos = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    v = torch.empty((n, 4), device="cuda")
    rc = lib.einspline_gb300_eval_3d_sorted_noalloc(G.table, C.byref(opts), n, C.c_void_p(pos.data_ptr()),
                                                    C.c_void_p(v.data_ptr()), None, None, None)
    assert rc == 4  # EINSPLINE_GB300_ESIZE
    assert b"262144" in lib.einspline_gb300_last_error_message()
    lib.einspline_gb300_clear_error()
