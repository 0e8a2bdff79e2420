"""Edge cases: batches beyond the reference's 65,535-point launch limit,
tiny and odd spline counts, non-periodic tables through the reference-shaped
entry, strided host outputs, and argument errors reported as status codes."""
import ctypes as C

import numpy as np
import pytest

from einspline_gb300 import _lib as L
from einspline_gb300 import api, synth

from helpers import TOL, assert_close, build_pair, cpu_to_gpu_layout, table_box

P, D1, D2, FL, NA, AP = 0, 1, 2, 3, 4, 5


@pytest.mark.gpu
def test_more_points_than_reference_grid_limit(orc):
    import torch
    G, T, _ = build_pair(orc, "s", [(0.0, 1.0, 10)] * 3, [(P, P)] * 3, 5, seed=91)
    c = G.to_cuda()
    n = 70000
    pos = synth.points_uniform(92, n).astype(np.float32)
    v, g, h = c.eval_multi(torch.from_numpy(pos).cuda(), vgh=True)
    sub = np.r_[0:50, 65530:65545, n - 50:n]
    ref = cpu_to_gpu_layout("s", *T.eval(pos[sub].astype(np.float64), sem=1))
    got = (v.cpu().numpy()[sub], g.cpu().numpy()[sub].reshape(-1, 5, 3), h.cpu().numpy()[sub].reshape(-1, 5, 6))
    assert_close(got, ref, TOL["s"], "70k points")


@pytest.mark.gpu
@pytest.mark.parametrize("kind,N", [("s", 1), ("s", 33), ("c", 1), ("d", 3), ("z", 5)])
def test_small_and_odd_spline_counts(orc, kind, N):
    import torch
    grids, bcs = [(0.0, 2.0, 7), (1.0, 2.0, 9), (-1.0, 0.0, 6)], [(P, P), (NA, FL), (AP, AP)]
    G, T, _ = build_pair(orc, kind, grids, bcs, N, seed=93)
    lo, hi = table_box(grids)
    pos = synth.points_uniform(94, 123, lo, hi)
    got = [x.cpu().numpy() for x in G.eval(torch.from_numpy(pos).cuda(), rule=0, layout=1)]
    assert_close(got, T.eval(pos, sem=0), TOL[kind], f"{kind} N={N}")


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sd")
def test_nonperiodic_table_through_cuda_entry(orc, kind):
    """The reference's create_*_cuda assumes periodic tables
    (src/multi_bspline_create_cuda.cu:449); here any boundary condition works,
    with dim = cells per axis and the reference's clamp rule."""
    import torch
    grids = [(0.0, 1.5, 10), (0.0, 1.0, 8), (0.0, 2.0, 9)]
    bcs = [(NA, NA), (D1, D2, 0.3, 0.0, -0.2, 0.0), (FL, FL)]
    G, T, _ = build_pair(orc, kind, grids, bcs, 11, seed=95)
    c = G.to_cuda()
    assert (c.fields.dim.x, c.fields.dim.y, c.fields.dim.z) == (9, 7, 8)
    pos = synth.points_uniform(96, 200, (0, 0, 0), (1.5, 1.0, 2.0))
    f64 = kind == "d"
    if not f64:
        pos = pos.astype(np.float32).astype(np.float64)
    dt = torch.float64 if f64 else torch.float32
    v, g, h = c.eval_multi(torch.from_numpy(pos).to(dt).cuda(), vgh=True)
    ref = cpu_to_gpu_layout(kind, *T.eval(pos, sem=1))
    got = (v.cpu().numpy(), g.cpu().numpy().reshape(ref[1].shape), h.cpu().numpy().reshape(ref[2].shape))
    assert_close(got, ref, TOL[kind], "non-periodic cuda entry")


@pytest.mark.gpu
def test_host_entry_with_strides(orc):
    G, T, _ = build_pair(orc, "s", [(0.0, 1.0, 12)] * 3, [(P, P)] * 3, 9, seed=97)
    pos = synth.points_uniform(98, 40)
    vs, gs, hs = 13, 3 * 9 + 2, 6 * 9 + 1
    v = np.full((40, vs), -5.0, np.float32)
    g = np.full((40, gs), -5.0, np.float32)
    h = np.full((40, hs), -5.0, np.float32)
    o = L.EvalOpts(1, 1, 0, 0, 0, vs, gs, hs)
    L.load().einspline_gb300_eval_3d_host(G.table, C.byref(o), 40, C.c_void_p(pos.ctypes.data),
                                          C.c_void_p(v.ctypes.data), C.c_void_p(g.ctypes.data),
                                          C.c_void_p(h.ctypes.data))
    api.check()
    ref = cpu_to_gpu_layout("s", *T.eval(pos, sem=0))
    assert_close((v[:, :9], g[:, :27].reshape(40, 9, 3), h[:, :54].reshape(40, 9, 6)), ref, TOL["s"], "strided host")
    assert (v[:, 9:] == -5).all() and (g[:, 27:] == -5).all() and (h[:, 54:] == -5).all()


@pytest.mark.gpu
@pytest.mark.parametrize("pad", [0, 3])
def test_host_entry_many_chunks(pad):
    """1024 splines (output chunks of about 200 points, then twice as many
    each time up to about 3,300), 5,000 points: five chunks on the two
    pipeline streams, the last partial, into packed host rows (one linear
    copy per output) or rows `pad` elements longer (strided copies);
    bit-identical to the device entry."""
    import torch
    n, npts = 1024, 5000
    G = api.MultiUBspline3D("s", [(0.0, 1.0, 8)] * 3, [(P, P)] * 3, n)
    buf = torch.empty((n, 8, 8, 8), dtype=torch.float32, device="cuda")
    api.fill_uniform(buf, 411, -1.0, 1.0)
    G.set_device(0, buf)
    G.flush()
    pos = synth.points_uniform(412, npts)
    ref = [x.cpu().numpy() for x in G.eval(torch.from_numpy(pos).cuda(), rule=0, layout=0)]
    vs, gs, hs = n + pad, 3 * n + pad, 6 * n + pad
    v = np.full((npts, vs), -5.0, np.float32)
    g = np.full((npts, gs), -5.0, np.float32)
    h = np.full((npts, hs), -5.0, np.float32)
    o = L.EvalOpts(1, 1, 0, 0, 0, vs, gs, hs)
    L.load().einspline_gb300_eval_3d_host(G.table, C.byref(o), npts, C.c_void_p(pos.ctypes.data),
                                          C.c_void_p(v.ctypes.data), C.c_void_p(g.ctypes.data),
                                          C.c_void_p(h.ctypes.data))
    api.check()
    assert np.array_equal(v[:, :n], ref[0])
    assert np.array_equal(g[:, :3 * n].reshape(npts, n, 3), ref[1])
    assert np.array_equal(h[:, :6 * n].reshape(npts, n, 6), ref[2])
    assert (v[:, n:] == -5).all() and (g[:, 3 * n:] == -5).all() and (h[:, 6 * n:] == -5).all()


@pytest.mark.gpu
def test_argument_errors_on_gpu():
    lib = L.load()
    G = api.MultiUBspline3D("s", [(0.0, 1.0, 8)] * 3, [(P, P)] * 3, 4)
    with pytest.raises(api.EinsplineError, match="outside"):
        G.set(4, np.zeros((8, 8, 8), np.float32))
    with pytest.raises(api.EinsplineError, match="outside"):
        G.set(-1, np.zeros((8, 8, 8), np.float32))
    o = L.EvalOpts(1, 1, 0, 0, 0, 0, 0, 0)
    rc = lib.einspline_gb300_eval_3d(G.table, C.byref(o), 10, None, None, None, None, None)
    assert rc == 1 and b"NULL" in lib.einspline_gb300_last_error_message()
    assert lib.einspline_gb300_set_tile(G.table, 48, 1, 1) == 1
    assert lib.einspline_gb300_set_load_mode(G.table, 7) == 1
    lib.einspline_gb300_clear_error()
    with pytest.raises(ValueError):
        api.MultiUBspline3D("d", [(0.0, 1.0, 8)] * 3, [(P, P)] * 3, 4, storage=api.STORE_F16)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1])
def test_host_entry_copy_and_direct_modes_agree(orc, mode):
    """Pinned buffers: results written by the kernel straight into mapped host
    memory (mode 1) or staged through device memory (mode 0) are identical."""
    import torch
    G, T, _ = build_pair(orc, "s", [(0.0, 1.0, 12)] * 3, [(P, P)] * 3, 16, seed=99)
    pos = torch.from_numpy(synth.points_uniform(100, 500)).pin_memory()
    out = (torch.empty((500, 16), pin_memory=True), torch.empty((500, 16, 3), pin_memory=True),
           torch.empty((500, 16, 6), pin_memory=True))
    G.set_host_direct(mode)
    got = G.eval_host(pos.numpy(), out=tuple(o.numpy() for o in out))
    G.set_host_direct(0)
    ref = [x.cpu().numpy() for x in G.eval(pos.cuda(), rule=0, layout=0)]
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_empty_batches_launch_nothing(orc):
    """Zero points (or walkers) is a valid batch for every batched entry: no
    kernel runs, nothing is written, no error is left.  A request server
    refuses an empty request (there is nothing to wait for)."""
    import torch
    lib = L.load()
    G, T, _ = build_pair(orc, "s", [(0.0, 1.0, 10)] * 3, [(P, P)] * 3, 6, seed=141)
    C1 = G.to_cuda()
    empty = torch.empty((0, 3), dtype=torch.float64, device="cuda")
    opts = L.EvalOpts(1, 1, 0, 0, 1, 0, 0, 0)
    # the allocation-free entry's first call on a device is its set-up (it
    # loads its kernels, running its sort once); empty calls after it launch
    # nothing
    assert lib.einspline_gb300_eval_3d_sorted_noalloc(G.table, C.byref(opts), 0, None, None, None, None, None) == 0
    torch.cuda.synchronize()
    n0 = api.launch_count()
    for sort in (False, True):
        v, g, h = G.eval(empty, sort=sort)
        assert v.shape[0] == 0 and g.shape[0] == 0 and h.shape[0] == 0
    v, g, h = G.eval_host(np.zeros((0, 3)))
    assert v.shape[0] == 0
    v, g, h = C1.eval_multi(empty.float())
    assert v.shape[0] == 0
    assert lib.einspline_gb300_eval_3d_sorted_noalloc(G.table, C.byref(opts), 0, C.c_void_p(1), C.c_void_p(1),
                                                      C.c_void_p(1), C.c_void_p(1), None) == 0
    dopts = L.DetOpts(6, 0, 6, 1, 0)
    assert lib.einspline_gb300_det_ratio(G.table, C.byref(dopts), 0, *([None] * 7)) == 0
    assert lib.einspline_gb300_det_update(C.byref(dopts), 0, None, None, None, None, None) == 0
    torch.cuda.synchronize()
    assert api.launch_count() == n0
    assert lib.einspline_gb300_last_error() == 0
    S = api.Server(G)
    with pytest.raises(api.EinsplineError):
        S.submit(np.zeros((0, 3)))
    S.close()
    C1.destroy()
