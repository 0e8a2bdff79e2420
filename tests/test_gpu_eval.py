"""GPU evaluation against the oracle on the same table, for every entry:
the CPU-shaped single-point calls, the flat batched extension in both cell
rules and layouts, and the reference-shaped eval_multi_multi_*_cuda calls
with per-point pointer arrays."""
import numpy as np
import pytest

from einspline_gb300 import api, synth

from helpers import TOL, assert_close, build_pair, cpu_to_gpu_layout, table_box

P, D1, D2, FL, NA, AP = 0, 1, 2, 3, 4, 5

PERIODIC_UNIT = [(0.0, 1.0, 14), (0.0, 1.0, 12), (0.0, 1.0, 13)]
MIXED = ([(0.3, 1.9, 9), (-1.0, 1.0, 13), (0.0, 2.5, 8)],
         [(NA, D1, 0.0, 0.0, 0.4, -0.2), (AP, AP), (D2, FL, 0.6, 0.1, 0.0, 0.0)])


def torch_pos(pos, f64=True):
    import torch
    return torch.from_numpy(np.ascontiguousarray(pos, np.float64 if f64 else np.float32)).cuda()


def oracle_table(G, T):
    """The oracle evaluates the GPU's own stored table (dequantized for
    16-bit storage) so that only evaluation is compared here."""
    if G.info().storage in (api.STORE_F16, api.STORE_BF16, api.STORE_I16):
        v = G.table_values().astype(np.float32)
        return np.ascontiguousarray(v)
    return None


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sdcz")
@pytest.mark.parametrize("bcase", ["periodic", "mixed"])
def test_single_point_cpu_entry(orc, kind, bcase):
    grids, bcs = (PERIODIC_UNIT, [(P, P)] * 3) if bcase == "periodic" else MIXED
    G, T, _ = build_pair(orc, kind, grids, bcs, 10, seed=41)
    lo, hi = table_box(grids)
    pos = synth.points_uniform(42, 12, lo, hi)
    for p in pos:
        got_v = G.eval_point(*p, vgh=False)
        got = G.eval_point(*p, vgh=True)
        ref = T.eval(p[None], vgh=True)
        ref = tuple(r[0] for r in ref)
        assert_close(got, ref, TOL[kind], f"{kind} vgh")
        assert np.array_equal(got_v[0], got[0])  # value-only equals vgh's value


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sdcz")
@pytest.mark.parametrize("layout", [0, 1])
def test_batched_rule0(orc, kind, layout):
    grids, bcs = MIXED
    G, T, _ = build_pair(orc, kind, grids, bcs, 21, seed=43)
    lo, hi = table_box(grids)
    pos = synth.points_uniform(44, 300, lo, hi)
    got = [x.cpu().numpy() for x in G.eval(torch_pos(pos), vgh=True, rule=0, layout=layout)]
    ref = T.eval(pos, vgh=True, sem=0)
    if layout == 0:
        ref = cpu_to_gpu_layout(kind, *ref)
    assert_close(got, ref, TOL[kind], f"{kind} layout{layout}")
    val = G.eval(torch_pos(pos), vgh=False, rule=0, layout=layout)[0].cpu().numpy()
    assert np.array_equal(val, got[0])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sdcz")
def test_reference_cuda_entry(orc, kind):
    """eval_multi_multi_UBspline_3d_*_vgh_cuda: positions from the grid
    origin, cell clamped, GPU layout, pointer arrays."""
    grids = PERIODIC_UNIT
    bcs = [(P, P)] * 3
    G, T, _ = build_pair(orc, kind, grids, bcs, 37, seed=45)
    c = G.to_cuda()
    f = c.fields
    assert f.dim.x == 14 and f.dim.y == 12 and f.dim.z == 13 and f.num_splines == 37
    pos = synth.points_uniform(46, 257, (0, 0, 0), (1, 1, 1))
    f64 = kind in "dz"
    if not f64:
        pos = pos.astype(np.float32).astype(np.float64)
    v, g, h = c.eval_multi(torch_pos(pos, f64), vgh=True)
    ref = cpu_to_gpu_layout(kind, *T.eval(pos, vgh=True, sem=1))
    P_ = pos.shape[0]
    got = (v.cpu().numpy().reshape(ref[0].shape), g.cpu().numpy().reshape(ref[1].shape),
           h.cpu().numpy().reshape(ref[2].shape))
    assert_close(got, ref, TOL[kind], f"{kind} cuda entry")
    v0, _, _ = c.eval_multi(torch_pos(pos, f64), vgh=False)
    assert np.array_equal(v0.cpu().numpy(), v.cpu().numpy())
    # clamped cells: points outside [0, 1) are clamped as the reference does
    out = np.array([[-0.2, 0.5, 1.3], [1.0, 1.0, 1.0], [0.0, 0.0, 0.0]])
    v1, g1, h1 = c.eval_multi(torch_pos(out, f64), vgh=True)
    ref1 = cpu_to_gpu_layout(kind, *T.eval(out, vgh=True, sem=1))
    assert_close((v1.cpu().numpy().reshape(ref1[0].shape), g1.cpu().numpy().reshape(ref1[1].shape),
                  h1.cpu().numpy().reshape(ref1[2].shape)), ref1, TOL[kind], f"{kind} clamped")
    del P_


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sd")
def test_edges_and_outside_points(orc, kind):
    """Points on and beyond the box edges: the edge cell is extrapolated
    (rule 0) exactly as the oracle does."""
    grids, bcs = MIXED
    G, T, _ = build_pair(orc, kind, grids, bcs, 8, seed=47)
    lo, hi = table_box(grids)
    pts = np.array([lo, hi, [lo[0] - 0.1, hi[1] + 0.05, 0.5 * (lo[2] + hi[2])],
                    [np.nextafter(hi[0], 0), lo[1], hi[2]]])
    got = [x.cpu().numpy() for x in G.eval(torch_pos(pts), rule=0, layout=1)]
    assert_close(got, T.eval(pts, sem=0), TOL[kind], "edges")


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [api.STORE_F16, api.STORE_BF16, api.STORE_I16])
def test_16bit_eval_matches_oracle_on_same_table(orc, storage):
    grids, bcs = MIXED
    G, T, _ = build_pair(orc, "s", grids, bcs, 24, seed=49, storage=storage)
    lo, hi = table_box(grids)
    pos = synth.points_uniform(50, 200, lo, hi)
    got = [x.cpu().numpy() for x in G.eval(torch_pos(pos), rule=0, layout=1)]
    ref = T.eval(pos, sem=0, coefs=oracle_table(G, T))
    assert_close(got, ref, TOL["s"], "16-bit")


@pytest.mark.gpu
@pytest.mark.parametrize("storage,mode", [(api.STORE_NATIVE, 0), (api.STORE_NATIVE, 2), (api.STORE_F16, 3),
                                          (api.STORE_F16, 4)])
def test_last_wave_groups_are_bit_identical(storage, mode):
    """A batch of many waves gives its last wave's points to blocks of pb/4
    points; results equal a launch of one point per block (no such split),
    in every load mode, sorted and unsorted."""
    import torch
    G = api.MultiUBspline3D("s", PERIODIC_UNIT, [(P, P)] * 3, 45, storage=storage)
    data = synth.grid_data_uniform(61, (14, 12, 13), 45, np.float32)
    G.set_device(0, torch.from_numpy(data).cuda())
    G.flush()
    pt = torch_pos(synth.points_uniform(62, 120000, (0, 0, 0), (1, 1, 1)))
    G.set_load_mode(0)
    G.set_tile(32, 1, 1)
    base = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0)]
    G.set_load_mode(mode)
    for shape in [(32, 1, 8), (32, 1, 16), (64, 1, 5)]:
        G.set_tile(*shape)
        for srt in (False, True):
            got = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0, sort=srt)]
            G.wait_status()
            for a, b in zip(got, base):
                assert np.array_equal(a, b), (shape, srt)
    G.set_load_mode(-1)
    G.set_tile(0, 0, 0)


@pytest.mark.gpu
def test_sorted_batches_of_changing_size_share_the_sort_scratch():
    """Sorted calls on one table alternate between the counting sort (up
    to 131,072 points, 16 to 64 slices) and the radix sort of larger batches
    over the same scratch; every call equals the unsorted evaluation bit for
    bit."""
    import torch
    G = api.MultiUBspline3D("s", PERIODIC_UNIT, [(P, P)] * 3, 45, storage=api.STORE_F16)
    G.set_device(0, torch.from_numpy(synth.grid_data_uniform(71, (14, 12, 13), 45, np.float32)).cuda())
    G.flush()
    for i, n in enumerate([5000, 140000, 3000, 3001, 32768, 32769, 2, 100, 131072, 131073, 70000, 17000]):
        pt = torch_pos(synth.points_uniform(72 + i, n, (0, 0, 0), (1, 1, 1)))
        base = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0)]
        got = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0, sort=True)]
        for a, b in zip(got, base):
            assert np.array_equal(a, b), n


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sz")
def test_shapes_sorting_and_host_entry_are_bit_identical(orc, kind):
    """Results do not depend on the launch shape, on cell sorting, on batch
    composition or on the host-buffer pipeline."""
    import torch
    grids, bcs = PERIODIC_UNIT, [(P, P)] * 3
    G, T, _ = build_pair(orc, kind, grids, bcs, 45, seed=51)
    pos = synth.points_uniform(52, 1000, (0, 0, 0), (1, 1, 1))
    pt = torch_pos(pos)
    base = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0)]
    for tx, ty, pb in [(32, 1, 1), (32, 8, 16), (64, 2, 8), (128, 1, 3), (256, 1, 64)]:
        G.set_tile(tx, ty, pb)
        got = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0)]
        for a, b in zip(got, base):
            assert np.array_equal(a, b), (tx, ty, pb)
    for mode, shapes in ((1, [(32, 2, 8), (256, 1, 4)]), (2, [(32, 1, 1), (64, 1, 5), (256, 1, 16)]),
                         (3, [(32, 1, 3), (128, 1, 8)])):
        G.set_load_mode(mode)
        for tx, ty, pb in shapes:
            G.set_tile(tx, ty, pb)
            got = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0)]
            for a, b in zip(got, base):
                assert np.array_equal(a, b), ("mode", mode, tx, ty, pb)
    G.set_load_mode(-1)
    G.set_tile(0, 0, 0)
    srt = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0, sort=True)]
    for a, b in zip(srt, base):
        assert np.array_equal(a, b)
    host = G.eval_host(np.ascontiguousarray(pos), rule=0, layout=0)
    for a, b in zip(host, base):
        assert np.array_equal(a, b)
    # a sub-batch alone equals the same points inside the full batch
    part = [x.cpu().numpy() for x in G.eval(pt[300:417], rule=0, layout=0)]
    for a, b in zip(part, base):
        assert np.array_equal(a, b[300:417])


@pytest.mark.gpu
def test_unaligned_strided_outputs(orc):
    """Per-point output strides that break 16-byte alignment fall back to
    scalar stores and still land every value."""
    import torch
    grids, bcs = PERIODIC_UNIT, [(P, P)] * 3
    N = 7
    G, T, _ = build_pair(orc, "s", grids, bcs, N, seed=53)
    pos = synth.points_uniform(54, 33, (0, 0, 0), (1, 1, 1))
    vs, gs, hs = N + 3, 3 * N + 1, 6 * N + 5
    v = torch.full((33, vs), -7.0, device="cuda")
    g = torch.full((33, gs), -7.0, device="cuda")
    h = torch.full((33, hs), -7.0, device="cuda")
    import ctypes as C
    from einspline_gb300 import _lib as L
    o = L.EvalOpts(1, 1, 0, 0, 0, vs, gs, hs)
    pt = torch_pos(pos)
    L.load().einspline_gb300_eval_3d(G.table, C.byref(o), 33, C.c_void_p(pt.data_ptr()), C.c_void_p(v.data_ptr()),
                                     C.c_void_p(g.data_ptr()), C.c_void_p(h.data_ptr()), None)
    torch.cuda.synchronize()
    ref = cpu_to_gpu_layout("s", *T.eval(pos, sem=0))
    got = (v[:, :N].cpu().numpy(), g[:, :3 * N].cpu().numpy().reshape(33, N, 3),
           h[:, :6 * N].cpu().numpy().reshape(33, N, 6))
    assert_close(got, ref, TOL["s"], "strided")
    assert (v[:, N:] == -7).all() and (g[:, 3 * N:] == -7).all() and (h[:, 6 * N:] == -7).all()


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [api.STORE_F32, api.STORE_F16, api.STORE_BF16])
def test_sorted_tuning_changes_no_result(orc, storage):
    """A shape tuned for cell-sorted launches is used by them only; results
    stay bit-identical to the random-order launch, and the random-order
    choice is untouched."""
    G, T, _ = build_pair(orc, "s", PERIODIC_UNIT, [(P, P)] * 3, 40, seed=131, storage=storage)
    pos = synth.points_uniform(132, 3000, (0, 0, 0), (1, 1, 1))
    pt = torch_pos(pos)
    base = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0)]
    tile0, mode0 = G.get_tile(), G.get_load_mode()
    G.autotune(3000, sorted=True)
    assert G.get_tile() == tile0 and G.get_load_mode() == mode0
    assert G.launch_shape() == tuple(tile0) + (mode0,)
    assert all(x > 0 for x in G.launch_shape(sorted=True)[:3])
    for sort in (True, False):
        got = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0, sort=sort)]
        for a, b in zip(got, base):
            assert np.array_equal(a, b), sort
    G.autotune(3000)
    got = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0, sort=True)]
    for a, b in zip(got, base):
        assert np.array_equal(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,storage", [("d", api.STORE_NATIVE), ("s", api.STORE_NATIVE), ("s", api.STORE_F16)])
def test_planewave_interpolation_converges_on_gpu(kind, storage):
    """The GPU path against the analytic value, gradient and Hessian of a
    periodic plane-wave sum (the reference's analytic known-answer pattern,
    src/test_bspline_d.c:40-188): FP64 and FP32 tables converge at the cubic
    spline's rates (h^4, h^3, h^2); the F16 table stays within 1e-3 relative
    of the analytic value on the 48^3 grid, where its per-spline rounding,
    not the interpolation, sets the error."""
    import torch
    from helpers import CONVERGENCE_RATIOS, planewave_analytic, rms_rel
    S = 16
    pos = synth.points_uniform(93, 4000)
    err = {}
    for M in (24, 48):
        data, k, amp = synth.grid_data_planewaves(92, (M, M, M), S, waves=8, kmax=2, noise=0.0,
                                                  dtype=np.float64 if kind == "d" else np.float32)
        G = api.MultiUBspline3D(kind, [(0.0, 1.0, M)] * 3, [(P, P)] * 3, S, storage=storage)
        G.set_device(0, torch.from_numpy(data).cuda())
        G.flush()
        v, g, h = (x.cpu().numpy() for x in G.eval(torch_pos(pos), rule=0, layout=1))
        va, ga, ha = planewave_analytic(k, amp, pos)
        err[M] = (rms_rel(v, va), rms_rel(g, ga), rms_rel(h.reshape(ha.shape), ha))
    if storage == api.STORE_F16:
        assert err[48][0] < 1e-3 and err[48][1] < 1e-3 and err[48][2] < 5e-3, err
        return
    for q, (lo, hi) in enumerate(CONVERGENCE_RATIOS):
        assert lo <= err[24][q] / err[48][q] <= hi, (q, err)
    assert err[48][0] < 3e-5 and err[48][1] < 3e-4 and err[48][2] < 5e-3, err


# The reference's own tolerance ladder (src/test_multi.c: absolute
# differences, value / gradient / Hessian; 1e-6 / 1e-4 / 1e-3 in single
# precision, :345, :364, :418; 1e-12 / 1e-10 / 1e-10 in double, :768, :793, :822).
LADDER = {"s": (1e-6, 1e-4, 1e-3), "c": (1e-6, 1e-4, 1e-3), "d": (1e-12, 1e-10, 1e-10), "z": (1e-12, 1e-10, 1e-10)}


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["s_periodic", "s_mixed", "d_periodic", "d_mixed", "c_periodic", "c_mixed",
                                  "z_periodic", "z_mixed"])
def test_gpu_matches_reference_outputs_within_its_ladder(name):
    """The library, fed through the reference's create/set entries, against
    the outputs the compiled reference itself produced for the same data and
    points (tests/golden, made by tests/golden/make_golden.py), within the
    absolute tolerances the reference's own multi-spline test uses: the
    CPU-shaped single-point entry and the batched entry (CPU layout)."""
    import os
    import torch
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name + ".npz"))
    kind = str(z["kind"])
    grids = [tuple(g[:2]) + (int(g[2]),) for g in z["grids"]]
    bcs = [tuple([int(b[0]), int(b[1])] + list(b[2:])) for b in z["bcs"]]
    N = int(z["num_splines"])
    G = api.MultiUBspline3D(kind, grids, bcs, N)
    for i in range(N):
        G.set(i, z["data"][i])
    G.flush()
    tv, tg, th = LADDER[kind]
    pos = z["pos"]
    ref = (z["vals"], z["grads"], z["hess"])
    batched = [x.cpu().numpy() for x in G.eval(torch_pos(pos), rule=0, layout=1)]
    for got, want, tol, what in zip(batched, ref, (tv, tg, th), ("value", "gradient", "hessian")):
        d = np.abs(got.reshape(want.shape).astype(np.float64) - want).max()
        assert d <= tol, (name, "batched", what, d)
    for p in range(0, pos.shape[0], 7):
        v, g, h = G.eval_point(*pos[p])
        for got, want, tol, what in zip((v, g, h), (ref[0][p], ref[1][p], ref[2][p]), (tv, tg, th),
                                        ("value", "gradient", "hessian")):
            d = np.abs(np.asarray(got).reshape(want.shape).astype(np.float64) - want).max()
            assert d <= tol, (name, "point", p, what, d)
    v0 = G.eval(torch_pos(pos), vgh=False, rule=0, layout=1)[0].cpu().numpy()
    assert np.abs(v0.reshape(z["value"].shape).astype(np.float64) - z["value"]).max() <= tv
