"""Load mode 5: F16 and BF16 tables reduced on the tensor cores (tcgen05.mma
with the stencil as the MN-major operand and the point's weights, split into
f16 high and low parts or bf16 high, middle and low parts, as the other).
The products are exact and the sums FP32, so the results agree with the FMA
kernels to FP32 rounding (held to
the FP32 parity tolerance, max |diff| / max |ref| per quantity), for every
boundary condition, output form, partial last tile, point order and entry
point; tables it does not serve fall back to their copy pipeline, bit for
bit."""
import ctypes as C

import numpy as np
import pytest

from einspline_gb300 import _lib as L
from einspline_gb300 import api, synth

from helpers import TOL, assert_close, build_pair, table_box

P, D1, D2, FL, NA, AP = 0, 1, 2, 3, 4, 5
PERIODIC_UNIT = [(0.0, 1.0, 14), (0.0, 1.0, 12), (0.0, 1.0, 13)]
MIXED = ([(0.3, 1.9, 9), (-1.0, 1.0, 13), (0.0, 2.5, 8)],
         [(NA, D1, 0.0, 0.0, 0.4, -0.2), (AP, AP), (D2, FL, 0.6, 0.1, 0.0, 0.0)])


def tpos(pos):
    import torch
    return torch.from_numpy(np.ascontiguousarray(pos, np.float64)).cuda()


def run(G, pt, mode, shape, vgh=True, rule=0, layout=0, sort=False):
    G.set_load_mode(mode)
    G.set_tile(*shape)
    out = [x.cpu().numpy() for x in G.eval(pt, vgh=vgh, rule=rule, layout=layout, sort=sort) if x is not None]
    G.wait_status()
    return out


def same(a, b, what):
    for x, y in zip(a, b):
        assert np.array_equal(x, y), what


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [api.STORE_F16, api.STORE_BF16])
@pytest.mark.parametrize("kind", "sc")
@pytest.mark.parametrize("bcase", ["periodic", "mixed"])
@pytest.mark.parametrize("nspl", [45, 300])
def test_tc_matches_fma_kernels(orc, kind, bcase, nspl, storage):
    grids, bcs = (PERIODIC_UNIT, [(P, P)] * 3) if bcase == "periodic" else MIXED
    # 45 splines: one partial tile; 300 (600 complex columns): several, the last partial
    G, T, _ = build_pair(orc, kind, grids, bcs, nspl, seed=801, storage=storage)
    lo, hi = table_box(grids)
    pt = tpos(synth.points_uniform(802, 700, lo, hi))
    for vgh in (True, False):
        ref = run(G, pt, 3, (32, 1, 8), vgh=vgh)
        for pb in (1, 3, 8, 16):
            assert_close(run(G, pt, 5, (128, 1, pb), vgh=vgh), ref, TOL[kind], f"tc vgh={vgh} pb={pb}")
    for rule in (0, 1):
        for layout in (0, 1):
            ref = run(G, pt, 3, (32, 1, 8), rule=rule, layout=layout)
            got = run(G, pt, 5, (128, 1, 8), rule=rule, layout=layout)
            if kind == "c" and layout == 1:
                same(got, ref, "complex CPU layout falls back to the wide pipeline")
            else:
                assert_close(got, ref, TOL[kind], f"tc rule={rule} layout={layout}")
    G.set_load_mode(-1)
    G.set_tile(0, 0, 0)


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [api.STORE_F16, api.STORE_BF16])
def test_tc_sorted_many_points_and_last_wave(orc, storage):
    """1024 splines (four 256-column blocks), 60,000 points: several
    waves, so the last wave's points go to shorter blocks; random and
    cell-sorted order give the same results (each point's arithmetic does
    not depend on its block), close to the FMA kernels."""
    grids = [(0.0, 1.0, 10)] * 3
    G, T, _ = build_pair(orc, "s", grids, [(P, P)] * 3, 1024, seed=811, storage=storage)
    pt = tpos(synth.points_uniform(812, 60000))
    ref = run(G, pt, 3, (32, 1, 8))
    tc = run(G, pt, 5, (128, 1, 8))
    assert_close(tc, ref, TOL["s"], "tc vs fma")
    same(run(G, pt, 5, (128, 1, 8), sort=True), tc, "sorted")
    same(run(G, pt, 5, (128, 1, 32)), tc, "pb 32")
    same(run(G, pt, 5, (128, 1, 2)), tc, "pb 2")


@pytest.mark.gpu
def test_tc_reference_entries_and_server(orc):
    """The reference-shaped *_cuda entries (vgh, value, vgl with lattice
    transform and sign) and the request server take the table's mode 5."""
    import torch
    from einspline_gb300 import _lib as L
    grids = [(0.0, 1.0, 12)] * 3
    G, T, _ = build_pair(orc, "s", grids, [(P, P)] * 3, 200, seed=821, storage=api.STORE_F16)
    pos = synth.points_uniform(822, 257)
    pt = torch.from_numpy(pos).float().cuda()
    linv = torch.tensor([1.1, 0.1, 0.0, 0.0, 0.9, 0.2, 0.3, 0.0, 1.0], dtype=torch.float32).cuda()
    sign = torch.from_numpy(np.where(np.arange(257) % 3 == 0, -1.0, 1.0)).float().cuda()
    C = G.to_cuda()
    lib = L.load()

    def outs():
        r = [x.cpu().numpy() for x in C.eval_multi(pt)]
        r += [C.eval_multi(pt, vgh=False)[0].cpu().numpy()]
        r += [x.cpu().numpy() for x in C.eval_multi_vgl(pt, linv, sign=sign)]
        return r

    assert lib.einspline_gb300_set_load_mode(C.table, 3) == 0
    base = outs()
    assert lib.einspline_gb300_set_load_mode(C.table, 5) == 0
    got = outs()
    for i, (x, y) in enumerate(zip(got, base)):
        assert_close([x], [y], TOL["s"], f"cuda entry output {i}")
    assert lib.einspline_gb300_wait_status(C.table) == 0
    C.destroy()
    G.set_load_mode(5)
    G.set_tile(128, 1, 8)
    direct = [x.cpu().numpy() for x in G.eval(tpos(pos), rule=0, layout=0)]
    S = api.Server(G, max_inflight=3, max_batch_points=1024)
    ids = [(S.submit(pos[i:i + 50]), i) for i in range(0, 250, 50)]
    for r, i in ids:
        S.wait(r)
        got = S.result(r, 50)
        assert np.array_equal(got[0], direct[0][i:i + 50])
        assert np.array_equal(got[1], direct[1][i:i + 50].reshape(50, -1))
        S.release(r)
    S.close()
    # single-point CPU-shaped entry with mode 5: one point, one launch
    one = pos[:1]
    v, g, h = G.eval_point(*one[0])
    ref = [x[0] for x in run(G, tpos(one), 3, (32, 1, 8), layout=1)]
    assert_close([v, g, h], ref, TOL["s"], "single point")
    G.wait_status()


@pytest.mark.gpu
def test_tc_other_tables_fall_back(orc):
    """FP32, I16 and FP64 tables take their usual kernels when mode 5 is
    asked for: results bit-identical to those kernels."""
    grids = [(0.0, 1.0, 9)] * 3
    for kind, storage, fb in (("s", api.STORE_F32, 2), ("s", api.STORE_I16, 3), ("d", api.STORE_NATIVE, 0)):
        G, T, _ = build_pair(orc, kind, grids, [(P, P)] * 3, 33, seed=831, storage=storage)
        pt = tpos(synth.points_uniform(832, 500))
        same(run(G, pt, 5, (128, 1, 8)), run(G, pt, fb, (128, 1, 8)), (kind, storage))


@pytest.mark.gpu
def test_tc_accuracy_against_fp64_full_size():
    """64^3 x 1024 F16 table against the library's IEEE FP64 table of the
    same data at 2,048 points, all splines: the tensor-core reduction keeps
    the F16 table's accuracy (per-point relative L2 of the values <= 1e-3,
    as for the FMA kernels)."""
    import torch
    g, n = 64, 1024
    grids = [(0.0, 1.0, g)] * 3
    bcs = [(P, P)] * 3
    F = api.MultiUBspline3D("s", grids, bcs, n, storage=api.STORE_F16)
    D = api.MultiUBspline3D("d", grids, bcs, n, storage=api.STORE_NATIVE)
    buf = torch.empty((128, g, g, g), dtype=torch.float64, device="cuda")
    for f in range(0, n, 128):
        api.fill_uniform(buf, 20261203, -1.0, 1.0, offset=f * g ** 3)
        D.set_device(f, buf)
        F.set_device(f, buf.float())
    F.flush()
    D.flush()
    del buf
    pt = tpos(synth.points_uniform(841, 2048))
    ref = [x.cpu().numpy() for x in D.eval(pt, rule=0, layout=0)]
    F.set_load_mode(5)
    tc = [x.cpu().numpy() for x in F.eval(pt, rule=0, layout=0)]
    F.set_load_mode(3)
    fma = [x.cpu().numpy() for x in F.eval(pt, rule=0, layout=0)]
    for a, b, name in zip(tc, ref, ("value", "gradient", "hessian")):
        d = (a - b).reshape(a.shape[0], -1)
        r = b.reshape(b.shape[0], -1)
        per_point = np.sqrt((d ** 2).sum(1) / (r ** 2).sum(1))
        assert per_point.max() <= 1e-3, (name, per_point.max())
    assert_close(tc, fma, TOL["s"], "tc vs fma at full size")
    F.wait_status()


@pytest.mark.gpu
def test_tc_bounded_wait_runs_out_and_reports():
    """As for the TMA pipeline: the test hook makes the first block issue no
    stencil copy for its point 1 and shortens every wait to 2 ms; the launch
    ends by itself, reports ETIMEOUT once, frees its tensor memory, and the
    next launch on the table is clean and the same as before."""
    import torch
    from einspline_gb300 import _lib as L
    lib = L.load()
    G = api.MultiUBspline3D("s", [(0.0, 1.0, 16)] * 3, [(P, P)] * 3, 256, storage=api.STORE_F16)
    data = synth.grid_data_uniform(851, (16, 16, 16), 256, np.float32)
    for i in range(256):
        G.set(i, data[i])
    G.flush()
    pt = tpos(synth.points_uniform(852, 3000))
    base = run(G, pt, 5, (128, 1, 8))
    assert lib.einspline_gb300_test_wait_timeout(G.table, 1, 0.002) == 0
    G.eval(pt, rule=0, layout=0)
    torch.cuda.synchronize()
    assert lib.einspline_gb300_wait_status(G.table) == 6  # EINSPLINE_GB300_ETIMEOUT
    lib.einspline_gb300_clear_error()
    assert lib.einspline_gb300_wait_status(G.table) == 0
    same(run(G, pt, 5, (128, 1, 8)), base, "after the timed-out launch")
    assert lib.einspline_gb300_wait_status(G.table) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [api.STORE_F16, api.STORE_BF16])
@pytest.mark.parametrize("nspl", [1, 7, 33, 129])
def test_tc_tiny_and_odd_spline_counts(orc, storage, nspl):
    """Spline counts far below and just past one 128-column tile: the TMA
    boxes past the padded row read zeros and count their bytes, only real
    columns are written (the output rows' padding stays untouched), and the
    results agree with the FMA kernel."""
    import torch
    grids = [(0.0, 1.0, 9), (0.0, 1.0, 10), (0.0, 1.0, 8)]
    G, T, _ = build_pair(orc, "s", grids, [(P, P)] * 3, nspl, seed=871, storage=storage)
    pt = tpos(synth.points_uniform(872, 333))
    ref = run(G, pt, 3, (32, 1, 8))
    G.set_load_mode(5)
    G.set_tile(128, 1, 8)
    pad = 5
    out = (torch.full((333, nspl + pad), -7.0, device="cuda"), torch.full((333, 3 * nspl + pad), -7.0, device="cuda"),
           torch.full((333, 6 * nspl + pad), -7.0, device="cuda"))
    o = L.EvalOpts(1, 1, 0, 0, 0, nspl + pad, 3 * nspl + pad, 6 * nspl + pad)
    lib = L.load()
    rc = lib.einspline_gb300_eval_3d(G.table, C.byref(o), 333, C.c_void_p(pt.data_ptr()), C.c_void_p(out[0].data_ptr()),
                                     C.c_void_p(out[1].data_ptr()), C.c_void_p(out[2].data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    G.wait_status()
    got = [out[0][:, :nspl].cpu().numpy(), out[1][:, :3 * nspl].cpu().numpy().reshape(333, nspl, 3),
           out[2][:, :6 * nspl].cpu().numpy().reshape(333, nspl, 6)]
    assert_close(got, ref, TOL["s"], f"tc nspl={nspl}")
    for x, n in zip(out, (nspl, 3 * nspl, 6 * nspl)):
        assert bool((x[:, n:] == -7.0).all())
    G.set_load_mode(-1)
    G.set_tile(0, 0, 0)
