"""Load mode 4: the stencil slices of each point's x-planes arrive in shared
memory by tiled tensor-map (TMA) copies.  Only the data movement differs
from the other modes, so results are bit-identical to them for every table
type, tile shape (one box or several per stage, partial last tiles),
boundary condition, output form and entry point."""
import numpy as np
import pytest

from einspline_gb300 import api, synth

from helpers import TOL, assert_close, build_pair, table_box

P, D1, D2, FL, NA, AP = 0, 1, 2, 3, 4, 5
PERIODIC_UNIT = [(0.0, 1.0, 14), (0.0, 1.0, 12), (0.0, 1.0, 13)]
MIXED = ([(0.3, 1.9, 9), (-1.0, 1.0, 13), (0.0, 2.5, 8)],
         [(NA, D1, 0.0, 0.0, 0.4, -0.2), (AP, AP), (D2, FL, 0.6, 0.1, 0.0, 0.0)])
SHAPES = [(32, 1, 1), (32, 1, 3), (64, 1, 8), (128, 1, 5), (256, 1, 16)]


def tpos(pos):
    import torch
    return torch.from_numpy(np.ascontiguousarray(pos, np.float64)).cuda()


def run(G, pt, mode, shape, vgh=True, rule=0, layout=0):
    G.set_load_mode(mode)
    G.set_tile(*shape)
    out = [x.cpu().numpy() for x in G.eval(pt, vgh=vgh, rule=rule, layout=layout) if x is not None]
    G.wait_status()
    return out


def same(a, b, what):
    for x, y in zip(a, b):
        assert np.array_equal(x, y), what


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [api.STORE_F32, api.STORE_F16, api.STORE_BF16, api.STORE_I16])
@pytest.mark.parametrize("kind", "sc")
@pytest.mark.parametrize("bcase", ["periodic", "mixed"])
def test_tma_bit_identical_to_other_modes(orc, storage, kind, bcase):
    grids, bcs = (PERIODIC_UNIT, [(P, P)] * 3) if bcase == "periodic" else MIXED
    # 45 splines: no tile width divides the columns, so last tiles are partial
    G, T, _ = build_pair(orc, kind, grids, bcs, 45, seed=601, storage=storage)
    lo, hi = table_box(grids)
    pos = synth.points_uniform(602, 700, lo, hi)
    pt = tpos(pos)
    wide = 3 if storage != api.STORE_F32 else 2
    for vgh in (True, False):
        base = run(G, pt, 0, (32, 1, 1), vgh=vgh)
        ref = run(G, pt, wide, (32, 1, 8), vgh=vgh)
        same(ref, base, ("pipeline", vgh))
        for shape in SHAPES:
            same(run(G, pt, 4, shape, vgh=vgh), base, ("tma", vgh, shape))
    for rule in (0, 1):
        for layout in (0, 1):
            a = run(G, pt, 0, (32, 1, 1), rule=rule, layout=layout)
            b = run(G, pt, 4, (64, 1, 8), rule=rule, layout=layout)
            same(b, a, ("rule/layout", rule, layout))
    if storage == api.STORE_F32:
        got = run(G, pt, 4, (32, 1, 8))
        from test_gpu_eval import cpu_to_gpu_layout
        ref = cpu_to_gpu_layout(kind, *T.eval(pos, vgh=True, sem=0))
        assert_close(got, ref, TOL[kind], "tma vs oracle")
    G.set_load_mode(-1)
    G.set_tile(0, 0, 0)


@pytest.mark.gpu
def test_tma_many_boxes_per_stage(orc):
    """1024 F16 splines at 256 threads a block: four 256-column boxes per
    stage; 1000 FP32 splines: four boxes and a partial last tile."""
    for storage, N in ((api.STORE_F16, 1024), (api.STORE_F32, 1000)):
        grids = [(0.0, 1.0, 10)] * 3
        G, T, _ = build_pair(orc, "s", grids, [(P, P)] * 3, N, seed=611, storage=storage)
        pt = tpos(synth.points_uniform(612, 300))
        base = run(G, pt, 0, (256, 1, 2))
        for shape in ((256, 1, 4), (128, 1, 8), (32, 1, 2)):
            same(run(G, pt, 4, shape), base, (storage, shape))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "dz")
def test_tma_double_float(orc, kind):
    """FP64 tables in double-float mode read the (hi, lo) shadow through the
    same tensor-map path; IEEE FP64 ignores mode 4 (direct loads)."""
    grids, bcs = MIXED
    G, T, _ = build_pair(orc, kind, grids, bcs, 21, seed=621)
    lo, hi = table_box(grids)
    pt = tpos(synth.points_uniform(622, 400, lo, hi))
    ieee = run(G, pt, 0, (32, 1, 1))
    same(run(G, pt, 4, (64, 1, 8)), ieee, "IEEE FP64 in mode 4")
    G.set_fp64_mode(1)
    base = run(G, pt, 2, (128, 1, 8))
    for shape in SHAPES:
        same(run(G, pt, 4, shape), base, ("df tma", shape))
    G.set_fp64_mode(0)


@pytest.mark.gpu
def test_tma_reference_entries_and_server(orc):
    """The reference-shaped *_cuda entries (vgh, value, vgl with sign) and
    the request server take their table's load mode."""
    import torch
    from einspline_gb300 import _lib as L
    grids = [(0.0, 1.0, 12)] * 3
    G, T, _ = build_pair(orc, "s", grids, [(P, P)] * 3, 40, seed=631, storage=api.STORE_F16)
    pos = synth.points_uniform(632, 257)
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

    assert lib.einspline_gb300_set_load_mode(C.table, 0) == 0
    base = outs()
    for tile in ((32, 1, 4), (128, 1, 8)):
        assert lib.einspline_gb300_set_load_mode(C.table, 4) == 0
        assert lib.einspline_gb300_set_tile(C.table, *tile) == 0
        same(outs(), base, ("cuda entries", tile))
    assert lib.einspline_gb300_wait_status(C.table) == 0
    C.destroy()
    G.set_load_mode(4)
    G.set_tile(64, 1, 8)
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
    G.wait_status()


@pytest.mark.gpu
def test_tma_mode_arguments():
    G = api.MultiUBspline3D("s", [(0.0, 1.0, 8)] * 3, [(P, P)] * 3, 4)
    G.set_load_mode(4)
    assert G.get_load_mode() == 4
    with pytest.raises(api.EinsplineError):
        G.set_load_mode(6)
    G.wait_status()


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [api.STORE_F32, api.STORE_F16])
def test_tma_bounded_wait_runs_out_and_reports(storage):
    """A wait that runs out, made without a fault: through the test hook the
    first block of one launch issues no copy for its stage 1, so that stage's
    barrier never completes.  With the wait limit shortened to 2 ms the
    launch must end by itself, report ETIMEOUT through
    einspline_gb300_wait_status (once: the status is cleared by reading it),
    leave the context usable, and the next launch on the same table must be
    clean and bit-identical to the copy-pipeline results."""
    import torch
    from einspline_gb300 import _lib as L
    lib = L.load()
    G = api.MultiUBspline3D("s", [(0.0, 1.0, 16)] * 3, [(P, P)] * 3, 256, storage=storage)
    data = synth.grid_data_uniform(641, (16, 16, 16), 256, np.float32)
    for i in range(256):
        G.set(i, data[i])
    G.flush()
    pt = tpos(synth.points_uniform(642, 3000))
    base = run(G, pt, 2, (64, 1, 8))
    G.set_load_mode(4)
    G.set_tile(64, 1, 8)
    assert lib.einspline_gb300_test_wait_timeout(G.table, 1, 0.002) == 0
    G.eval(pt, rule=0, layout=0)
    torch.cuda.synchronize()
    assert lib.einspline_gb300_wait_status(G.table) == 6  # EINSPLINE_GB300_ETIMEOUT
    assert b"bounded wait" in lib.einspline_gb300_last_error_message()
    lib.einspline_gb300_clear_error()
    assert lib.einspline_gb300_wait_status(G.table) == 0
    # the hook applied to one launch only: the next one completes, bit-identical
    again = run(G, pt, 4, (64, 1, 8))
    same(again, base, "after the timed-out launch")
    assert lib.einspline_gb300_wait_status(G.table) == 0
    # a cancelled hook leaves the next launch alone
    assert lib.einspline_gb300_test_wait_timeout(G.table, 1, 0.002) == 0
    assert lib.einspline_gb300_test_wait_timeout(G.table, -1, 0.0) == 0
    same(run(G, pt, 4, (64, 1, 8)), base, "cancelled hook")
    with pytest.raises(api.EinsplineError):
        lib.einspline_gb300_test_wait_timeout(G.table, 1, 5.0)
        L.check()
