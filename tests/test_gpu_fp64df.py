"""FP64 tables evaluated in double-float arithmetic (einspline_gb300_set_fp64_mode
1): every 3D entry against the FP64 oracle at the FP64 tolerance (1e-12
relative), and against the IEEE FP64 path of the same table."""
import numpy as np
import pytest

from einspline_gb300 import api, synth

from helpers import TOL, assert_close, build_pair, cpu_to_gpu_layout, rel_err, table_box

P, D1, D2, FL, NA, AP = 0, 1, 2, 3, 4, 5
CASES = {
    "periodic": ([(0.0, 1.0, 14), (0.0, 1.0, 12), (0.0, 1.0, 13)], [(P, P)] * 3),
    "mixed": ([(0.3, 1.9, 9), (-1.0, 1.0, 13), (0.0, 2.5, 8)],
              [(NA, D1, 0.0, 0.0, 0.4, -0.2), (AP, AP), (D2, FL, 0.6, 0.1, 0.0, 0.0)]),
}


def tpos(pos):
    import torch
    return torch.from_numpy(np.ascontiguousarray(pos, np.float64)).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "dz")
@pytest.mark.parametrize("case", list(CASES))
def test_df_flat_and_point_entries(orc, kind, case):
    grids, bcs = CASES[case]
    G, T, _ = build_pair(orc, kind, grids, bcs, 11, seed=501)
    lo, hi = table_box(grids)
    pos = synth.points_uniform(502, 300, lo, hi)
    ieee = [[x.cpu().numpy() for x in G.eval(tpos(pos), rule=r, layout=l)] for r in (0, 1) for l in (0, 1)]
    G.set_fp64_mode(1)
    k = 0
    for r in (0, 1):
        for lay in (0, 1):
            got = [x.cpu().numpy() for x in G.eval(tpos(pos), rule=r, layout=lay)]
            ref = T.eval(pos, vgh=True, sem=r)
            if lay == 0:
                ref = cpu_to_gpu_layout(kind, *ref)
            assert_close(got, ref, TOL[kind], f"df rule {r} layout {lay}")
            for a, b in zip(got, ieee[k]):
                assert rel_err(a, b) <= TOL[kind]
            k += 1
    v = G.eval(tpos(pos), vgh=False, rule=0)[0].cpu().numpy()
    assert rel_err(v, T.eval(pos, vgh=False)[0]) <= TOL[kind]
    # the single-point CPU entry takes the same path
    for p in pos[:3]:
        got = G.eval_point(*p)
        ref = [x[0] for x in T.eval(p[None], vgh=True)]
        assert_close(got, ref, TOL[kind], "df point")


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "dz")
def test_df_cuda_handle_and_refresh(orc, kind):
    """The *_cuda handle's own table in double-float mode; a table re-set
    after the mode is on evaluates its new data (the copy is rebuilt)."""
    import torch
    grids, bcs = CASES["periodic"]
    G, T, data = build_pair(orc, kind, grids, bcs, 6, seed=511)
    C = G.to_cuda()
    C.set_fp64_mode(1)
    pos = synth.points_uniform(512, 200)
    v, g, h = (x.cpu().numpy() for x in C.eval_multi(tpos(pos), vgh=True))
    rv, rg, rh = cpu_to_gpu_layout(kind, *T.eval(pos, vgh=True, sem=1))
    assert_close((v.reshape(rv.shape), g.reshape(rg.shape), h.reshape(rh.shape)), (rv, rg, rh), TOL[kind], "cuda df")
    G.set_fp64_mode(1)
    new = synth.grid_data_uniform(513, T.M, 1, np.float64, complex_=kind == "z")[0]
    G.set(3, new)
    T.set_spline(3, new)
    got = [x.cpu().numpy() for x in G.eval(tpos(pos), rule=0, layout=1)]
    assert_close(got, T.eval(pos, vgh=True), TOL[kind], "after re-set")
    C.destroy()


@pytest.mark.gpu
def test_df_mode_errors(orc):
    G, _, _ = build_pair(orc, "s", *CASES["periodic"], 4, seed=521)
    with pytest.raises(api.EinsplineError):
        G.set_fp64_mode(1)                     # not an FP64 table
    G.set_fp64_mode(0)                         # a no-op on float tables
    Gd, _, _ = build_pair(orc, "d", *CASES["periodic"], 4, seed=522)
    with pytest.raises(api.EinsplineError):
        Gd.set_fp64_mode(2)


@pytest.mark.gpu
def test_df_planewaves_48cube_512(orc):
    """The 48^3 x 512 FP64 plane-wave workload (128 walkers x 256 points):
    double-float results against the IEEE FP64 path at full size, and
    against the oracle on sampled columns."""
    import torch
    M, N = (48, 48, 48), 512
    data, _, _ = synth.grid_data_planewaves(77, M, N)
    grids = [(0.0, 1.0, 48)] * 3
    G = api.MultiUBspline3D("d", grids, [(P, P)] * 3, N)
    G.set_device(0, torch.from_numpy(data).cuda())
    G.flush()
    pos = tpos(synth.points_uniform(78, 128 * 256))
    ieee = [x.cpu().numpy() for x in G.eval(pos, rule=0, layout=0)]
    G.set_fp64_mode(1)
    got = [x.cpu().numpy() for x in G.eval(pos, rule=0, layout=0)]
    for a, b in zip(got, ieee):
        assert rel_err(a, b) <= TOL["d"]
    cols = [0, 1, 200, 511]
    T = orc.Table("d", grids, [(P, P)] * 3, len(cols))
    for j, c in enumerate(cols):
        T.set_spline(j, data[c])
    sub = np.arange(0, 128 * 256, 64)
    ref = cpu_to_gpu_layout("d", *T.eval(pos.cpu().numpy()[sub], sem=0))
    assert_close((got[0][sub][:, cols], got[1][sub][:, cols], got[2][sub][:, cols]), ref, TOL["d"], "48^3 df")


@pytest.mark.gpu
def test_df_server(orc):
    """A request server on a double-float table returns FP64-tolerance
    results; the mode cannot change under a running server."""
    grids, bcs = CASES["mixed"]
    G, T, _ = build_pair(orc, "d", grids, bcs, 9, seed=531)
    G.set_fp64_mode(1)
    S = api.Server(G, vgh=True, pos_f64=True, rule=0)
    lo, hi = table_box(grids)
    reqs = [synth.points_uniform(532 + i, 40 + 17 * i, lo, hi) for i in range(5)]
    ids = [S.submit(p) for p in reqs]
    for rid, p in zip(ids, reqs):
        S.wait(rid)
        v, g, h = S.result(rid, p.shape[0])
        rv, rg, rh = cpu_to_gpu_layout("d", *T.eval(p, vgh=True, sem=0))
        assert_close((v, g.reshape(rg.shape), h.reshape(rh.shape)), (rv, rg, rh), TOL["d"], "server df")
        S.release(rid)
    with pytest.raises(api.EinsplineError):
        G.set_fp64_mode(0)
    S.close()
    G.set_fp64_mode(0)
