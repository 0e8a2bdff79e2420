"""1D and 2D multi-splines (create/set/eval_multi_UBspline_{1,2}d_* and the
batched 1D GPU entries) against the oracle, which is pinned bit for bit to
the reference's std backend (tests/test_oracle.py)."""
import numpy as np
import pytest

from einspline_gb300 import api, synth

from helpers import TOL, oracle_bcs, rel_err

P, D1, D2, FL, NA, AP = 0, 1, 2, 3, 4, 5
CASES = [
    ([(0.0, 1.0, 11)], [(P, P)]),
    ([(-0.4, 1.2, 9)], [(NA, D1, 0.0, 0.0, 0.6, -0.2)]),
    ([(0.0, 2.0, 8)], [(AP, AP)]),
    ([(0.0, 1.0, 8), (0.0, 1.0, 7)], [(P, P)] * 2),
    ([(0.2, 1.4, 7), (-1.0, 0.5, 9)], [(D2, FL, 0.3, 0.1, 0.0, 0.0), (AP, AP)]),
]
IDS = ["1d_periodic", "1d_mixed", "1d_anti", "2d_periodic", "2d_mixed"]


def build_ld(orc, kind, grids, bcs, N, seed):
    M = tuple(g[2] for g in grids)
    dt = np.float32 if kind in "sc" else np.float64
    data = synth.grid_data_uniform(seed, M, N, dt, complex_=kind in "cz")
    G = api.MultiUBsplineLD(kind, grids, bcs, N)
    T = orc.Table(kind, grids, oracle_bcs(kind, bcs), N)
    for i in range(N):
        G.set(i, data[i])
        T.set_spline(i, data[i].astype(np.float64))
    G.flush()
    return G, T, data


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sdcz")
@pytest.mark.parametrize("case", range(len(CASES)), ids=IDS)
def test_lowdim_table_and_eval(orc, kind, case):
    grids, bcs = CASES[case]
    N = 7
    G, T, _ = build_ld(orc, kind, grids, bcs, N, seed=400 + case)
    # the FP64 solve on the GPU equals the oracle's (and the reference's) bit
    # for bit; s/c tables are that result rounded once
    tab = G.table_values()
    ref = T.coefs64 if kind in "dz" else T.coefs.astype(np.float64)
    assert np.array_equal(tab, ref)
    lo, hi = [g[0] for g in grids], [g[1] for g in grids]
    pos = synth.points_uniform(410 + case, 6, lo, hi)
    for form in range(4):
        want = T.eval_ld(pos, form)
        for p in range(pos.shape[0]):
            y = pos[p, 1] if len(grids) == 2 else 0.0
            got = G.eval_point(pos[p, 0], y, form)
            for a, b in zip(got, want):
                if b is not None:
                    e = rel_err(a, b[p])
                    assert e <= TOL[kind], (form, e)
    # outside the box the edge cell is extrapolated, as in 3D
    v, _, _ = G.eval_point(hi[0] + 0.3 * (hi[0] - lo[0]), lo[-1] - 0.1, 0)
    assert np.all(np.isfinite(v))


@pytest.mark.gpu
@pytest.mark.parametrize("kind,conv", [("s", False), ("c", False), ("d", False), ("z", False), ("d", True),
                                       ("z", True)])
def test_lowdim_cuda_1d(orc, kind, conv):
    """eval_multi_multi_UBspline_1d_*[_vgl]_cuda: the reference GPU cell rule
    and derivatives in cell units (not multiplied by gridInv)."""
    torch = pytest.importorskip("torch")
    grids, bcs = [(0.0, 1.0, 37)], [(P, P)]
    N = 70                                  # not a multiple of the reference's 64-wide blocks
    G, T, _ = build_ld(orc, kind, grids, bcs, N, seed=420)
    C = G.to_cuda(conv=conv)
    f = C.fields
    assert f.num_splines == N and f.dim == 37 and abs(f.gridInv - 37.0) < 1e-5
    ck = C.kind
    pos = synth.points_uniform(421, 300, [0.0], [1.0])[:, 0]
    pt = torch.from_numpy(pos.astype(np.float32 if ck in "sc" else np.float64)).cuda()
    v0, _, _ = C.eval_multi(pt, vgl=False)
    v, g, lap = C.eval_multi(pt, vgl=True)
    torch.cuda.synchronize()
    assert torch.equal(v0, v)
    # oracle in position units; the entries return d/du = delta * d/dx
    delta = 1.0 / 37
    rv, rg, rl = T.eval_ld(pt.cpu().numpy().astype(np.float64), 3)
    tol = TOL["s"] if ck in "sc" else TOL["d"]
    if conv:
        tol = 1e-5                          # table rounded to float from the FP64 solve
    nr = N * (2 if kind in "cz" else 1)
    assert rel_err(v.cpu().numpy(), rv.reshape(-1, nr)) <= tol
    assert rel_err(g.cpu().numpy(), rg.reshape(-1, nr) * delta) <= tol
    assert rel_err(lap.cpu().numpy(), rl.reshape(-1, nr) * delta * delta) <= 4 * tol
    C.destroy()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "dz")
def test_lowdim_set_bc(orc, kind):
    """set_multi_UBspline_1d_{d,z}_BC: one spline with its own boundary values."""
    grids, bcs = [(0.0, 1.5, 10)], [(D1, D2, 0.5, 0.0, -0.25, 0.0)]
    other = (D1, D2, -1.5, 0.75, 2.0, -0.5)
    N = 4
    G, T, data = build_ld(orc, kind, grids, bcs, N, seed=430)
    G.set_bc(2, data[2], other)
    T2 = orc.Table(kind, grids, [other if kind == "z" else other[:3] + (0.0, other[4], 0.0)], N)
    T2.set_spline(2, data[2])
    tab = G.table_values()
    assert np.array_equal(tab[..., 2, :] if kind == "z" else tab[..., 2], T2.coefs64[..., 2, :] if kind == "z"
                          else T2.coefs64[..., 2])
    assert np.array_equal(tab[..., 1, :] if kind == "z" else tab[..., 1],
                          T.coefs64[..., 1, :] if kind == "z" else T.coefs64[..., 1])
    with pytest.raises(api.EinsplineError):
        G.set_bc(0, data[0], (P, P))        # periodicity differs from the table's


@pytest.mark.gpu
def test_lowdim_errors(orc):
    torch = pytest.importorskip("torch")
    G, _, _ = build_ld(orc, "s", [(0.0, 1.0, 9)], [(P, P)], 3, seed=440)
    o = api.L.EvalOpts(1, 0, 0, 0, 0, 0, 0, 0)
    pos = torch.zeros(4, 3, device="cuda")
    out = torch.zeros(4 * 3 * 10, device="cuda")
    import ctypes as C
    api._lib().einspline_gb300_eval_3d(G.table, C.byref(o), 4, C.c_void_p(pos.data_ptr()),
                                       C.c_void_p(out.data_ptr()), C.c_void_p(out.data_ptr()),
                                       C.c_void_p(out.data_ptr()), None)
    with pytest.raises(api.EinsplineError):
        api.check()                          # a 1D table is not a 3D table
    G2, _, _ = build_ld(orc, "s", [(0.0, 1.0, 9), (0.0, 1.0, 8)], [(P, P)] * 2, 3, seed=441)
    with pytest.raises(AssertionError):
        G2.to_cuda()                         # no 2D GPU entries (as in the reference)
