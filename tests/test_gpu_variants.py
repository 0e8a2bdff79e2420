"""The other epilogues of the same gather: the reference GPU entries' sign
and vgl (lattice-transformed gradient and laplacian) forms, and the CPU
entries' vg, vgl and vghgh (third derivatives) forms, against the oracle
on the same table."""
import numpy as np
import pytest

from einspline_gb300 import api, synth

from helpers import TOL, assert_close, build_pair, rel_err, table_box

P, D1, NA, AP = 0, 1, 4, 5
PERIODIC_UNIT = [(0.0, 1.0, 12), (0.0, 1.0, 13), (0.0, 1.0, 11)]
MIXED = ([(0.3, 1.9, 9), (-1.0, 1.0, 13), (0.0, 2.5, 8)], [(NA, D1, 0.0, 0.0, 0.4, -0.2), (AP, AP), (P, P)])
LINV = np.array([[1.3, 0.2, -0.1], [0.0, 0.9, 0.4], [0.25, -0.3, 1.1]])


def vgl_reference(kind, v, g, h, G):
    """Oracle vgh (CPU layout) -> reference GPU vgl rows (src/multi_bspline_cuda_s_impl.h:706-733)."""
    GG = G.T @ G
    if kind in "cz":
        gr = np.einsum("rc,pncq->pnrq", G, g)        # [P][N][3][2]
        lap = np.einsum("ab,pnabq->pnq", GG, h)       # [P][N][2]
        rows = np.concatenate([gr, lap[:, :, None, :]], axis=2)  # [P][N][4][2]
        return v.reshape(v.shape[0], -1), np.moveaxis(rows, 2, 1).reshape(v.shape[0], 4, -1)
    gr = np.einsum("rc,pnc->pnr", G, g)
    lap = np.einsum("ab,pnab->pn", GG, h)
    rows = np.concatenate([gr, lap[:, :, None]], axis=2)
    return v, np.moveaxis(rows, 2, 1)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sdcz")
@pytest.mark.parametrize("sign", [False, True])
def test_cuda_vgl(orc, kind, sign):
    import torch
    if sign and kind != "s":
        pytest.skip("the reference has a vgl_sign entry for s only")
    N = 23
    G, T, _ = build_pair(orc, kind, PERIODIC_UNIT, [(P, P)] * 3, N, seed=81)
    c = G.to_cuda()
    pos = synth.points_uniform(82, 150)
    f64 = kind in "dz"
    if not f64:
        pos = pos.astype(np.float32).astype(np.float64)
    dt = torch.float64 if f64 else torch.float32
    pt = torch.from_numpy(pos).to(dt).cuda()
    linv = torch.from_numpy(LINV.reshape(-1)).to(dt).cuda()
    Gm = LINV.astype(np.float32).astype(np.float64) if not f64 else LINV
    sg = np.where(np.arange(150) % 3 == 0, -1.0, 1.0)
    rs = N + 5
    if sign:
        v, gl = c.eval_multi_vgl(pt, linv, row_stride=rs, sign=torch.from_numpy(sg).float().cuda())
    else:
        v, gl = c.eval_multi_vgl(pt, linv, row_stride=rs)
    rv, rgl = vgl_reference(kind, *T.eval(pos, vgh=True, sem=1), Gm)
    if sign:
        rv = rv * sg[:, None]
        rgl = rgl * sg[:, None, None]
    nr = N * (2 if kind in "cz" else 1)
    gl = gl.cpu().numpy()
    assert rel_err(v.cpu().numpy(), rv) <= TOL[kind]
    for r in range(3):
        assert rel_err(gl[:, r, :nr], rgl[:, r]) <= TOL[kind]
    assert rel_err(gl[:, 3, :nr], rgl[:, 3]) <= 2 * TOL[kind]
    assert (gl[:, :, nr:] == -7).all()  # row padding beyond N untouched


@pytest.mark.gpu
def test_cuda_sign():
    import torch
    from einspline_gb300 import api
    grids = PERIODIC_UNIT
    G = api.MultiUBspline3D("s", grids, [(P, P)] * 3, 40)
    data = synth.grid_data_uniform(83, G.M, 40, np.float32)
    for i in range(40):
        G.set(i, data[i])
    c = G.to_cuda()
    pos = torch.from_numpy(synth.points_uniform(84, 77).astype(np.float32)).cuda()
    sg = torch.from_numpy(synth.uniform(85, 77, -2.0, 2.0).astype(np.float32)).cuda()
    plain = c.eval_multi(pos, vgh=False)[0]
    signed = c.eval_multi_sign(pos, sg)
    assert np.array_equal(signed.cpu().numpy(), (plain * sg[:, None]).cpu().numpy())


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sdcz")
def test_cpu_vg_vgl(orc, kind):
    grids, bcs = MIXED
    G, T, _ = build_pair(orc, kind, grids, bcs, 9, seed=86)
    lo, hi = table_box(grids)
    for p in synth.points_uniform(87, 6, lo, hi):
        rv, rg, rh = (x[0] for x in T.eval(p[None], vgh=True))
        v, g = G.eval_point_vg(*p)
        assert_close((v, g), (rv, rg), TOL[kind], "vg")
        v2, g2, lap = G.eval_point_vgl(*p)
        assert np.array_equal(v2, v) and np.array_equal(g2, g)
        rl = rh[:, 0, 0] + rh[:, 1, 1] + rh[:, 2, 2]
        assert rel_err(lap, rl) <= 4 * TOL[kind]


def _sym_ok(gh):
    """gh [N][3][3][3] (complex: trailing re/im axis) is symmetric in its
    three derivative indices."""
    for perm in [(0, 2, 1, 3), (0, 1, 3, 2), (0, 3, 2, 1)]:
        if not np.array_equal(gh, np.transpose(gh, perm + tuple(range(4, gh.ndim)))):
            return False
    return True


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sdcz")
def test_cpu_vghgh(orc, kind):
    """eval_multi_UBspline_3d_*_vghgh: value/gradient/Hessian equal the vgh
    entry bit for bit; third derivatives match the oracle (which is pinned to
    the reference's std backend) within the type's tolerance."""
    for grids, bcs in ((PERIODIC_UNIT, [(P, P)] * 3), MIXED):
        G, T, _ = build_pair(orc, kind, grids, bcs, 9, seed=88)
        lo, hi = table_box(grids)
        for p in synth.points_uniform(89, 5, lo, hi):
            v, g, h, gh = G.eval_point_vghgh(*p)
            v0, g0, h0 = G.eval_point(*p, vgh=True)
            assert np.array_equal(v, v0) and np.array_equal(g, g0) and np.array_equal(h, h0)
            rv, rg, rh, rgh = (x[0] for x in T.eval_vghgh(p[None]))
            assert_close((v, g, h), (rv, rg, rh), TOL[kind], "vghgh")
            e = rel_err(gh, rgh)
            assert e <= TOL[kind], f"third derivatives: rel err {e:.3e}"
            assert _sym_ok(gh)


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [api.STORE_F16, api.STORE_BF16, api.STORE_I16])
def test_cpu_vghgh_16bit(orc, storage):
    """16-bit tables: the same entry against the oracle on the dequantized table."""
    grids, bcs = MIXED
    G, T, _ = build_pair(orc, "s", grids, bcs, 12, seed=90, storage=storage)
    tab = np.ascontiguousarray(G.table_values().astype(np.float32))
    lo, hi = table_box(grids)
    for p in synth.points_uniform(91, 4, lo, hi):
        got = G.eval_point_vghgh(*p)
        ref = [x[0] for x in T.eval_vghgh(p[None], coefs=tab)]
        for a, b in zip(got, ref):
            assert rel_err(a, b) <= TOL["s"]
