"""The workloads at their full sizes, checked through properties that do not
need an oracle of the whole table.  Against FP64 the FP32 results carry the
reference's single-precision position rule (u = (x - start) * delta_inv
rounded to float, an offset error of up to ulp(M)/2 in cell units), so their
tolerance is 2e-5 of the largest magnitude; FP64 results are held to 1e-12.
  * interpolation: at every grid node the spline equals its data;
  * sampled columns: splines are independent, so the oracle solves a few
    columns in FP64 and every GPU result for those columns must match;
  * order independence: sorted, unsorted and sub-batched evaluations agree
    bit for bit;
and the FP16/BF16 tables' error against FP64."""
import numpy as np
import pytest

from einspline_gb300 import api, synth

from helpers import TOL, assert_close, cpu_to_gpu_layout, rel_err

P = 0
F32_VS_F64 = 2e-5


def device_table(kind, M, N, seed, storage=api.STORE_NATIVE, box=(0.0, 1.0)):
    import torch
    grids = [(box[0], box[1], m) for m in M]
    G = api.MultiUBspline3D(kind, grids, [(P, P)] * 3, N, storage=storage)
    per = int(np.prod(M)) * (2 if kind in "cz" else 1)
    dt = torch.float32 if kind in "sc" else torch.float64
    chunk = max(1, min(N, (256 << 20) // (per * 8)))
    shape = tuple(M) + ((2,) if kind in "cz" else ())
    buf = torch.empty((chunk,) + shape, dtype=dt, device="cuda")
    for f in range(0, N, chunk):
        n = min(chunk, N - f)
        api.fill_uniform(buf[:n], seed, -1.0, 1.0, offset=f * per)
        G.set_device(f, buf[:n])
    G.flush()
    return G, grids


def column_data(kind, M, seed, col):
    per = int(np.prod(M)) * (2 if kind in "cz" else 1)
    d = synth.uniform(seed, per, -1.0, 1.0, offset=col * per)
    if kind in "sc":
        d = d.astype(np.float32).astype(np.float64)
    return d.reshape(tuple(M) + ((2,) if kind in "cz" else ()))


def sampled_oracle(orc, kind, grids, M, seed, cols):
    T = orc.Table("d" if kind in "sd" else "z", grids, [(P, P)] * 3, len(cols))
    for j, c in enumerate(cols):
        T.set_spline(j, column_data(kind, M, seed, c))
    return T


def check_nodes(G, kind, M, N, seed, npts, tol):
    """Spline value at grid nodes == data, for all splines."""
    import torch
    rng = np.random.default_rng(seed)
    nodes = rng.integers(0, M, size=(npts, 3))
    pos = nodes / np.asarray(M, np.float64)
    v = G.eval(torch.from_numpy(pos).cuda(), vgh=False, rule=0, layout=1)[0].cpu().numpy()
    nc = 2 if kind in "cz" else 1
    per = int(np.prod(M)) * nc
    flat = (nodes[:, 0] * M[1] + nodes[:, 1]) * M[2] + nodes[:, 2]
    idx = (np.arange(N)[None, :, None] * per + flat[:, None, None] * nc + np.arange(nc)[None, None, :])
    data = synth.uniform_at(seed, idx, -1.0, 1.0)
    if kind in "sc":
        data = data.astype(np.float32).astype(np.float64)
    data = data.reshape(v.shape)
    e = rel_err(v, data)
    assert e <= tol, f"interpolation at nodes: rel err {e:.3e}"


@pytest.mark.gpu
def test_fp64_planewaves_48cube_512(orc):
    """multi_UBspline_3d_d, periodic 48^3, 512 splines of 8 plane waves plus
    noise; 128 walkers x 256 points vgh in one batched launch."""
    import torch
    M, N = (48, 48, 48), 512
    data, _, _ = synth.grid_data_planewaves(77, M, N)
    grids = [(0.0, 1.0, 48)] * 3
    G = api.MultiUBspline3D("d", grids, [(P, P)] * 3, N)
    G.set_device(0, torch.from_numpy(data).cuda())
    G.flush()
    pos = synth.points_uniform(78, 128 * 256)
    v, g, h = (x.cpu().numpy() for x in G.eval(torch.from_numpy(pos).cuda(), rule=0, layout=0))
    cols = [0, 1, 200, 511]
    T = orc.Table("d", grids, [(P, P)] * 3, len(cols))
    for j, c in enumerate(cols):
        T.set_spline(j, data[c])
    sub = np.arange(0, pos.shape[0], 64)
    ref = cpu_to_gpu_layout("d", *T.eval(pos[sub], sem=0))
    assert_close((v[sub][:, cols], g[sub][:, cols], h[sub][:, cols]), ref, TOL["d"], "FP64 48^3 sampled")
    # interpolation at nodes, all 512 splines
    rng = np.random.default_rng(5)
    nodes = rng.integers(0, 48, size=(64, 3))
    vn = G.eval(torch.from_numpy(nodes / 48.0).cuda(), vgh=False)[0].cpu().numpy()
    dn = data[:, nodes[:, 0], nodes[:, 1], nodes[:, 2]].T
    assert rel_err(vn, dn) <= 1e-12


@pytest.mark.gpu
def test_complex_64cube_256_sorted(orc):
    """multi_UBspline_3d_c, periodic 64^3, 256 complex splines (0.6 GB);
    256 walkers x 128 points vgh; sorted by cell vs random order."""
    import torch
    M, N, seed = (64, 64, 64), 256, 303
    G, grids = device_table("c", M, N, seed)
    pos = synth.points_uniform(304, 256 * 128)
    pt = torch.from_numpy(pos).cuda()
    a = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0)]
    b = [x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0, sort=True)]
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    cols = [0, 77, 255]
    T = sampled_oracle(orc, "c", grids, M, seed, cols)
    sub = np.arange(0, pos.shape[0], 128)
    ref = cpu_to_gpu_layout("z", *T.eval(pos[sub], sem=0))
    got = (a[0][sub][:, cols], a[1][sub][:, cols], a[2][sub][:, cols])
    assert_close(got, ref, F32_VS_F64, "complex 64^3 sampled vs FP64")
    check_nodes(G, "c", M, N, seed, 128, F32_VS_F64)


# Value error against FP64 per storage: (max |dv| / max |v|, ||dv|| / ||v||).
# FP16 keeps 11 significant bits of each coefficient; the B-spline
# coefficients of rough data are several times larger than the data, so its
# worst case sits near 1e-3 of the largest value (bounded by 2.44e-4 times the
# largest coefficient, up to 2e-3 of the largest value) while its relative L2 error
# is 3-4 times smaller.  I16 (uniform 16-bit steps) is ten times tighter.
STORAGE_TOL = {api.STORE_F32: (2e-5, 1e-5), api.STORE_F16: (2e-3, 1e-3), api.STORE_I16: (2e-4, 1e-4),
               api.STORE_BF16: (1.5e-2, 1e-2)}


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [api.STORE_F32, api.STORE_F16, api.STORE_I16, api.STORE_BF16])
def test_serving_table_64cube_1024_errors_vs_fp64(orc, storage):
    """multi_UBspline_3d_s, 64^3, 1024 splines: FP32 and 16-bit tables
    against the FP64 solve and evaluation on sampled columns."""
    import torch
    tol_max, tol_l2 = STORAGE_TOL[storage]
    M, N, seed = (64, 64, 64), 1024, 404
    G, grids = device_table("s", M, N, seed, storage=storage)
    pos = synth.points_uniform(405, 512)
    v, g, h = (x.cpu().numpy() for x in G.eval(torch.from_numpy(pos).cuda(), rule=0, layout=0))
    cols = list(range(0, N, 128))
    T = sampled_oracle(orc, "s", grids, M, seed, cols)
    rv, rg, rh = cpu_to_gpu_layout("d", *T.eval(pos, sem=0))
    for name, a, b in (("value", v[:, cols], rv), ("gradient", g[:, cols], rg), ("hessian", h[:, cols], rh)):
        assert rel_err(a, b) <= tol_max, (name, rel_err(a, b))
        assert rel_l2(a, b) <= tol_l2, (name, rel_l2(a, b))
    check_nodes(G, "s", M, N, seed, 64, max(tol_max, F32_VS_F64))


@pytest.mark.gpu
def test_large_table_128cube_2048_int64_offsets(orc):
    """multi_UBspline_3d_s, 128^3, 2048 splines: 4.6e9 table elements
    (18.4 GB FP32), beyond 32-bit offsets; sampled columns vs FP64."""
    import torch
    M, N, seed = (128, 128, 128), 2048, 505
    G, grids = device_table("s", M, N, seed)
    assert G.info().table_bytes > 2 ** 34
    pos = synth.points_uniform(506, 4096)
    pt = torch.from_numpy(pos).cuda()
    v, g, h = (x.cpu().numpy() for x in G.eval(pt, rule=0, layout=0))
    cols = [0, 1023, 2047]
    T = sampled_oracle(orc, "s", grids, M, seed, cols)
    sub = np.arange(0, 4096, 16)
    ref = cpu_to_gpu_layout("d", *T.eval(pos[sub], sem=0))
    assert_close((v[sub][:, cols], g[sub][:, cols], h[sub][:, cols]), ref, 4 * F32_VS_F64, "128^3 sampled vs FP64")
    # the high corner of the table (offsets past 2^32 elements)
    corner = np.array([[0.999, 0.999, 0.999], [0.995, 0.5, 0.999]])
    vc = G.eval(torch.from_numpy(corner).cuda(), rule=0, layout=0)
    ref_c = cpu_to_gpu_layout("d", *T.eval(corner, sem=0))
    assert_close((vc[0].cpu().numpy()[:, cols], vc[1].cpu().numpy()[:, cols], vc[2].cpu().numpy()[:, cols]),
                 ref_c, 4 * F32_VS_F64, "128^3 corner")
    del G
    torch.cuda.empty_cache()


@pytest.mark.gpu
def test_plain_32cube_128_value_and_vgh(orc):
    """multi_UBspline_3d_s, periodic 32^3, 128 splines, 10,000 points, value
    and vgh, against the FP64 evaluation of the same data."""
    import torch
    M, N, seed = (32, 32, 32), 128, 101
    data = synth.grid_data_uniform(seed, M, N, np.float32)
    grids = [(0.0, 1.0, 32)] * 3
    G = api.MultiUBspline3D("s", grids, [(P, P)] * 3, N)
    for i in range(N):
        G.set(i, data[i])
    T = orc.Table("d", grids, [(P, P)] * 3, N)
    for i in range(N):
        T.set_spline(i, data[i].astype(np.float64))
    pos = synth.points_uniform(102, 10000)
    pt = torch.from_numpy(pos).cuda()
    val = G.eval(pt, vgh=False, rule=0, layout=1)[0].cpu().numpy()
    v, g, h = (x.cpu().numpy() for x in G.eval(pt, rule=0, layout=1))
    rv, rg, rh = T.eval(pos, sem=0)
    assert np.array_equal(val, v)
    assert_close((v, g, h), (rv, rg, rh), F32_VS_F64, "32^3 vs FP64")
