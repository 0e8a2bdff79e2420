"""GPU coefficient solve (set_multi_UBspline_3d_*) against the oracle.

FP64 tables (d, z) must be bit-identical to the oracle's FP64 solve, which
is itself bit-identical to the reference's set_multi_UBspline_3d_d/z.  FP32
tables (s, c) must equal that FP64 solve rounded once to float.  16-bit tables
must be the FP64 solve times a per-spline factor, rounded once.
"""
import os

import numpy as np
import pytest

from einspline_gb300 import api, synth

from helpers import build_pair

P, D1, D2, FL, NA, AP = 0, 1, 2, 3, 4, 5

CASES = [
    ("periodic", [(0.0, 1.0, 12), (0.0, 1.0, 10), (0.0, 1.0, 11)], [(P, P)] * 3),
    ("mixed", [(0.3, 1.9, 9), (-1.0, 1.0, 13), (0.0, 2.5, 8)],
     [(NA, D1, 0.0, 0.0, 0.4, -0.2), (AP, AP), (D2, FL, 0.6, 0.1, 0.0, 0.0)]),
    ("flat_deriv", [(0.0, 1.0, 7), (0.0, 3.0, 9), (-2.0, 0.0, 10)],
     [(FL, FL), (D1, D2, -0.3, 0.2, 0.5, 0.5), (P, P)]),
]


def gpu_table(G):
    t, _ = G.table_host()
    ti = G.info()
    t = t[..., :ti.ncol]
    if G.ncomp == 2:
        t = t.reshape(t.shape[:3] + (G.N, 2))
    return t


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sdcz")
@pytest.mark.parametrize("name,grids,bcs", CASES, ids=[c[0] for c in CASES])
def test_table_matches_oracle(orc, kind, name, grids, bcs):
    N = 13
    G, T, _ = build_pair(orc, kind, grids, bcs, N, seed=101)
    got = gpu_table(G)
    if kind in "dz":
        assert np.array_equal(got, T.coefs64)
    else:
        assert np.array_equal(got, T.coefs64.astype(np.float32))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "dz")
@pytest.mark.parametrize("name,grids,bcs", CASES, ids=[c[0] for c in CASES])
def test_table_bit_identical_across_magnitudes(orc, kind, name, grids, bcs):
    """Data from 2^-1000 to 2^900 in magnitude with exact zeros and negative
    zeros: the device divides by the band divisors through their split
    reciprocals (Markstein's correction) inside an exponent window and by
    the IEEE division outside it; the tables keep the reference's bits,
    signed zeros included."""
    M = tuple(g[2] for g in grids)
    N = 9
    rng = np.random.default_rng(121)
    base = synth.grid_data_uniform(122, M, N, np.float64, complex_=kind == "z")
    data = np.ldexp(base, rng.integers(-1000, 900, size=base.shape))
    flat = data.reshape(-1)
    flat[rng.choice(flat.size, flat.size // 20, replace=False)] = 0.0
    flat[rng.choice(flat.size, flat.size // 20, replace=False)] = -0.0
    G, T, _ = build_pair(orc, kind, grids, bcs, N, data=data)
    got = np.ascontiguousarray(gpu_table(G))
    assert np.array_equal(got.view(np.uint64), np.ascontiguousarray(T.coefs64).view(np.uint64))


@pytest.mark.gpu
def test_padding_and_unset_columns_are_zero(orc):
    grids, bcs = CASES[0][1], CASES[0][2]
    G = api.MultiUBspline3D("s", grids, bcs, 5)
    data = synth.grid_data_uniform(3, G.M, 5, np.float32)
    G.set(1, data[1])
    G.set(3, data[3])
    t, _ = G.table_host()
    assert not t[..., 0].any() and not t[..., 2].any() and not t[..., 4:].any()
    assert t[..., 1].any() and t[..., 3].any()


@pytest.mark.gpu
def test_set_order_resets_and_batches(orc, monkeypatch):
    """Random set order, a spline set twice before the solve (the last data
    wins), and a solve budget small enough to force several batches."""
    grids, bcs = CASES[1][1], CASES[1][2]
    N = 9
    monkeypatch.setenv("EINSPLINE_GB300_SOLVE_BUDGET_MB", "0.1")
    G = api.MultiUBspline3D("d", grids, bcs, N)
    T = orc.Table("d", grids, bcs, N)
    data = synth.grid_data_uniform(5, G.M, N, np.float64)
    junk = synth.grid_data_uniform(6, G.M, 1, np.float64)[0]
    G.set(4, junk)
    for i in [3, 0, 8, 4, 1, 7, 2, 6, 5]:
        G.set(i, data[i])
        T.set_spline(i, data[i])
    assert np.array_equal(gpu_table(G), T.coefs64)
    G.set(2, junk)  # reset after a solve
    T.set_spline(2, junk)
    assert np.array_equal(gpu_table(G), T.coefs64)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sz")
def test_bulk_device_set_equals_host_set(orc, kind):
    import torch
    grids, bcs = CASES[2][1], CASES[2][2]
    N = 6
    G, T, data = build_pair(orc, kind, grids, bcs, N, seed=9)
    H = api.MultiUBspline3D(kind, grids, bcs, N)
    H.set_device(0, torch.from_numpy(np.ascontiguousarray(data)).cuda())
    assert np.array_equal(gpu_table(H), gpu_table(G))


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [api.STORE_F16, api.STORE_BF16, api.STORE_I16])
@pytest.mark.parametrize("kind", "sc")
def test_16bit_tables_are_scaled_fp64_solve(orc, kind, storage):
    """Each stored value is round(c * inv) of the FP64 coefficient c, with the
    per-spline factor inv chosen from the spline's largest |c| (shared by re/im)."""
    grids, bcs = CASES[0][1], CASES[0][2]
    N = 11
    G, T, _ = build_pair(orc, kind, grids, bcs, N, seed=21, storage=storage)
    raw, sc = G.table_host()
    ti = G.info()
    ref = T.coefs64.reshape(T.coefs64.shape[:3] + (-1,))
    m = np.abs(ref).max(axis=(0, 1, 2)).astype(np.float32).astype(np.float64)
    if kind == "c":
        m = np.repeat(np.maximum(m[0::2], m[1::2]), 2)
        assert np.array_equal(sc[0::2], sc[1::2])
    if storage == api.STORE_F16:
        inv = (65504.0 * (1.0 - 2.0 ** -20)) / m
    elif storage == api.STORE_I16:
        inv = 32767.0 / m
    else:
        e = np.frexp(m)[1]
        inv = np.ldexp(1.0, 15 - e)
    assert np.array_equal(sc, (1.0 / inv).astype(np.float32))
    scaled = ref * inv
    got = raw[..., :ti.ncol]
    if storage == api.STORE_F16:
        assert np.array_equal(got, scaled.astype(np.float16))
        assert np.abs(got.astype(np.float64)).max() <= 65504
    elif storage == api.STORE_I16:
        q = np.clip(np.rint(scaled), -32767, 32767).astype(np.int64) + 32768
        assert np.array_equal(got.astype(np.int64), q)
    else:
        import torch
        expect = torch.from_numpy(scaled).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
        assert np.array_equal(got, expect)


@pytest.mark.gpu
def test_conv_and_from_d_copies(orc):
    """create_multi_UBspline_3d_s_cuda_conv rounds the FP64 table once; the
    16-bit copies from an FP64 table use the same per-spline scale rule."""
    grids, bcs = CASES[1][1], CASES[1][2]
    G, T, _ = build_pair(orc, "d", grids, bcs, 7, seed=31)
    c = G.to_cuda("conv")
    from einspline_gb300 import _lib as L
    import ctypes as C
    ti = L.TableInfo()
    L.load().einspline_gb300_get_table_info(c.table, C.byref(ti))
    assert ti.kind == ord("s") and ti.storage == api.STORE_F32
    out = np.empty((ti.nx, ti.ny, ti.nz, ti.ncol_pad), np.float32)
    L.load().einspline_gb300_copy_table(c.table, out.ctypes.data, None)
    assert np.array_equal(out[..., :7], T.coefs64.astype(np.float32))
    h = G.to_cuda(api.STORE_F16)
    L.load().einspline_gb300_get_table_info(h.table, C.byref(ti))
    assert ti.storage == api.STORE_F16
