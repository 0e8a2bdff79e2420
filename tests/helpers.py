"""Shared helpers for the parity tests: the same seeded spline built by the
GPU library and by the oracle, output-layout conversions and tolerances."""
from __future__ import annotations

import numpy as np

from einspline_gb300 import api, synth

# Parity tolerances, as max |gpu - oracle| / max |oracle| per quantity
# (value, gradient, Hessian separately).  FP32 arithmetic (s/c, and the
# 16-bit tables which compute in FP32) vs the oracle's FP32 on the same
# table: a few ulps of the accumulated sum.  FP64 (d/z): 1e-12 relative.
TOL = {"s": 2e-5, "c": 2e-5, "d": 1e-12, "z": 1e-12}

HESS6 = [0, 1, 2, 4, 5, 8]  # (xx, xy, xz, yy, yz, zz) in a row-major 3x3


def build_pair(orc, kind, grids, bcs, N, seed=11, storage=api.STORE_NATIVE, data=None):
    """(gpu spline, oracle table, data): data set through set_multi_UBspline_3d_*."""
    M = tuple(g[2] for g in grids)
    cpx = kind in "cz"
    dt = np.float32 if kind in "sc" else np.float64
    if data is None:
        data = synth.grid_data_uniform(seed, M, N, dt, complex_=cpx)
    G = api.MultiUBspline3D(kind, grids, bcs, N, storage=storage)
    T = orc.Table(kind, grids, oracle_bcs(kind, bcs), N)
    for i in range(N):
        G.set(i, data[i])
        T.set_spline(i, data[i].astype(np.float64))
    G.flush()
    return G, T, data


def oracle_bcs(kind, bcs):
    """Boundary values as the C API carries them: float for s/c
    (BCtype_s/BCtype_c), double for d/z."""
    if kind not in "sc":
        return bcs
    return [tuple(b[:2]) + tuple(float(np.float32(v)) for v in b[2:]) for b in bcs]


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


def assert_close(got, ref, tol, what=""):
    names = ("value", "gradient", "hessian")
    for n, x, y in zip(names, got, ref):
        if x is None or y is None:
            continue
        e = rel_err(x, y)
        assert e <= tol, f"{what} {n}: rel err {e:.3e} > {tol:.1e}"


def cpu_to_gpu_layout(kind, v, g, h):
    """Oracle CPU layout -> reference GPU layout (hess [N][6]; complex
    grads/hess [N][re,im][3|6])."""
    if kind in "cz":
        P, N = v.shape[:2]
        g2 = np.moveaxis(g, -1, -2)               # [P][N][2][3]
        hh = h.reshape(P, N, 9, 2)[:, :, HESS6, :]  # [P][N][6][2]
        h2 = np.moveaxis(hh, -1, -2)              # [P][N][2][6]
        return v, g2, h2
    P, N = v.shape[:2]
    return v, g, h.reshape(P, N, 9)[:, :, HESS6]


def table_box(grids):
    return [g[0] for g in grids], [g[1] for g in grids]


def planewave_analytic(k, amp, pos):
    """Value, gradient and Hessian of the real part of sum_w amp[s, w]
    exp(2 pi i k[s, w] . r) at pos [P, 3]: [P, S], [P, S, 3], [P, S, 3, 3]
    (the functions synth.grid_data_planewaves samples on the grid)."""
    e = np.exp(2j * np.pi * np.einsum("swa,pa->psw", k, pos)) * amp[None]
    tk = 2j * np.pi * k
    return (e.sum(-1).real, np.einsum("psw,swa->psa", e, tk).real,
            np.einsum("psw,swa,swb->psab", e, tk, tk).real)


def rms_rel(a, b):
    """RMS of a - b relative to the RMS of b."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


# Cubic B-spline interpolation of smooth periodic data converges as h^4
# (value), h^3 (gradient) and h^2 (Hessian): halving the grid spacing divides
# the errors by about 16, 8 and 4.
CONVERGENCE_RATIOS = ((13.0, 20.0), (6.5, 10.5), (3.3, 4.8))
