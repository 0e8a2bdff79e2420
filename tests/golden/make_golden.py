"""Generate the golden vectors in this directory from the reference's own CPU
library (oracle/_ref/libeinspline_ref.so, built from the reference sources by
``make -C oracle ref``).

Each 3D case stores the seeded input data, the table the reference's
set_multi_UBspline_3d_* produced (its float solve for s/c, double for d/z),
evaluation points, and the reference's eval_multi_UBspline_3d_*, _vgh and
_vghgh outputs at those points.  The ld1_*/ld2_* cases do the same for the
1D and 2D multi-splines (value, vg, vgl and vgh forms); det_update holds the
reference's host Sherman-Morrison update (src/determinant_update.cu:171-187)
on seeded inputs.  The tests then pin the
oracle against these vectors on machines where the reference cannot be built.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from einspline_gb300 import synth  # noqa: E402

P, D1, D2, FL, NA, AP = O.PERIODIC, O.DERIV1, O.DERIV2, O.FLAT, O.NATURAL, O.ANTIPERIODIC

# (name, kind, grids, bcs, num_splines, npts)
CASES = [
    ("s_periodic", "s", [(0.0, 1.0, 8), (0.0, 1.0, 7), (0.0, 1.0, 9)], [(P, P)] * 3, 6, 40),
    ("s_mixed", "s", [(-0.3, 1.1, 7), (0.2, 0.9, 6), (0.0, 2.0, 8)],
     [(NA, D1, 0.0, 0.0, 0.4, 0.0), (D2, FL, -0.7, 0.0, 0.0, 0.0), (AP, AP)], 5, 40),
    ("d_periodic", "d", [(0.0, 1.0, 9), (0.0, 1.0, 8), (0.0, 1.0, 7)], [(P, P)] * 3, 5, 40),
    ("d_mixed", "d", [(0.5, 1.7, 6), (-1.0, 1.0, 9), (0.0, 1.3, 7)],
     [(D1, D2, 0.25, 0.0, -0.5, 0.0), (AP, AP), (FL, NA)], 4, 40),
    ("c_periodic", "c", [(0.0, 1.0, 7), (0.0, 1.0, 8), (0.0, 1.0, 6)], [(P, P)] * 3, 4, 30),
    ("c_mixed", "c", [(0.0, 1.5, 6), (0.1, 1.0, 7), (-0.2, 0.8, 8)],
     [(NA, NA), (D1, D1, 0.3, -0.1, 0.2, 0.6), (AP, AP)], 3, 30),
    ("z_periodic", "z", [(0.0, 1.0, 6), (0.0, 1.0, 7), (0.0, 1.0, 8)], [(P, P)] * 3, 3, 30),
    ("z_mixed", "z", [(0.0, 2.0, 7), (0.3, 0.9, 6), (0.0, 1.0, 9)],
     [(D2, D1, 0.1, 0.2, -0.3, 0.4), (P, P), (FL, FL)], 3, 30),
]


def make_case(name, kind, grids, bcs, N, npts, seed):
    R = O.RefSpline(kind, grids, bcs, N)
    M = tuple(g[2] for g in grids)
    cpx = kind in "cz"
    dt = np.float32 if kind in "sc" else np.float64
    data = synth.grid_data_uniform(seed, M, N, dt, complex_=cpx)
    for i in range(N):
        R.set_spline(i, data[i])
    lo = [g[0] for g in grids]
    hi = [g[1] for g in grids]
    pos = synth.points_uniform(seed + 1, npts, lo, hi)
    v0, _, _ = R.eval(pos, vgh=False)
    v, g, h = R.eval(pos, vgh=True)
    t3 = R.eval_vghgh(pos[:8])
    bc_arr = np.array([list(b) + [0.0] * (6 - len(b)) for b in bcs], dtype=np.float64)
    return dict(kind=np.array(kind), grids=np.array(grids, dtype=np.float64), bcs=bc_arr,
                num_splines=np.array(N), data=data, table=R.table(), pos=pos,
                value=v0, vals=v, grads=g, hess=h,
                vghgh_vals=t3[0], vghgh_grads=t3[1], vghgh_hess=t3[2], vghgh_gradhess=t3[3])


# 1D and 2D multi-splines: (name, kind, grids, bcs, num_splines, npts)
LD_CASES = [
    ("ld1_s_periodic", "s", [(0.0, 1.0, 11)], [(P, P)], 6, 24),
    ("ld1_d_mixed", "d", [(-0.4, 1.2, 9)], [(NA, D1, 0.0, 0.0, 0.6, 0.0)], 5, 24),
    ("ld1_z_anti", "z", [(0.0, 2.0, 8)], [(AP, AP)], 3, 20),
    ("ld2_c_periodic", "c", [(0.0, 1.0, 8), (0.0, 1.0, 7)], [(P, P)] * 2, 3, 20),
    ("ld2_d_mixed", "d", [(0.2, 1.4, 7), (-1.0, 0.5, 9)], [(D2, FL, 0.3, 0.0, 0.0, 0.0), (AP, AP)], 4, 24),
    ("ld2_s_mixed", "s", [(0.0, 1.5, 9), (0.0, 1.0, 6)], [(FL, NA), (P, P)], 5, 24),
]


def make_ld_case(kind, grids, bcs, N, npts, seed):
    R = O.RefSplineLD(kind, grids, bcs, N)
    M = tuple(g[2] for g in grids)
    dt = np.float32 if kind in "sc" else np.float64
    data = synth.grid_data_uniform(seed, M, N, dt, complex_=kind in "cz")
    for i in range(N):
        R.set_spline(i, data[i])
    pos = synth.points_uniform(seed + 1, npts, [g[0] for g in grids], [g[1] for g in grids])
    out = {}
    for form in range(4):
        for key, arr in zip(("v", "g", "lh"), R.eval_ld(pos, form)):
            if arr is not None:
                out[f"f{form}_{key}"] = arr
    bc_arr = np.array([list(b) + [0.0] * (6 - len(b)) for b in bcs], dtype=np.float64)
    return dict(kind=np.array(kind), grids=np.array(grids, dtype=np.float64), bcs=bc_arr,
                num_splines=np.array(N), data=data, table=R.table(), pos=pos, **out)


def make_det_case(seed=3000):
    """The reference's own Sherman-Morrison host update on seeded inputs."""
    rng = np.random.default_rng(seed)
    N, k = 48, 11
    A = (rng.standard_normal((N, N)) + 6 * np.eye(N)).astype(np.float32)
    ainv = np.linalg.inv(A.astype(np.float64)).astype(np.float32)
    u = rng.standard_normal(N).astype(np.float32)
    delta = (u - A[k]).astype(np.float32)
    return dict(A=A, ainv=ainv, u=u, k=np.array(k), ainv_ref=O.ref_det_update(ainv, delta, k))


def main():
    if not O.ref_available():
        sys.exit("reference library missing: run `make -C oracle ref` first")
    np.savez_compressed(os.path.join(HERE, "det_update.npz"), **make_det_case())
    print("wrote det_update")
    for k, (name, kind, grids, bcs, N, npts) in enumerate(CASES):
        case = make_case(name, kind, grids, bcs, N, npts, seed=1000 + 17 * k)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **case)
        print("wrote", name)
    for k, (name, kind, grids, bcs, N, npts) in enumerate(LD_CASES):
        case = make_ld_case(kind, grids, bcs, N, npts, seed=2000 + 19 * k)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **case)
        print("wrote", name)


if __name__ == "__main__":
    main()
