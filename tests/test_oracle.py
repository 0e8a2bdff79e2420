"""The oracle against the reference: bit-exact on the committed golden
vectors (made by the compiled reference, tests/golden/make_golden.py) and,
where the reference sources can be compiled, against the live reference."""
import glob
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                if not os.path.basename(p).startswith(("ld", "det")))
GOLDEN_DET = os.path.join(HERE, "golden", "det_update.npz")
REF_DET_BUILT = os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libdetupdate_ref.so"))
GOLDEN_LD = sorted(glob.glob(os.path.join(HERE, "golden", "ld*.npz")))
REF_BUILT = os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libeinspline_ref.so"))


def _load(path):
    z = np.load(path)
    kind = str(z["kind"])
    grids = [tuple(g[:2]) + (int(g[2]),) for g in z["grids"]]
    bcs = [tuple([int(b[0]), int(b[1])] + list(b[2:])) for b in z["bcs"]]
    return kind, grids, bcs, int(z["num_splines"]), z


def test_golden_present():
    assert len(GOLDEN) == 8 and len(GOLDEN_LD) == 6


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_table(orc, path):
    kind, grids, bcs, N, z = _load(path)
    T = orc.Table(kind, grids, bcs, N)
    for i in range(N):
        T.set_spline(i, z["data"][i])
    if kind in "dz":
        # FP64 solve: bit-identical to the reference's set_multi_UBspline_3d_d/z.
        assert np.array_equal(T.coefs64, z["table"])
    else:
        # The reference solves s/c in float; the FP64 solve rounded once
        # differs from it by float rounding only.
        ref = z["table"].astype(np.float64)
        rel = np.abs(T.coefs64 - ref).max() / np.abs(ref).max()
        assert rel < 1e-6


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_eval(orc, path):
    kind, grids, bcs, N, z = _load(path)
    T = orc.Table(kind, grids, bcs, N)
    table = np.ascontiguousarray(z["table"])
    v0, _, _ = T.eval(z["pos"], vgh=False, coefs=table)
    v, g, h = T.eval(z["pos"], vgh=True, coefs=table)
    assert np.array_equal(v0, z["value"])
    assert np.array_equal(v, z["vals"])
    assert np.array_equal(g, z["grads"])
    assert np.array_equal(h, z["hess"])


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref",
                                                    "libeinspline_ref.so")),
                    reason="reference library not built here (make -C oracle ref)")
@pytest.mark.parametrize("kind", "sdcz")
def test_live_reference(orc, kind):
    from einspline_gb300 import synth
    P, NA, D1, D2, FL, AP = orc.PERIODIC, orc.NATURAL, orc.DERIV1, orc.DERIV2, orc.FLAT, orc.ANTIPERIODIC
    cases = [([(0.0, 1.0, 10), (0.0, 1.0, 11), (0.0, 1.0, 12)], [(P, P)] * 3),
             ([(0.2, 1.4, 9), (-1.0, 0.5, 7), (0.0, 3.0, 10)],
              [(FL, D2, 0, 0, 0.7, -0.3), (AP, AP), (D1, NA, -0.4, 0.9, 0, 0)])]
    for grids, bcs in cases:
        N = 7
        T = orc.Table(kind, grids, bcs, N)
        R = orc.RefSpline(kind, grids, bcs, N)
        data = synth.grid_data_uniform(77, T.M, N, np.float64, complex_=kind in "cz")
        for i in range(N):
            T.set_spline(i, data[i])
            R.set_spline(i, data[i])
        if kind in "dz":
            assert np.array_equal(T.coefs64, R.table())
        R.load_table(T.coefs)
        pos = synth.points_uniform(5, 64, [g[0] for g in grids], [g[1] for g in grids])
        for vgh in (False, True):
            a = T.eval(pos, vgh=vgh)
            b = R.eval(pos, vgh=vgh)
            for x, y in zip(a, b):
                if x is not None:
                    assert np.array_equal(x, y)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(HERE), "oracle", "_ref",
                                                    "libeinspline_ref.so")),
                    reason="reference library not built here (make -C oracle ref)")
@pytest.mark.parametrize("kind", "sdcz")
def test_live_reference_vghgh(orc, kind):
    """Third derivatives (eval_multi_UBspline_3d_*_vghgh of the std backend),
    bit for bit on the reference's own table."""
    from einspline_gb300 import synth
    P, NA, D1, D2, FL, AP = orc.PERIODIC, orc.NATURAL, orc.DERIV1, orc.DERIV2, orc.FLAT, orc.ANTIPERIODIC
    cases = [([(0.0, 1.3, 7), (-0.5, 0.7, 9), (0.1, 1.0, 6)], [(P, P)] * 3),
             ([(0.0, 1.3, 7), (-0.5, 0.7, 9), (0.1, 1.0, 6)],
              [(NA, D1, 0.0, 0.0, 0.3, -0.2), (D2, FL, 0.5, 0.1, 0.0, 0.0), (AP, AP)])]
    for grids, bcs in cases:
        N = 5
        T = orc.Table(kind, grids, bcs, N)
        R = orc.RefSpline(kind, grids, bcs, N)
        data = synth.grid_data_uniform(78, T.M, N, np.float64, complex_=kind in "cz")
        for i in range(N):
            R.set_spline(i, data[i])
        tab = np.ascontiguousarray(R.table())
        pos = synth.points_uniform(6, 24, [g[0] for g in grids], [g[1] for g in grids])
        for x, y in zip(T.eval_vghgh(pos, coefs=tab), R.eval_vghgh(pos)):
            assert np.array_equal(x, y)


def test_det_oracle_algebra(orc):
    """The determinant-step restatement is the textbook algebra: the ratio is
    det(A')/det(A) and the Sherman-Morrison update is inv(A')."""
    rng = np.random.default_rng(5)
    N, k = 24, 9
    A = rng.standard_normal((N, N)) + 5 * np.eye(N)
    Ai = np.linalg.inv(A)
    u = rng.standard_normal(N)
    A2, Ai2 = orc.sm_update(A, Ai, k, u)
    assert np.abs(Ai2 - np.linalg.inv(A2)).max() <= 1e-12 * np.abs(Ai2).max()
    r, _, _ = orc.det_ratio(u[None], None, None, Ai[None], k)
    assert abs(r[0] - np.linalg.det(A2) / np.linalg.det(A)) <= 1e-12 * abs(r[0])


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_vghgh(orc, path):
    """Third derivatives (the std backend's eval_multi_UBspline_3d_*_vghgh)
    on the reference's own table, bit for bit."""
    kind, grids, bcs, N, z = _load(path)
    T = orc.Table(kind, grids, bcs, N)
    got = T.eval_vghgh(z["pos"][:8], coefs=np.ascontiguousarray(z["table"]))
    for a, key in zip(got, ("vals", "grads", "hess", "gradhess")):
        assert np.array_equal(a, z["vghgh_" + key])


@pytest.mark.parametrize("path", GOLDEN_LD, ids=[os.path.basename(p)[:-4] for p in GOLDEN_LD])
def test_golden_lowdim(orc, path):
    """1D/2D multi-splines: the FP64 solve (d/z bit-identical, s/c to float
    rounding) and every evaluation form on the reference's table."""
    kind, grids, bcs, N, z = _load(path)
    T = orc.Table(kind, grids, bcs, N)
    for i in range(N):
        T.set_spline(i, z["data"][i])
    ref = z["table"]
    if kind in "dz":
        assert np.array_equal(T.coefs64, ref)
    else:
        assert np.abs(T.coefs64 - ref).max() / np.abs(ref).max() < 1e-6
    table = np.ascontiguousarray(ref)
    for form in range(4):
        got = T.eval_ld(z["pos"], form, coefs=table)
        for key, a in zip(("v", "g", "lh"), got):
            if a is not None:
                assert np.array_equal(a, z[f"f{form}_{key}"]), (form, key)


@pytest.mark.skipif(not REF_BUILT, reason="reference library not built here (make -C oracle ref)")
@pytest.mark.parametrize("kind", "sdcz")
def test_live_reference_lowdim(orc, kind):
    """1D and 2D create/set/eval against the live reference, every BC family
    and evaluation form."""
    from einspline_gb300 import synth
    P, NA, D1, D2, FL, AP = orc.PERIODIC, orc.NATURAL, orc.DERIV1, orc.DERIV2, orc.FLAT, orc.ANTIPERIODIC
    cases = [([(0.0, 1.3, 9)], [(P, P)]), ([(-0.5, 0.7, 11)], [(NA, D1, 0.0, 0.0, 0.3, -0.2)]),
             ([(0.1, 1.0, 8)], [(AP, AP)]), ([(0.0, 1.3, 9), (-0.5, 0.7, 7)], [(P, P)] * 2),
             ([(0.0, 1.3, 9), (-0.5, 0.7, 7)], [(D2, FL, 0.5, 0.1, 0.0, 0.0), (AP, AP)])]
    for grids, bcs in cases:
        N = 5
        T = orc.Table(kind, grids, bcs, N)
        R = orc.RefSplineLD(kind, grids, bcs, N)
        data = synth.grid_data_uniform(3, T.M[:len(grids)], N, np.float64, complex_=kind in "cz")
        for i in range(N):
            T.set_spline(i, data[i])
            R.set_spline(i, data[i])
        if kind in "dz":
            assert np.array_equal(T.coefs64, R.table())
        R.load_table(T.coefs)
        pos = synth.points_uniform(5, 16, [g[0] for g in grids], [g[1] for g in grids])
        for form in range(4):
            for a, b in zip(T.eval_ld(pos, form), R.eval_ld(pos, form)):
                if a is not None:
                    assert np.array_equal(a, b)


def test_golden_det_update(orc):
    """The Sherman-Morrison restatement against the reference's own host
    update_inverse (float) on the committed fixture."""
    z = np.load(GOLDEN_DET)
    k = int(z["k"])
    _, got = orc.sm_update(z["A"], z["ainv"], k, z["u"])
    ref = z["ainv_ref"].astype(np.float64)
    assert np.abs(got - ref).max() <= 5e-6 * np.abs(ref).max()


@pytest.mark.skipif(not REF_DET_BUILT, reason="reference determinant update not built here (make -C oracle ref)")
@pytest.mark.parametrize("N,k", [(8, 0), (37, 20), (128, 127)])
def test_live_reference_det_update(orc, N, k):
    rng = np.random.default_rng(N + k)
    A = (rng.standard_normal((N, N)) + 6 * np.eye(N)).astype(np.float32)
    ainv = np.linalg.inv(A.astype(np.float64)).astype(np.float32)
    u = rng.standard_normal(N).astype(np.float32)
    ref = orc.ref_det_update(ainv, u - A[k], k).astype(np.float64)
    _, got = orc.sm_update(A, ainv, k, u)
    assert np.abs(got - ref).max() <= 5e-6 * np.abs(ref).max()


def test_reference_gpu_basis_table(orc):
    """The constant table the reference's GPU kernels read (Acuda, filled by
    create_multi_UBspline_3d_s_cuda, src/multi_bspline_create_cuda.cu:428-441),
    as the launcher builds it from the basis polynomials: power-basis rows
    (t^3, t^2, t, 1) of b0..b3, their first and their second derivatives."""
    import ref_gpu
    s = 1.0 / 6.0
    expect = [-s, 3 * s, -3 * s, s, 3 * s, -1.0, 0.0, 4 * s, -3 * s, 3 * s, 3 * s, s, s, 0.0, 0.0, 0.0,
              0.0, -0.5, 1.0, -0.5, 0.0, 1.5, -2.0, 0.0, 0.0, -1.5, 1.0, 0.5, 0.0, 0.5, 0.0, 0.0,
              0.0, 0.0, -1.0, 1.0, 0.0, 0.0, 3.0, -2.0, 0.0, 0.0, -3.0, 1.0, 0.0, 0.0, 1.0, 0.0]
    assert np.array_equal(ref_gpu.basis_table(), np.asarray(expect, dtype=np.float32))


def test_planewave_interpolation_converges(orc):
    """The analytic known-answer pattern of the reference's single-spline
    tests (src/test_bspline_d.c:40-188: a periodic plane-wave sum,
    interpolated and compared with its analytic value, gradient and Hessian;
    the reference prints the errors without a threshold).  Here the errors
    must fall at the cubic spline's rates as the grid is refined."""
    from einspline_gb300 import synth
    from helpers import CONVERGENCE_RATIOS, planewave_analytic, rms_rel
    S = 8
    pos = synth.points_uniform(91, 2000)
    err = {}
    for M in (24, 48):
        data, k, amp = synth.grid_data_planewaves(90, (M, M, M), S, waves=8, kmax=2, noise=0.0)
        T = orc.Table("d", [(0.0, 1.0, M)] * 3, [(0, 0)] * 3, S)
        for i in range(S):
            T.set_spline(i, data[i])
        v, g, h = T.eval(pos, vgh=True, sem=0)
        va, ga, ha = planewave_analytic(k, amp, pos)
        err[M] = (rms_rel(v, va), rms_rel(g, ga), rms_rel(h.reshape(ha.shape), ha))
    for q, (lo, hi) in enumerate(CONVERGENCE_RATIOS):
        assert lo <= err[24][q] / err[48][q] <= hi, (q, err)
    assert err[48][0] < 3e-5 and err[48][1] < 3e-4 and err[48][2] < 5e-3, err
