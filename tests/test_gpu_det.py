"""The fused determinant step (einspline_gb300_det_ratio / _det_update): the
consumer of the orbital row in the reference's QMC prototype
(src/cuda_walker.cu:69-201, src/determinant_update.h:9-111), against the
oracle's float64 restatement of the same algebra."""
import numpy as np
import pytest

from einspline_gb300 import api, synth

from helpers import build_pair

P = 0
GRIDS = [(0.0, 1.0, 12), (0.0, 1.0, 11), (0.0, 1.0, 13)]
SMALL = [(0.0, 1.0, 7), (0.0, 1.0, 8), (0.0, 1.0, 6)]
NSPL, NELEC, LD = 40, 37, 40


def _population(torch, orc, G, T, W, seed, trans, nelec=NELEC, ld=LD, distinct=None):
    """W walkers: electrons at random positions, A[e][j] = phi_j(r_e) from the
    oracle (GPU cell rule), Ainv = inv(A); float32 on the device.  With
    distinct=m only m different matrices are made and repeated."""
    rng = np.random.default_rng(seed)
    A = np.zeros((W, ld, ld), np.float32)
    Ai = np.zeros((W, ld, ld), np.float32)
    m = W if distinct is None else distinct
    for w in range(m):
        R = rng.random((nelec, 3))
        v = T.eval(R, vgh=False, sem=1)[0][:, :nelec].astype(np.float64)
        A[w, :nelec, :nelec] = v
        inv = np.linalg.inv(v)
        Ai[w, :nelec, :nelec] = inv.T if trans else inv
    for w in range(m, W):
        A[w], Ai[w] = A[w % m], Ai[w % m]
    dev = "cuda"
    D = api.Determinants(torch.from_numpy(A).to(dev), torch.from_numpy(Ai).to(dev), nelec, trans=trans)
    return D, A, Ai


def _check_ratio(orc, torch, G, D, Ai, pos, k, trans, nelec):
    """Ratios of the fused kernel against float64 sums of the flat
    evaluation's per-orbital outputs, the value row bit for bit with the
    flat evaluation in the table's load mode (the tensor cores for F16 and
    BF16 tables by default, the FMA reduction in modes 0-4)."""
    W, ld = Ai.shape[0], Ai.shape[1]
    rows = torch.zeros(W, ld, dtype=torch.float32, device="cuda")
    r, g, lap = D.ratio(G, pos, k, grad_lapl=True, rows=rows)
    r0, g0, l0 = D.ratio(G, pos, k, grad_lapl=False)
    r2, g2, l2 = D.ratio(G, pos, k, grad_lapl=True)
    torch.cuda.synchronize()
    assert torch.equal(r, r2) and torch.equal(g, g2) and torch.equal(lap, l2)
    assert g0 is None and l0 is None
    v, gr, h = G.eval(pos, vgh=True, rule=1, layout=1)
    assert torch.equal(rows[:, :nelec], v[:, :nelec])
    assert torch.count_nonzero(rows[:, nelec:]) == 0
    Astd = _ainv_std(Ai, trans)[:, :nelec, :nelec]
    vv, gg, hh = (x.cpu().numpy()[:, :nelec] for x in (v, gr, h))
    ref = orc.det_ratio(vv, gg, hh, Astd, k)
    sr, sg, sl = orc.det_ratio_bound(vv, gg, hh, Astd, k)
    R = r.cpu().numpy().astype(np.float64)
    eps = 1e-5
    assert np.all(np.abs(R - ref[0]) <= eps * sr)
    assert np.all(np.abs(r0.cpu().numpy() - ref[0]) <= eps * sr)
    Rr = np.abs(ref[0])
    gb = eps * (sg / Rr[:, None] + np.abs(ref[1]) * (sr / Rr)[:, None])
    assert np.all(np.abs(g.cpu().numpy() - ref[1]) <= gb)
    lb = eps * (sl / Rr + np.abs(ref[2]) * sr / Rr)
    assert np.all(np.abs(lap.cpu().numpy() - ref[2]) <= lb)
    return R, Astd


def _ainv_std(Ai, trans):
    """Ainv indexed [orbital j][electron e] whatever the storage."""
    return np.transpose(Ai, (0, 2, 1)) if trans else Ai


@pytest.mark.gpu
@pytest.mark.parametrize("trans", [0, 1])
@pytest.mark.parametrize("storage,mode", [(api.STORE_F32, -1), (api.STORE_F16, -1), (api.STORE_F16, 3),
                                          (api.STORE_BF16, -1), (api.STORE_I16, -1)])
def test_det_ratio(orc, trans, storage, mode):
    """F16 and BF16 tables take the tensor-core ratio kernel in their default
    load mode and the FMA kernel in modes 0-4 (mode 3 here)."""
    torch = pytest.importorskip("torch")
    G, T, _ = build_pair(orc, "s", GRIDS, [(P, P)] * 3, NSPL, seed=301, storage=storage)
    G.set_load_mode(mode)
    W, k = 9, 5
    D, A, Ai = _population(torch, orc, G, T, W, 302, trans)
    pos = torch.from_numpy(synth.points_uniform(303, W, [0.0] * 3, [1.0] * 3).astype(np.float32)).cuda()
    R, Astd = _check_ratio(orc, torch, G, D, Ai, pos, k, trans, NELEC)
    if storage == api.STORE_F32:
        # and against the oracle's own evaluation of the same table
        ov, og, oh = (x[:, :NELEC] for x in T.eval(pos.cpu().numpy().astype(np.float64), vgh=True, sem=1))
        oref = orc.det_ratio(ov, og, oh, Astd, k)
        sr = orc.det_ratio_bound(ov, og, oh, Astd, k)[0]
        assert np.all(np.abs(R - oref[0]) <= 4e-5 * sr)


@pytest.mark.gpu
@pytest.mark.parametrize("storage,nelec", [(api.STORE_F32, 600), (api.STORE_F16, 1100), (api.STORE_BF16, 700)])
def test_det_ratio_column_groups(orc, storage, nelec):
    """More orbitals than one block's column group (512 FP32 / 1024 16-bit
    columns for the FMA kernel) or 128-orbital tiles (the tensor-core
    kernel: 9 and 6 of them, the last partial): the per-walker sums run over
    several groups."""
    torch = pytest.importorskip("torch")
    nspl, ld = nelec + 24, nelec + 4
    G, T, _ = build_pair(orc, "s", SMALL, [(P, P)] * 3, nspl, seed=341, storage=storage)
    W, k = 3, nelec - 2
    D, A, Ai = _population(torch, orc, G, T, W, 342, 1, nelec=nelec, ld=ld)
    pos = torch.from_numpy(synth.points_uniform(343, W, [0.0] * 3, [1.0] * 3).astype(np.float32)).cuda()
    _check_ratio(orc, torch, G, D, Ai, pos, k, 1, nelec)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [-1, 3])
def test_det_ratio_many_walkers(orc, mode):
    """Enough walkers that a block takes several: the FMA kernel (mode 3)
    packs walkers per block beyond one wave, the tensor-core kernel (the F16
    default) spreads them evenly over whole waves of at most 7 a block."""
    torch = pytest.importorskip("torch")
    G, T, _ = build_pair(orc, "s", GRIDS, [(P, P)] * 3, NSPL, seed=351, storage=api.STORE_F16)
    G.set_load_mode(mode)
    W, k = 5000, 11
    D, A, Ai = _population(torch, orc, G, T, W, 352, 0, distinct=16)
    pos = torch.from_numpy(synth.points_uniform(353, W, [0.0] * 3, [1.0] * 3).astype(np.float32)).cuda()
    _check_ratio(orc, torch, G, D, Ai, pos, k, 0, NELEC)


@pytest.mark.gpu
@pytest.mark.parametrize("trans", [0, 1])
def test_det_update(orc, trans):
    torch = pytest.importorskip("torch")
    G, T, _ = build_pair(orc, "s", GRIDS, [(P, P)] * 3, NSPL, seed=311)
    W, k = 6, 7
    D, A, Ai = _population(torch, orc, G, T, W, 312, trans)
    pos = torch.from_numpy(synth.points_uniform(313, W, [0.0] * 3, [1.0] * 3).astype(np.float32)).cuda()
    rows = torch.zeros(W, LD, dtype=torch.float32, device="cuda")
    D.ratio(G, pos, k, grad_lapl=False, rows=rows)
    accepted = [0, 2, 3, 5]
    D.update(k, accepted, rows)
    torch.cuda.synchronize()
    A2, Ai2, U = D.A.cpu().numpy(), D.ainv.cpu().numpy(), rows.cpu().numpy()
    for w in range(W):
        if w not in accepted:
            assert np.array_equal(A2[w], A[w]) and np.array_equal(Ai2[w], Ai[w])
            continue
        rA, rAi = orc.sm_update(A[w, :NELEC, :NELEC], _ainv_std(Ai, trans)[w, :NELEC, :NELEC], k, U[w, :NELEC])
        assert np.array_equal(A2[w, k, :NELEC], U[w, :NELEC])
        others = [e for e in range(LD) if e != k]
        assert np.array_equal(A2[w, others], A[w, others])
        got = _ainv_std(Ai2, trans)[w, :NELEC, :NELEC]
        ai0 = _ainv_std(Ai, trans)[w, :NELEC, :NELEC].astype(np.float64)
        x = (U[w, :NELEC].astype(np.float64) - A[w, k, :NELEC]) @ ai0
        scale = np.abs(ai0).max() + np.abs(ai0[:, k]).max() * np.abs(x).max() / abs(1.0 + x[k])
        assert np.abs(got - rAi).max() <= 1e-5 * scale
        # padding outside the N x N block is untouched
        assert np.array_equal(Ai2[w, NELEC:], Ai[w, NELEC:]) and np.array_equal(Ai2[w, :, NELEC:], Ai[w, :, NELEC:])


@pytest.mark.gpu
def test_det_sequence_stays_inverse(orc):
    """A sweep of accepted moves over every electron: the updated inverse
    still inverts the updated matrix (float32 drift bounded)."""
    torch = pytest.importorskip("torch")
    G, T, _ = build_pair(orc, "s", GRIDS, [(P, P)] * 3, NSPL, seed=321)
    W = 4
    D, A, Ai = _population(torch, orc, G, T, W, 322, 1)
    rows = torch.zeros(W, LD, dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(323)
    logdet = np.zeros(W)
    for e in range(NELEC):
        pos = torch.from_numpy(rng.random((W, 3)).astype(np.float32)).cuda()
        r, _, _ = D.ratio(G, pos, e, grad_lapl=False, rows=rows)
        D.update(e, list(range(W)), rows)
        logdet += np.log(np.abs(r.cpu().numpy().astype(np.float64)))
    torch.cuda.synchronize()
    A2 = D.A.cpu().numpy()[:, :NELEC, :NELEC].astype(np.float64)
    Ai2 = np.transpose(D.ainv.cpu().numpy(), (0, 2, 1))[:, :NELEC, :NELEC].astype(np.float64)
    for w in range(W):
        err = np.abs(A2[w] @ Ai2[w] - np.eye(NELEC)).max()
        assert err < 1e-2, err
        # the product of the ratios is the determinant ratio
        d0 = np.linalg.slogdet(A[w, :NELEC, :NELEC].astype(np.float64))[1]
        d1 = np.linalg.slogdet(A2[w])[1]
        assert abs((d1 - d0) - logdet[w]) < 1e-2


@pytest.mark.gpu
def test_det_errors(orc):
    torch = pytest.importorskip("torch")
    G, T, _ = build_pair(orc, "s", GRIDS, [(P, P)] * 3, NSPL, seed=331)
    D, A, Ai = _population(torch, orc, G, T, 2, 332, 0)
    pos = torch.zeros(2, 3, dtype=torch.float32, device="cuda")
    with pytest.raises(api.EinsplineError):
        D.ratio(G, pos, NELEC)          # k out of range
    big = torch.zeros(2, 48, 48, dtype=torch.float32, device="cuda")
    Dbig = api.Determinants(big, big.clone(), NSPL + 1)
    with pytest.raises(api.EinsplineError):
        Dbig.ratio(G, pos, 0)           # more electrons than orbitals
    Gd, _, _ = build_pair(orc, "d", GRIDS, [(P, P)] * 3, 8, seed=333)
    with pytest.raises(api.EinsplineError):
        D.ratio(Gd, pos, 0)             # FP64 tables are not taken


@pytest.mark.gpu
def test_det_update_matches_reference_fixture(orc):
    """The GPU update against the reference's own host update_inverse
    (src/determinant_update.cu:171-187) on the committed fixture."""
    import os
    torch = pytest.importorskip("torch")
    z = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "det_update.npz"))
    A, ainv, u, k = z["A"], z["ainv"], z["u"], int(z["k"])
    N = A.shape[0]
    D = api.Determinants(torch.from_numpy(A[None].copy()).cuda(), torch.from_numpy(ainv[None].copy()).cuda(), N,
                         trans=0)
    rows = torch.from_numpy(u[None].copy()).cuda()
    D.update(k, [0], rows)
    torch.cuda.synchronize()
    got = D.ainv.cpu().numpy()[0].astype(np.float64)
    ref = z["ainv_ref"].astype(np.float64)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    assert np.array_equal(D.A.cpu().numpy()[0][k], u)


@pytest.mark.gpu
def test_det_tc_bounded_wait_runs_out_and_reports(orc):
    """The tensor-core ratio kernel's waits are bounded: the test hook makes
    the first block issue no stencil copy for its first walker and shortens
    every wait to 2 ms; the launch ends by itself, reports ETIMEOUT once,
    frees its tensor memory, and the next launch is clean and the same as
    before."""
    torch = pytest.importorskip("torch")
    from einspline_gb300 import _lib as L
    lib = L.load()
    G, T, _ = build_pair(orc, "s", GRIDS, [(P, P)] * 3, NSPL, seed=361, storage=api.STORE_F16)
    W, k = 9, 4
    D, A, Ai = _population(torch, orc, G, T, W, 362, 1)
    pos = torch.from_numpy(synth.points_uniform(363, W, [0.0] * 3, [1.0] * 3).astype(np.float32)).cuda()
    base = [x.clone() for x in D.ratio(G, pos, k, grad_lapl=True)]
    torch.cuda.synchronize()
    assert lib.einspline_gb300_wait_status(G.table) == 0
    assert lib.einspline_gb300_test_wait_timeout(G.table, 0, 0.002) == 0
    D.ratio(G, pos, k, grad_lapl=True)
    torch.cuda.synchronize()
    assert lib.einspline_gb300_wait_status(G.table) == 6  # EINSPLINE_GB300_ETIMEOUT
    lib.einspline_gb300_clear_error()
    assert lib.einspline_gb300_wait_status(G.table) == 0
    again = D.ratio(G, pos, k, grad_lapl=True)
    torch.cuda.synchronize()
    for a, b in zip(again, base):
        assert torch.equal(a, b)
    assert lib.einspline_gb300_wait_status(G.table) == 0
