"""Request server: continuous batching with admission by device memory.
Each request's results are bit-identical alone and in a mix of concurrent
requests, and equal to the direct batched evaluation."""
import numpy as np
import pytest

from einspline_gb300 import api, synth

P = 0


def make_spline(kind="s", N=96, M=20, storage=api.STORE_NATIVE):
    grids = [(0.0, 1.0, M)] * 3
    G = api.MultiUBspline3D(kind, grids, [(P, P)] * 3, N, storage=storage)
    data = synth.grid_data_uniform(61, (M, M, M), N, np.float32 if kind in "sc" else np.float64,
                                   complex_=kind in "cz")
    for i in range(N):
        G.set(i, data[i])
    G.flush()
    return G


@pytest.mark.gpu
@pytest.mark.parametrize("use_graphs,sort", [(True, False), (False, False), (True, True)])
def test_alone_equals_in_mix(use_graphs, sort):
    """(sort: each batch visited in cell order, with its own sort scratch per
    in-flight slot; the results are the same bits.)"""
    import torch
    G = make_spline()
    S = api.Server(G, use_graphs=use_graphs, max_inflight=3, max_batch_points=2048, sort=sort)
    probe = synth.points_uniform(62, 300)
    rid = S.submit(probe)
    S.wait(rid)
    alone = S.result(rid, 300)
    S.release(rid)
    # the same request in the middle of 120 uneven concurrent requests
    sizes = synth.walker_sizes(63, 120)
    others = [synth.points_uniform(64 + i, int(n)) for i, n in enumerate(sizes)]
    ids = []
    for i, p in enumerate(others):
        ids.append((S.submit(p), p.shape[0]))
        if i == 60:
            mid = S.submit(probe)
    for r, n in ids:
        S.wait(r)
    S.wait(mid)
    mixed = S.result(mid, 300)
    for a, b in zip(alone, mixed):
        assert np.array_equal(a, b)
    # and equal to the direct evaluation of the same points
    direct = G.eval(torch.from_numpy(probe).cuda(), rule=0, layout=0)
    assert np.array_equal(direct[0].cpu().numpy(), alone[0])
    assert np.array_equal(direct[1].cpu().numpy().reshape(300, -1), alone[1])
    assert np.array_equal(direct[2].cpu().numpy().reshape(300, -1), alone[2])
    # every other request also matches its direct evaluation
    for (r, n), p in list(zip(ids, others))[::17]:
        got = S.result(r, n)
        d = G.eval(torch.from_numpy(p).cuda(), rule=0, layout=0)[0].cpu().numpy()
        assert np.array_equal(got[0], d)
    st = S.stats()
    assert st.completed == 122 and st.batches >= 2
    S.close()


@pytest.mark.gpu
def test_admission_waits_for_memory_and_bounded_waits():
    G = make_spline(N=64, M=16)
    per_req = 100 * 64 * 10 * 4  # outputs of a 100-point request
    S = api.Server(G, max_inflight=2, max_batch_points=4096, hbm_budget_bytes=3 * per_req + 4096)
    pts = [synth.points_uniform(70 + i, 100) for i in range(8)]
    ids = [S.submit(p) for p in pts]
    S.wait(ids[0])
    S.wait(ids[2])
    # the budget holds three requests: the fourth cannot be admitted yet
    with pytest.raises(api.EinsplineError, match="not done"):
        S.wait(ids[3], timeout=0.3)
    for r in ids[:3]:
        S.release(r)
    for r in ids[3:]:
        S.wait(r)
        S.release(r)
    st = S.stats()
    assert st.peak_bytes_in_use <= st.budget_bytes
    assert st.completed == 8 and st.released == 8
    # refusals are status codes, not aborts
    with pytest.raises(api.EinsplineError, match="exceed"):
        S.submit(synth.points_uniform(80, 5000))
    with pytest.raises(api.EinsplineError, match="unknown"):
        S.release(123456)
    S.close()


@pytest.mark.gpu
def test_replay_poisson_trace():
    G = make_spline(N=128, M=24, storage=api.STORE_F16)
    S = api.Server(G, max_inflight=3, max_batch_points=8192)
    n = 300
    sizes = synth.walker_sizes(90, n)
    arr = synth.poisson_arrivals(91, n, 3000.0)
    pos = synth.points_uniform(92, int(sizes.sum()))
    lat, wall = S.replay(arr, sizes, pos)
    assert (lat > 0).all()
    assert wall >= arr[-1]
    st = S.stats()
    assert st.completed == n and st.released == n
    S.close()


@pytest.mark.gpu
@pytest.mark.parametrize("use_graphs", [True, False])
def test_concurrent_clients(use_graphs):
    """Four host threads submit, wait for, check and release uneven requests
    at once against one server with a tight memory budget (admission must
    wait for releases); every result equals the direct evaluation bit for
    bit and the server's counters balance at the end."""
    import threading

    import torch
    G = make_spline(N=64, M=16)
    per_pt = 10 * 64 * 4
    S = api.Server(G, use_graphs=use_graphs, max_inflight=3, max_batch_points=2048,
                   hbm_budget_bytes=6 * 512 * per_pt)
    errors = []

    def client(c):
        try:
            rng = np.random.default_rng(700 + c)
            for r in range(60):
                n = int(rng.integers(1, 512))
                pos = synth.points_uniform(800 + 97 * c + r, n)
                rid = S.submit(pos)
                S.wait(rid, timeout=60.0)
                got = S.result(rid, n)
                S.release(rid)
                ref = G.eval(torch.from_numpy(pos).cuda(), vgh=True, rule=0, layout=0)
                for a, b in zip(got, ref):
                    if not np.array_equal(a, b.cpu().numpy().reshape(a.shape)):
                        errors.append((c, r))
                        return
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append((c, repr(e)))

    threads = [threading.Thread(target=client, args=(c,)) for c in range(4)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not any(t.is_alive() for t in threads), "a client did not finish"
    assert not errors, errors[:3]
    st = S.stats()
    assert st.submitted == st.completed == st.released == 240
    S.close()
