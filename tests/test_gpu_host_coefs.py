"""Host mirror of the coefficients (einspline_gb300_host_coefs / _push /
_release): the reference keeps spline->coefs in host memory
(src/multi_bspline_structs.h:155-164), so callers read and write it there;
the mirror gives them the same layout and value type, and a push makes host
edits the table the GPU evaluates."""
import numpy as np
import pytest

from einspline_gb300 import api, synth

from helpers import build_pair

P = 0
GRIDS = [(0.0, 1.0, 10), (0.0, 1.0, 9), (0.0, 1.0, 11)]


def tpos(pos):
    import torch
    return torch.from_numpy(np.ascontiguousarray(pos, np.float64)).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", "sdcz")
def test_mirror_equals_the_table_and_push_replaces_it(orc, kind):
    """The mirror holds the device table in the value type; copying table B's
    mirror into table A's and pushing makes A evaluate exactly as B, also in
    double-float mode for FP64 tables (its copy is rebuilt)."""
    A, _, _ = build_pair(orc, kind, GRIDS, [(P, P)] * 3, 21, seed=901)
    B, _, _ = build_pair(orc, kind, GRIDS, [(P, P)] * 3, 21, seed=902)
    raw, _ = A.table_host()
    ma = A.host_coefs()
    assert ma.dtype == (np.float64 if kind in "dz" else np.float32)
    assert np.array_equal(ma, raw.view(ma.dtype).reshape(ma.shape))
    pt = tpos(synth.points_uniform(903, 600))
    if kind == "d":
        A.set_fp64_mode(1)
        B.set_fp64_mode(1)
    ref = [x.cpu().numpy() for x in B.eval(pt, rule=0, layout=0)]
    before = [x.cpu().numpy() for x in A.eval(pt, rule=0, layout=0)]
    assert not np.array_equal(before[0], ref[0])
    ma[...] = B.host_coefs()
    A.push_host_coefs()
    got = [x.cpu().numpy() for x in A.eval(pt, rule=0, layout=0)]
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    # a second call refreshes the same mirror from the device
    assert np.array_equal(A.host_coefs(), B.host_coefs())
    A.release_host_coefs()
    B.release_host_coefs()
    A.release_host_coefs()  # releasing twice is harmless
    A.wait_status()


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [api.STORE_F16, api.STORE_BF16, api.STORE_I16])
def test_mirror_of_16bit_tables_is_dequantized_and_read_only(orc, storage):
    A, _, _ = build_pair(orc, "s", GRIDS, [(P, P)] * 3, 37, seed=911, storage=storage)
    m = A.host_coefs()
    vals = A.table_values()
    np.testing.assert_allclose(m[..., :37], vals, rtol=1e-6, atol=0)
    assert not m[..., 37:].any()
    with pytest.raises(api.EinsplineError):
        A.push_host_coefs()


@pytest.mark.gpu
def test_push_without_mirror_is_an_error():
    A = api.MultiUBspline3D("s", GRIDS, [(P, P)] * 3, 3)
    with pytest.raises(api.EinsplineError):
        A.push_host_coefs()
