import numpy as np

from einspline_gb300 import synth


def test_splitmix64_known_answer():
    # splitmix64 from state 0: published first outputs of the generator.
    z = synth.splitmix64(0, 3)
    assert [int(v) for v in z] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_uniform_range_and_offsets():
    a = synth.uniform(9, 1000, -1.0, 1.0)
    b = synth.uniform(9, 500, -1.0, 1.0, offset=500)
    assert a.min() >= -1.0 and a.max() < 1.0
    assert np.array_equal(a[500:], b)


def test_walkers_and_points():
    n = synth.walker_sizes(3, 1000)
    assert n.min() >= 32 and n.max() <= 512
    p = synth.points_uniform(4, 100, (0.0, -1.0, 2.0), (1.0, 1.0, 3.0))
    assert (p[:, 1] >= -1).all() and (p[:, 2] < 3).all()
