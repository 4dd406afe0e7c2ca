import numpy as np

from mhdproj import synth


def test_streams_are_deterministic_and_seeded():
    a = synth.normal(1, 3, 1000)
    b = synth.normal(1, 3, 1000)
    c = synth.normal(2, 3, 1000)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert abs(a.mean()) < 0.1 and abs(a.std() - 1) < 0.1


def test_workload_shapes():
    c = synth.make_case("jet128", scale=0.125)
    nx, ny, nz = c["dims"]
    assert c["alpha"].shape == (nz, ny, nx) and c["solid"].dtype == np.uint8
    assert c["u"].shape == (nz, ny, nx + 1) and c["v"].shape == (nz, ny + 1, nx) and c["w"].shape == (nz + 1, ny, nx)
    assert c["solid"][: nz // 4].any() and not c["solid"][nz // 2:].any()
    d = synth.make_case("adjoint128", scale=0.125)
    assert d["fu"].shape == d["u"].shape and d["steps"] == 8 and d["checkpoint_every"] == 4
