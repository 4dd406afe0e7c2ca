"""The phase/surface classification of FluidState::update_cells
(src/fluid/phase.wgsl:10-31, src/fluid/mod.rs:713-852).

CPU: the oracle's restatement against the rules read off the shader (mobility
threshold 1e-6, walls of other non-air materials, frozen liquid, the
[-1e-5, 1+1e-5] fraction tolerance of src/surface.rs:12, untouched cells and
lanes).  GPU (mhdproj_classify_cells): bit-identical masks, FluidCell records
and flags on random fields in both record layouts (plain arrays and the
reference's packed thermal/interface records), the reference's error for an
out-of-range fraction, and the update_cells flow into the GPU topology
labelling.
"""
import numpy as np
import pytest

N_MAT = 4


def _case(rng, n, surface, thermal=True, bad=0):
    materials = rng.integers(0, N_MAT, n).astype(np.uint32)
    mask = rng.integers(0, 2, n).astype(np.uint32)
    cells = rng.standard_normal((n, 16)).astype(np.float32)
    th = None
    if thermal:
        th = rng.random(n).astype(np.float32)
        th[rng.random(n) < 0.3] = 0.0
        th[rng.random(n) < 0.05] = np.float32(1e-6)
    it = None
    if surface:
        it = np.zeros((n, 2), np.float32)
        it[:, 0] = rng.random(n).astype(np.float32)
        it[rng.random(n) < 0.3, 0] = 0.0
        it[rng.random(n) < 0.1, 0] = np.float32(1.0 + 0.5e-5)
        it[rng.random(n) < 0.1, 0] = np.float32(-0.5e-5)
        it[:, 1] = rng.standard_normal(n).astype(np.float32)
        if bad:
            idx = rng.choice(n, bad, replace=False)
            it[idx[: bad // 2 + 1], 0] = np.float32(1.0 + 3e-5)
            it[idx[bad // 2 + 1:], 0] = np.nan
    return materials, mask, cells, th, it


def test_phase_rules(oracle_lib):
    mats = np.array([1, 1, 2, 0, 1], np.uint32)
    th = np.array([0.5, 1e-6, 0.9, 0.9, 2e-6], np.float32)
    mask = np.array([0, 1, 1, 1, 0], np.uint32)
    cells = np.zeros((5, 16), np.float32)
    flags = oracle_lib.classify_cells(mats, 1, mask, cells, thermal=th)
    assert list(mask) == [1, 0, 0, 0, 1] and flags == 1
    np.testing.assert_array_equal(cells[:, 13], np.array([0.5, 1e-6, 0.0, 0.0, 2e-6], np.float32))
    assert not cells[:, [0, 12, 14, 15]].any()
    again = oracle_lib.classify_cells(mats, 1, mask, cells, thermal=th)
    assert again == 0  # nothing changes the second time


def test_surface_rules(oracle_lib):
    mats = np.array([0, 1, 2, 1, 0, 2], np.uint32)          # 2 is a wall material
    a = np.array([0.0, 0.7, 0.3, 0.4, 1.0 + 0.9e-5, 0.0], np.float32)
    y = np.arange(6, dtype=np.float32)
    th = np.array([0.0, 0.0, 0.5, 0.5, 0.0, 0.0], np.float32)
    it = np.stack([a, y], 1)
    mask = np.zeros(6, np.uint32)
    cells = np.full((6, 16), 7.0, np.float32)
    flags = oracle_lib.classify_cells(mats, 1, mask, cells, thermal=th, interface=it)
    # cells 1 and 4 (a > 0, thermal phase 0): frozen, not mobile; cell 2: wall
    assert list(mask) == [1, 0, 0, 1, 0, 0] and flags == 1
    np.testing.assert_array_equal(cells[:, 12:16], np.stack([np.ones(6), [1, 0, 0.5, 0.5, 0, 1], a, y], 1)
                                  .astype(np.float32))
    assert (cells[:, :12] == 7.0).all()
    # without a thermal phase f = 1: the liquid cell 1 is mobile
    mask2 = np.zeros(6, np.uint32)
    oracle_lib.classify_cells(mats, 1, mask2, cells, interface=it)
    assert list(mask2) == [1, 1, 0, 1, 1, 0]


def test_out_of_range_fraction_is_flagged(oracle_lib):
    mats = np.zeros(4, np.uint32)
    for bad in (1.0 + 2e-5, -2e-5, np.nan, np.inf):
        it = np.array([[0.5, 0], [bad, 0], [0.2, 0], [0.0, 0]], np.float32)
        mask = np.zeros(4, np.uint32)
        cells = np.zeros((4, 16), np.float32)
        flags = oracle_lib.classify_cells(mats, 1, mask, cells, interface=it)
        assert flags & 2
        assert mask[1] == 0 and not cells[1].any()   # the bad cell is left untouched


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 1000, 257 * 311])
@pytest.mark.parametrize("mode", ["phase", "surface", "surface_no_thermal"])
@pytest.mark.parametrize("packed", [False, True])
def test_gpu_matches_oracle(gpu, oracle_lib, n, mode, packed):
    import mhdproj

    torch = gpu
    rng = np.random.default_rng(n + len(mode) + packed)
    surface = mode != "phase"
    materials, mask, cells, th, it = _case(rng, n, surface, thermal=mode != "surface_no_thermal")
    ts, is_ = 1, 2
    th_in, it_in = th, it
    if packed:  # the reference's records: thermal packet (16 floats, state.y at 1), interface vec4
        ts, is_ = 16, 4
        if th is not None:
            pk = rng.standard_normal((n, 16)).astype(np.float32)
            pk[:, 1] = th
            th_in = pk
        if it is not None:
            v4 = rng.standard_normal((n, 4)).astype(np.float32)
            v4[:, :2] = it
            it_in = v4
    m_ref, c_ref = mask.copy(), cells.copy()
    f_ref = oracle_lib.classify_cells(materials, 1, m_ref, c_ref, thermal=th, interface=it)
    t = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda()
    m_gpu = t(mask.view(np.int32))
    c_gpu = t(cells)
    # packed: a view of the whole packet starting at state.y (offset 1 float)
    th_t = None if th_in is None else (t(th_in).view(-1)[1:] if packed else t(th_in))
    it_t = t(it_in)
    flags = mhdproj.classify_cells((n, 1, 1), t(materials.view(np.int32)), 1, m_gpu, c_gpu, thermal=th_t,
                                   thermal_stride=ts, interface=it_t, interface_stride=is_)
    assert flags == f_ref
    np.testing.assert_array_equal(m_gpu.cpu().numpy().view(np.uint32), m_ref)
    np.testing.assert_array_equal(c_gpu.cpu().numpy().view(np.uint32), c_ref.view(np.uint32))


@pytest.mark.gpu
def test_gpu_out_of_range_raises(gpu):
    import mhdproj

    torch = gpu
    n = 5000
    rng = np.random.default_rng(9)
    materials, mask, cells, th, it = _case(rng, n, True, bad=3)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    with pytest.raises(mhdproj.ProjectionError) as e:
        mhdproj.classify_cells((n, 1, 1), t(materials.view(np.int32)), 1, t(mask.view(np.int32)), t(cells),
                               thermal=t(th), interface=t(it))
    assert e.value.code == 1 and "roundoff tolerance" in str(e.value)


@pytest.mark.gpu
def test_update_cells_flow_relabels_topology(gpu, oracle_lib):
    """update_cells: classify, and when mobility changed relabel the
    components on the GPU (mhdproj_set_coefficients) -- equal to the
    oracle's classification followed by the reference's anchors search."""
    import mhdproj

    torch = gpu
    dims = (40, 24, 16)
    n = dims[0] * dims[1] * dims[2]
    rng = np.random.default_rng(4)
    materials = np.where(rng.random(n) < 0.25, 2, 1).astype(np.uint32)
    it = np.stack([rng.random(n).astype(np.float32), np.zeros(n, np.float32)], 1)
    mask = np.ones(n, np.uint32)
    cells = np.zeros((n, 16), np.float32)
    m_ref = mask.copy()
    oracle_lib.classify_cells(materials, 1, m_ref, cells.copy(), interface=it)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    m_gpu, c_gpu = t(mask.view(np.int32)), t(cells)
    flags = mhdproj.classify_cells(dims, t(materials.view(np.int32)), 1, m_gpu, c_gpu, interface=t(it))
    assert flags & 1
    solid = (m_gpu == 0).to(torch.uint8).view(dims[2], dims[1], dims[0])
    alpha = c_gpu[:, 14].contiguous().view(dims[2], dims[1], dims[0])
    pr = mhdproj.PressureProjection(dims, 1e-4, outlet=False, solver="reference", rel_tol=1e-5)
    pr.set_coefficients(alpha, solid, 6440.0, 1.2)
    got, comps = pr.topology()
    want_c, want = oracle_lib.anchors(m_ref, list(dims), 0)
    assert comps == want_c
    np.testing.assert_array_equal(got, np.asarray(want, np.uint32))
    pr.close()
