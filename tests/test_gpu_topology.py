"""GPU connected-component labelling against the oracle's breadth-first search.

The reference labels the pressure graph's components on the host
(anchors(), src/fluid/mod.rs:1447-1493): class | root << 2 with the root the
first cell of the component in x-fastest order.  The library computes the
same labels on the GPU (union-find, topology_kernels.cu) inside
mhdproj_set_coefficients; these tests read them back through
mhdproj_copy_topology and require them bit-identical to the oracle's search:
the reference solver's encoded mask (oracle.anchors) and the GB300 solver's
gauge classes with the top-outlet rule (oracle.classify).  Cases: random
solid masks around the site-percolation threshold (many components), every
periodic combination, rows that are not a multiple of the 32-cell warp
chunk, degenerate extents, empty and full masks, a topology change between
calls, and the full 256^3 jet geometry.
"""
import numpy as np
import pytest

from mhdproj import synth

pytestmark = pytest.mark.gpu


def _solid_case(rng, dims, p):
    n = dims[0] * dims[1] * dims[2]
    return (rng.random(n) < p).astype(np.uint8).reshape(dims[2], dims[1], dims[0])


def _run(torch, mhdproj, dims, periodic_bits, solid, solver, outlet=False):
    per = tuple(bool(periodic_bits & (1 << a)) for a in range(3))
    pr = mhdproj.PressureProjection(dims, 1e-4, periodic=per, outlet=outlet, solver=solver, precision="fp32",
                                    preconditioner="jacobi", rel_tol=1e-5)
    alpha = torch.ones(dims[2], dims[1], dims[0], dtype=torch.float32, device="cuda")
    s = torch.from_numpy(np.ascontiguousarray(solid)).cuda()
    pr.set_coefficients(alpha, s, 1000.0, 1000.0)
    return pr


def _check_reference(torch, mhdproj, oracle_lib, dims, per, solid):
    pr = _run(torch, mhdproj, dims, per, solid, "reference")
    got, comps = pr.topology()
    want_c, want = oracle_lib.anchors((solid.reshape(-1) == 0).astype(np.uint32), list(dims), per)
    assert comps == want_c
    np.testing.assert_array_equal(got, np.asarray(want, np.uint32))
    pr.close()


def _check_classes(torch, mhdproj, oracle_lib, dims, per, solid, outlet):
    pr = _run(torch, mhdproj, dims, per, solid, "gb300", outlet=outlet)
    got, comps = pr.topology()
    g = oracle_lib.grid(dims[0], dims[1], dims[2], 1e-4, 1000.0, 1000.0, per, outlet)
    pinned, cls = oracle_lib.classify(g, solid)
    n_comp, _ = oracle_lib.anchors((solid.reshape(-1) == 0).astype(np.uint32), list(dims), per)
    if n_comp == 1 and pinned == 1:
        cls[cls == 2] = 1  # one closed component: mean-free gauge, no pinned cell
    np.testing.assert_array_equal(got.astype(np.uint8), cls)
    want_c, _ = oracle_lib.anchors((solid.reshape(-1) == 0).astype(np.uint32), list(dims), per)
    assert comps == want_c
    pr.close()


RANDOM = [((37, 23, 19), 0, 0.30), ((64, 16, 16), 7, 0.35), ((33, 1, 40), 1, 0.25), ((1, 45, 30), 2, 0.3),
          ((70, 9, 1), 5, 0.2), ((100, 30, 12), 6, 0.45), ((31, 31, 31), 3, 0.65), ((2, 2, 2), 7, 0.3),
          ((96, 40, 24), 4, 0.32)]


@pytest.mark.parametrize("dims,per,p", RANDOM)
def test_reference_mask_matches_search(gpu, oracle_lib, dims, per, p):
    import mhdproj

    rng = np.random.default_rng(hash((dims, per)) & 0xFFFF)
    _check_reference(gpu, mhdproj, oracle_lib, dims, per, _solid_case(rng, dims, p))


@pytest.mark.parametrize("dims,per,p", RANDOM)
@pytest.mark.parametrize("outlet", [False, True])
def test_gauge_classes_match_search(gpu, oracle_lib, dims, per, p, outlet):
    import mhdproj

    if outlet and per & 4:
        pytest.skip("a top outlet needs a non-periodic z axis")
    rng = np.random.default_rng((hash((dims, per)) + 7) & 0xFFFF)
    _check_classes(gpu, mhdproj, oracle_lib, dims, per, _solid_case(rng, dims, p), outlet)


def test_known_answer_two_components(gpu, oracle_lib):
    """[1,0,1] on a 3x1x1 grid: two components, classes [2,0,2], roots 0 and 2
    (src/fluid/tests.rs:186-195)."""
    import mhdproj

    solid = np.array([0, 1, 0], np.uint8).reshape(1, 1, 3)
    pr = _run(gpu, mhdproj, (3, 1, 1), 0, solid, "reference")
    m, comps = pr.topology()
    assert comps == 2 and list(m & 3) == [2, 0, 2] and [int(m[0] >> 2), int(m[2] >> 2)] == [0, 2]
    pr.close()
    pr = _run(gpu, mhdproj, (3, 1, 1), 1, solid, "reference")
    assert pr.topology()[1] == 1  # periodic x joins the two cells
    pr.close()


@pytest.mark.parametrize("fill", [0, 1])
@pytest.mark.parametrize("dims", [(1, 1, 1), (40, 3, 5)])
def test_empty_and_full_masks(gpu, oracle_lib, fill, dims):
    import mhdproj

    solid = np.full((dims[2], dims[1], dims[0]), fill, np.uint8)
    for per in (0, 7):
        _check_reference(gpu, mhdproj, oracle_lib, dims, per, solid)
        _check_classes(gpu, mhdproj, oracle_lib, dims, per, solid, False)


def test_topology_change_between_calls(gpu, oracle_lib):
    """A changed solid mask relabels; an unchanged one keeps the labels."""
    import mhdproj

    torch = gpu
    dims = (48, 20, 12)
    rng = np.random.default_rng(5)
    a = _solid_case(rng, dims, 0.3)
    b = _solid_case(rng, dims, 0.4)
    pr = _run(torch, mhdproj, dims, 0, a, "reference")
    alpha = torch.ones(dims[2], dims[1], dims[0], dtype=torch.float32, device="cuda")
    for s in (b, b, a):
        pr.set_coefficients(alpha, torch.from_numpy(s).cuda(), 1000.0, 1000.0)
        got, comps = pr.topology()
        want_c, want = oracle_lib.anchors((s.reshape(-1) == 0).astype(np.uint32), list(dims), 0)
        assert comps == want_c
        np.testing.assert_array_equal(got, np.asarray(want, np.uint32))
    pr.close()


def test_jet256_geometry(gpu, oracle_lib):
    """Full-size labelling: the 256^3 jet's nozzle mask, both encodings."""
    import mhdproj

    c = synth.make_case("jet256")
    _check_classes(gpu, mhdproj, oracle_lib, c["dims"], 0, c["solid"], True)
    # a random mask at full size: many components in both solvers' encodings
    rng = np.random.default_rng(11)
    solid = _solid_case(rng, (256, 256, 256), 0.3)
    _check_reference(gpu, mhdproj, oracle_lib, (256, 256, 256), 0, solid)


def test_column512_dims_random_mask(gpu, oracle_lib):
    """The 512x256x256 grid of the large column workload (33.5 M cells, rows
    of 16 warp chunks), with a random mask near the percolation threshold."""
    import mhdproj

    rng = np.random.default_rng(13)
    dims = (512, 256, 256)
    solid = _solid_case(rng, dims, 0.31)
    _check_reference(gpu, mhdproj, oracle_lib, dims, 0, solid)
