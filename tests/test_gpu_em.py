"""GPU EM induction step (csrc/em_solver.cu, through the mhdproj_em_* C ABI)
against the FP32 oracle (oracle/oracle_em.c), bit for bit.

Every case runs the same seeded inputs through both and compares, after
each step, the solver's status record (rz, rr, bb, threshold, alpha, beta,
iterations, state), the 14 field statistics, the accepted reaction
potential on every edge and the 16 per-cell outputs (B, J, J x B, heat,
applied B) as raw FP32 bits.  Cases: a driven conducting ring (16^3 and
32^3, the latter with more than 256 reduction groups so the single-block
reductions take their 256-stride path), a non-cubic grid with partial cells
(bit-31 material encoding), a permeability contrast and a motional EMF, the
power-of-two residual rescale of a tiny source, the applied-field (vacuum)
mode, the homogeneous-conductor eigenmode of src/em/tests.rs:272-333 against
its backward-Euler decay, the air-stencil operator check of
tests.rs:665-738, the nodal gradient correction (from the first pass and
switched in mid-solve), the motional EMF from fluid cell records, a failing
solve's rollback and a bad material id.
"""
import math

import numpy as np
import pytest

import oracle as O
from test_oracle_em import SIGMA_316, MU0, _props, _ring, _uniform_applied

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _assert_bits(got, want, what):
    g, w = _bits(got), _bits(want)
    if not np.array_equal(g, w):
        bad = np.flatnonzero(g.reshape(-1) != w.reshape(-1))
        gi = np.asarray(got, np.float32).reshape(-1)
        wi = np.asarray(want, np.float32).reshape(-1)
        raise AssertionError(f"{what}: {bad.size} differ, first {bad[:5]}: got {gi[bad[:5]]} want {wi[bad[:5]]}")


class Pair:
    """The same EM problem in the library and in the oracle."""

    def __init__(self, torch, mhdproj, dims, h, materials, props, dt=1e-5, tol=1e-5, max_it=1000,
                 origin=(0.0, 0.0, 0.0), mode="induction", nodal_switch_after=1024):
        self.torch = torch
        self.gpu = mhdproj.EmInduction(dims, h, dt_s=dt, relative_tolerance=tol, max_iterations=max_it,
                                       origin_m=origin, mode=mode, nodal_switch_after=nodal_switch_after)
        self.cpu = O.EmSolve(dims, h, dt=dt, rel_tol=tol, max_iterations=max_it, origin=origin,
                             vacuum=(mode == "applied"), nodal_switch_after=nodal_switch_after)
        assert self.gpu.edges == self.cpu.edges and self.gpu.cells == self.cpu.cells
        self.m = np.ascontiguousarray(materials, np.uint32)
        self.props = np.ascontiguousarray(props, np.float32)

    def dev(self, a):
        return self.torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()

    def set_materials(self, expect_error=False):
        want = self.cpu.set_materials(self.m, self.props)
        t = self.torch.from_numpy(self.m.view(np.int32)).cuda()
        if expect_error:
            import mhdproj

            with pytest.raises(mhdproj.ProjectionError):
                self.gpu.set_materials(t, self.props)
            self.gpu._materials = t
        else:
            rng = self.gpu.set_materials(t, self.props)
            assert rng[1] == want[2]
        coef = self.gpu.copy("coefficients").cpu().numpy()
        src = self.cpu.source()
        E = self.cpu.edges
        _assert_bits(coef[:, 0], src[:E, 2], "edge conductivity")
        _assert_bits(coef[:, 1], src[:E, 3], "edge diagonal")
        flags = coef[:, 2].astype(np.uint32)
        np.testing.assert_array_equal(flags & 1, (src[E:, 1] > 0.5).astype(np.uint32))
        np.testing.assert_array_equal((flags >> 1) & 1, (src[E:, 2] > 0.5).astype(np.uint32))
        np.testing.assert_array_equal((flags >> 2) & 1, (src[E:, 3] > 0.5).astype(np.uint32))
        return want

    def step(self, time_s, initial=False, applied=None, label=""):
        rc, st, stats = self.cpu.advance(time_s, initial=initial, applied=applied)
        assert rc == self.cpu.OK, (label, rc, st)
        d = self.gpu.advance(time_s, initial=initial, applied=None if applied is None else self.dev(applied))
        _assert_bits(np.array(list(d.status), np.float32), st, f"{label} status")
        _assert_bits(d.stats()[:14], stats[:14], f"{label} field statistics")
        _assert_bits(self.gpu.copy("reaction").cpu().numpy(), self.cpu.reaction(), f"{label} reaction potential")
        _assert_bits(self.gpu.copy("previous").cpu().numpy(), self.cpu.previous(), f"{label} previous potential")
        _assert_bits(self.gpu.copy("cells").cpu().numpy(), self.cpu.results(), f"{label} cell fields")
        return d, st, stats

    def close(self):
        self.gpu.close()
        self.cpu.close()


def _driven_pair(torch, mhdproj, n, sigma_scale=40.0, scale=1.0, max_it=1000, nodal_switch_after=1024):
    h = 1e-3
    origin = (-0.5 * n * h,) * 3
    pair = Pair(torch, mhdproj, (n, n, n), h, _ring(n, inner=0.19 * n, outer=0.38 * n, z0=n // 3, z1=n - n // 3),
                _props(SIGMA_316 * sigma_scale, 1.0), max_it=max_it, origin=origin,
                nodal_switch_after=nodal_switch_after)
    b = (np.float32(0.0), np.float32(0.0), np.float32(0.02))
    applied = lambda t: _uniform_applied(pair.cpu, h, origin, b, scale=scale * math.sin(2 * math.pi * 1e3 * t))
    return pair, applied


@pytest.mark.parametrize("n", [16, 32])
def test_driven_ring_bit_exact(gpu, n):
    import mhdproj

    pair, applied = _driven_pair(gpu, mhdproj, n)
    check = pair.set_materials()
    assert check[0] == 0 and check[3] > 0
    pair.step(0.0, initial=True, applied=applied(0.0), label="initial")
    t = 0.0
    for k in range(5):
        t += 1e-5
        d, st, _ = pair.step(t, applied=applied(t), label=f"step {k}")
        assert d.iterations > 0 and st[7] == 1.0
    # a held field (no new applied potential): hold_source
    d, _, _ = pair.step(t + 1e-5, applied=None, label="held")
    assert d.maxima[1] > 0.0  # the eddy currents decay but still flow
    pair.close()


def test_partial_cells_permeability_and_motional_emf(gpu):
    import mhdproj

    dims, h = (20, 14, 11), 5e-4
    rng = np.random.default_rng(7)
    m = np.zeros((dims[2], dims[1], dims[0]), np.uint32)
    m[3:8, 3:11, 4:16] = 2
    m[4:7, 5:9, 6:14] = 3
    # partial cells: fraction in bits 8..30 of material 2 on the block's skin
    frac = rng.integers(1, 0x7FFFFF, size=(dims[2], dims[1], dims[0]), dtype=np.uint32)
    skin = np.zeros_like(m, bool)
    skin[2:9, 2:12, 3:17] = True
    skin[3:8, 3:11, 4:16] = False
    m[skin] = 0x80000000 | (frac[skin] << 8) | 2
    props = np.array([[0.0, 1.0], [0.0, 1.0], [3.0e7, 1.0], [1.0e6, 2.5]], np.float32)
    origin = (-5e-3, -3.5e-3, -2.75e-3)
    pair = Pair(gpu, mhdproj, dims, h, m.reshape(-1), props, dt=2e-5, origin=origin, max_it=800)
    pair.set_materials()
    b = (np.float32(0.004), np.float32(-0.003), np.float32(0.01))
    applied = lambda t: _uniform_applied(pair.cpu, h, origin, b, scale=math.cos(2 * math.pi * 700 * t))
    pair.step(0.0, initial=True, applied=applied(0.0), label="initial")
    emf = (rng.standard_normal(pair.cpu.edges) * 1e-3).astype(np.float32)
    pair.cpu.set_motional(emf)
    pair.gpu.set_motional_emf(pair.dev(emf))
    t = 0.0
    for k in range(4):
        t += 2e-5 if k != 2 else 3e-5  # an uneven step: prediction ratio 1.5
        pair.step(t, applied=applied(t), label=f"step {k}")
    pair.close()


def test_tiny_source_rescale_bit_exact(gpu):
    import mhdproj

    pair, applied = _driven_pair(gpu, mhdproj, 16, scale=2.0 ** -30)
    pair.set_materials()
    pair.step(0.0, initial=True, applied=applied(0.0), label="initial")
    pair.step(1e-5, applied=applied(1e-5), label="rescaled")
    sc = pair.cpu.scalars()
    assert sc[24] != 1.0 and sc[24] > 0.0
    pair.close()


def test_applied_mode_bit_exact(gpu):
    import mhdproj

    n, h = 16, 1e-3
    origin = (-8e-3,) * 3
    pair = Pair(gpu, mhdproj, (n, n, n), h, _ring(n), _props(), origin=origin, mode="applied")
    pair.set_materials()
    b = (np.float32(0.003), np.float32(-0.004), np.float32(0.005))
    d, _, _ = pair.step(0.0, initial=True, applied=_uniform_applied(pair.cpu, h, origin, b), label="applied")
    cells = pair.gpu.copy("cells").cpu().numpy().reshape(n, n, n, 16)
    for k, want in enumerate(b):
        assert abs(float(cells[8, 8, 8, k]) - float(want)) < 1e-7
    with pytest.raises(mhdproj.ProjectionError):
        pair.gpu.advance(1e-5, initial=False)  # applied mode only evaluates initial solves
    pair.close()


def test_eigenmode_decay_bit_exact(gpu):
    """src/em/tests.rs:272-333 on the GPU: the homogeneous conductor fills
    the box (the material update reports it touching the boundary, as the
    reference does; the test proceeds as the reference's test does)."""
    import mhdproj

    n, h = 16, 1e-3
    total, steps = 2e-5, 2
    dt = total / steps
    pair = Pair(gpu, mhdproj, (n, n, n), h, np.full(n ** 3, 6, np.uint32), _props(), dt=dt, max_it=1000)
    pair.set_materials(expect_error=True)
    pair.step(0.0, initial=True, label="initial")
    initial = np.zeros(pair.cpu.edges, np.float32)
    for z in range(n + 1):
        for y in range(n + 1):
            initial[n * (y + (n + 1) * z):n * (y + (n + 1) * z) + n] = (
                np.float32(1e-5) * np.float32(math.sin(math.pi * y / n)) * np.float32(math.sin(math.pi * z / n)))
    pair.cpu.set_reaction(initial)
    pair.gpu.set_reaction(pair.dev(initial))
    t = 0.0
    for k in range(steps):
        t += dt
        pair.step(t, label=f"step {k}")
    lam = 8 * math.sin(math.pi / (2 * n)) ** 2
    centre = n // 2 + n * ((n // 2) + (n + 1) * (n // 2))
    ratio = float(pair.gpu.copy("reaction").cpu().numpy()[centre]) / float(initial[centre])
    expected = (1.0 / (1.0 + lam * dt / (MU0 * float(SIGMA_316) * h * h))) ** steps
    assert abs(ratio - expected) < 2e-5
    pair.close()


@pytest.mark.parametrize("sigma,mu", [(0.0, 1.0), (1.33e6, 1.0), (0.0, 2.0)])
def test_air_stencil_operator(gpu, sigma, mu):
    import mhdproj

    n = 16
    pair = Pair(gpu, mhdproj, (n, n, n), 1e-3, _ring(n), _props(sigma, mu))
    pair.set_materials()
    E = pair.cpu.edges
    i = np.arange(E, dtype=np.float32)
    p = ((np.sin(i * np.float32(1.2345)) + np.cos(i * np.float32(0.345))) * np.float32(0.01)).astype(np.float32)
    fast = pair.gpu.apply_operator(pair.dev(p), air_stencil=True).cpu().numpy()
    exact = pair.gpu.apply_operator(pair.dev(p), air_stencil=False).cpu().numpy()
    _assert_bits(fast, pair.cpu.apply_operator(p, use_air=True), "air stencil operator")
    _assert_bits(exact, pair.cpu.apply_operator(p, use_air=False), "full operator")
    f64, e64 = fast.astype(np.float64), exact.astype(np.float64)
    assert math.sqrt(((f64 - e64) ** 2).sum() / (e64 ** 2).sum()) < 2e-7
    pair.close()


def test_failed_step_rolls_back(gpu):
    import mhdproj

    pair, applied = _driven_pair(gpu, mhdproj, 16, max_it=2)
    pair.set_materials()
    pair.step(0.0, initial=True, applied=applied(0.0), label="initial")
    before = pair.gpu.copy("reaction").cpu().numpy()
    src = pair.gpu.copy("applied").cpu().numpy()
    with pytest.raises(mhdproj.ProjectionError) as e:
        pair.gpu.advance(1e-5, applied=pair.dev(applied(1e-5)))
    assert e.value.code == 3 and "did not converge" in str(e.value)
    _assert_bits(pair.gpu.copy("reaction").cpu().numpy(), before, "restored reaction")
    _assert_bits(pair.gpu.copy("applied").cpu().numpy(), src, "restored applied potential")
    pair.close()


def test_bad_material_id_is_rejected(gpu):
    import mhdproj

    em = mhdproj.EmInduction((8, 8, 8), 1e-3)
    m = np.zeros(512, np.int32)
    m[100] = 9
    with pytest.raises(mhdproj.ProjectionError) as e:
        em.set_materials(gpu.from_numpy(m).cuda(), _props())
    assert e.value.code == 1
    with pytest.raises(mhdproj.ProjectionError):
        mhdproj.EmInduction((0, 8, 8), 1e-3)
    em.close()


def test_motional_emf_from_fluid_cells_bit_exact(gpu):
    """EmState::set_velocity: the motional EMF from FluidCell records and the
    last B (motion.wgsl), then a step driven by it."""
    import mhdproj

    pair, applied = _driven_pair(gpu, mhdproj, 16)
    pair.set_materials()
    pair.step(0.0, initial=True, applied=applied(0.0), label="initial")
    pair.step(1e-5, applied=applied(1e-5), label="step 0")
    rng = np.random.default_rng(21)
    fluid = rng.standard_normal((pair.cpu.cells, 16)).astype(np.float32)
    fluid[:, 12] = (rng.random(pair.cpu.cells) < 0.6).astype(np.float32)
    pair.cpu.set_motion(fluid)
    pair.gpu.set_motion(pair.dev(fluid))
    E = pair.cpu.edges
    _assert_bits(pair.gpu.copy("coefficients").cpu().numpy()[:, 3], pair.cpu.source()[E:, 0], "motional EMF")
    pair.step(2e-5, applied=applied(2e-5), label="with motion")
    pair.close()


@pytest.mark.parametrize("n,after", [(16, 0), (32, 16)])
def test_nodal_correction_bit_exact(gpu, n, after):
    """The nodal gradient correction from the first pass, and switched in
    after the first 32-iteration batch at a true-residual restart."""
    import mhdproj

    pair, applied = _driven_pair(gpu, mhdproj, n, nodal_switch_after=after)
    pair.set_materials()
    pair.step(0.0, initial=True, applied=applied(0.0), label="initial")
    t = 0.0
    for k in range(3):
        t += 1e-5
        d, st, _ = pair.step(t, applied=applied(t), label=f"nodal step {k}")
        assert st[7] == 1.0
    pair.close()


def test_source_pass_against_oracle(gpu):
    """mhdproj_em_evaluate_sources (source.wgsl) against the oracle: the
    surface-current and uniform kinds use no logarithm and match bit for bit;
    wire segments call CUDA's logf, so they are held to a relative L2 error of
    1e-5 and a max error of 1e-5 of the largest value.  The GPU potential
    then drives a bit-exact step on both sides."""
    import mhdproj
    from mhdproj import synth

    n, h = 20, 0.5e-3
    origin = (-0.5 * n * h,) * 3
    pair = Pair(gpu, mhdproj, (n, n, n), h, _ring(n, inner=3.0, outer=6.0, z0=7, z1=13),
                _props(SIGMA_316 * 40, 1.0), origin=origin)
    pair.set_materials()
    block = synth.em_magnet_block_elements(1.5e-3, 1.0e-3, 1.0e-3, 5e5, 5, smoothing=1e-4)
    uni = synth.em_uniform_element((0.01, -0.02, 0.03), 0.5)
    dead = synth.em_uniform_element((1.0, 1.0, 1.0), 0.0)
    exact = np.concatenate([block, dead, uni, block[:7]])
    _assert_bits(pair.gpu.evaluate_sources(exact).cpu().numpy(), pair.cpu.evaluate_sources(exact),
                 "surface-current and uniform sources")
    loop = synth.em_loop_elements(3.5e-3, 50.0, 45, centre=(0.0, 0.0, 1e-3), core=2e-4)
    wires = np.concatenate([loop, exact[:40], loop[:13]])
    g = pair.gpu.evaluate_sources(wires).cpu().numpy().astype(np.float64)
    c = pair.cpu.evaluate_sources(wires).astype(np.float64)
    assert np.linalg.norm(g - c) <= 1e-5 * np.linalg.norm(c)
    assert np.abs(g - c).max() <= 1e-5 * np.abs(c).max()
    empty = pair.gpu.evaluate_sources(np.zeros((0, 12), np.float32)).cpu().numpy()
    assert not empty.any()
    a = g.astype(np.float32)
    pair.step(0.0, initial=True, applied=a * np.float32(0.0), label="initial")
    pair.step(1e-5, applied=a, label="driven by the GPU source pass")
    pair.close()


def test_body_forces_bit_exact(gpu):
    """mhdproj_em_body_forces (body-stats.wgsl) for three overlapping bodies."""
    import mhdproj

    pair, applied = _driven_pair(gpu, mhdproj, 32)
    pair.set_materials()
    pair.step(0.0, initial=True, applied=applied(0.0), label="initial")
    pair.step(1e-5, applied=applied(1e-5), label="step")
    rng = np.random.default_rng(17)
    masks = rng.integers(0, 8, pair.cpu.cells).astype(np.uint32)
    got = pair.gpu.body_forces(gpu.from_numpy(masks.view(np.int32)).cuda(), 3)
    _assert_bits(got, pair.cpu.body_forces(masks, 3), "body force and power")
    with pytest.raises(mhdproj.ProjectionError):
        pair.gpu.body_forces(gpu.from_numpy(masks.view(np.int32)).cuda(), 33)
    pair.close()


def test_energy_ledger_bit_exact(gpu):
    """mhdproj_em_energy (energy.wgsl) equals the oracle's ledger bit for bit
    after each driven step, and the ledger closes (src/em/tests.rs:633-663)."""
    import mhdproj

    n, h = 20, 0.8e-3
    origin = (-8e-3,) * 3
    pair = Pair(gpu, mhdproj, (n, n, n), h, _ring(n, inner=3.0, outer=7.0, z0=7, z1=13), _props(), origin=origin)
    pair.set_materials()
    b = (np.float32(0.0), np.float32(0.0), np.float32(0.01))
    applied = lambda t: _uniform_applied(pair.cpu, h, origin, b, scale=math.sin(2 * math.pi * 1e3 * t))
    pair.step(0.0, initial=True, applied=applied(0.0), label="initial")
    assert pair.gpu.energy() == pair.cpu.energy()
    t = 0.0
    for k in range(3):
        t += 1e-5
        pair.step(t, applied=applied(t), label=f"step {k}")
        g, c = pair.gpu.energy(), pair.cpu.energy()
        assert g == c, (g, c)
        scale = abs(g["external_j"]) + abs(g["delta_magnetic_j"]) + g["joule_j"] + g["backward_euler_j"]
        assert abs(g["balance_error_j"]) / scale < 1e-4
    pair.close()
