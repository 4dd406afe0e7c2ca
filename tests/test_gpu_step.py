"""GPU parity of the fluid step and the fields/diagnostics export.

FluidState::step (src/fluid/mod.rs:1246-1333) without a moving interface:
predict (semi-Lagrangian RK2 advection, src/fluid/solver.wgsl:127-141),
viscous (explicit viscosity, body and EM force, mobility, :143-163), the
warm-started projection, then fields and diagnostics (:256-291).  With the
reference solver every stage restates the reference in FP32 without fused
multiply-adds, so the GPU step is compared bit for bit with the oracle's
restatement chained the same way: velocity, pressure, the 16-float cell
records and the diagnostics, over several steps.  The GB300 solver's step is
checked stage by stage: its predict/viscous output projected by a second
context equals the step's result bit for bit, and its fields match the
oracle's on the same velocity and potential.
"""
import numpy as np
import pytest

import refcases as R

pytestmark = pytest.mark.gpu

bits = lambda a: np.asarray(a, np.float32).view(np.uint32)


def single_phase(c, dt):
    c = dict(c)
    c["two_phase"] = False
    c["rho_air"] = c["rho_liquid"]
    c["dt"] = dt
    return c


def oracle_step(oracle, c, vel, old_p, nu, acc, advection, em=None, phase=None, drag_rate=1e6):
    """One step on the oracle: predict, viscous, warm projection, fields."""
    dims = c["dims"]
    n = dims[0] * dims[1] * dims[2]
    mask01 = (np.asarray(c["solid"]).reshape(-1) == 0).astype(np.uint32)
    comps, mask = oracle.anchors(mask01, dims, c["periodic"])
    fluid = int((mask != 0).sum())
    occ = np.asarray(c["alpha"], np.float32).reshape(-1)
    p = oracle.make_params(dims, c["h"], c["dt"], c["rho_liquid"], c["rho_air"], False, c["periodic"],
                           c["rel_tol"], c["abs_div_tol"], fluid, phase is not None, drag_rate)
    p.physical[2] = nu
    p.flags[1] = int(advection)
    em_rec = None if em is None else np.asarray(em, np.float32).reshape(n, 4)
    ph = None if phase is None else np.asarray(phase, np.float32).reshape(-1)
    pred = oracle.predict(p, mask, R.soa_to_records(dims, *vel))
    visc = oracle.viscous(p, mask, occ, pred, acc, em=em_rec, phase=ph)
    ref = R.run_oracle(oracle, c, preconditioner=c.get("pre", "auto"), warm_start=True,
                       old_pressure=np.zeros(n, np.float32) if old_p is None else old_p,
                       u=R.records_to_soa(dims, visc), phase=ph, drag_rate=drag_rate)
    assert ref["result"].status == 0
    reserved = np.zeros((n, 4), np.float32)
    reserved[:, 1] = 0.0 if ph is None else ph
    reserved[:, 2] = occ
    cells, sc = oracle.fields(ref["params"], mask, occ, ref["work"],
                              R.soa_to_records(dims, ref["u"], ref["v"], ref["w"]), acc, em=em_rec,
                              reserved=reserved)
    return ref, cells, sc, visc


def diag_from_scalars(sc, c, fluid):
    h = np.float32(c["h"])
    h3 = h * h * h
    return dict(max_speed_m_s=sc[0], max_divergence_s_inv=sc[1],
                rms_divergence_s_inv=np.sqrt(np.float32(sc[2]) / np.float32(max(fluid, 1))),
                kinetic_energy_j=sc[3], fluid_mass_kg=np.float32(c["rho_liquid"]) * np.float32(sc[9]) * h3,
                max_pressure_pa=sc[4], net_flux_m3_s=np.float32(sc[5]) * h3, max_force_density=sc[6],
                max_face_speed_m_s=sc[8])


def make_ref_ctx(mhdproj, torch, c, preconditioner):
    per = tuple(bool(c["periodic"] & (1 << a)) for a in range(3))
    pr = mhdproj.PressureProjection(c["dims"], c["h"], periodic=per, outlet=False, solver="reference",
                                    preconditioner=preconditioner, rel_tol=c["rel_tol"],
                                    abs_div_tol=c["abs_div_tol"], two_phase=False, max_iterations=20000)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pr.set_coefficients(t(c["alpha"]), t(c["solid"]), c["rho_liquid"], c["rho_air"])
    return pr


STEP_CASES = [
    # name, case, preconditioner, steps, viscosity, advection, EM force
    ("walls17x13x9", lambda: R.wall_case((17, 13, 9), (0, 0, 0), True, False), "jacobi", 3, 0.1, True, True),
    ("walls16x12x8_periodic", lambda: R.wall_case((16, 12, 8), (1, 1, 0), True, True), "multigrid", 2, 0.05, True,
     False),
    ("cosine16_meanfree", lambda: R.cosine_case(), "jacobi", 2, 0.0, False, False),
]


@pytest.mark.parametrize("name,make_case,pre,steps,nu,adv,use_em", STEP_CASES)
def test_reference_step_bit_exact(gpu, oracle_lib, name, make_case, pre, steps, nu, adv, use_em):
    import mhdproj

    torch = gpu
    c = single_phase(make_case(), dt=0.02 if c_is_walls(name) else 5e-4)
    c["pre"] = pre
    dims = c["dims"]
    nx, ny, nz = dims
    n = nx * ny * nz
    rng = np.random.default_rng(17)
    em = (rng.standard_normal((nz, ny, nx, 4)) * 50.0 * c["rho_liquid"] * (1.0 if use_em else 0.0)).astype(
        np.float32) if use_em else None
    acc = np.array([0.3, -0.2, -9.81], np.float32)
    pr = make_ref_ctx(mhdproj, torch, c, pre)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    u = [t(c["u"]), t(c["v"]), t(c["w"])]
    em_t = None if em is None else t(em)
    p_out = torch.zeros((nz, ny, nx), dtype=torch.float32, device="cuda")
    cells = torch.zeros((nz, ny, nx, 16), dtype=torch.float32, device="cuda")
    vel = (c["u"], c["v"], c["w"])
    old_p = None
    fluid = int((np.asarray(c["solid"]).reshape(-1) == 0).sum())
    for k in range(steps):
        st, d = pr.fluid_step(u, c["dt"], acceleration=tuple(acc), viscosity=nu, advection=adv, em_force=em_t,
                              p_out=p_out, cells=cells)
        torch.cuda.synchronize()
        ref, ocells, sc, _ = oracle_step(oracle_lib, c, vel, old_p, nu, acc, adv, em=em)
        assert st["iterations"] == ref["result"].iterations, k
        for a, key in enumerate("uvw"):
            assert np.array_equal(bits(u[a].cpu().numpy()), bits(ref[key])), (k, key)
        assert np.array_equal(bits(p_out.cpu().numpy().reshape(-1)), bits(ref["p"])), k
        assert np.array_equal(bits(cells.cpu().numpy().reshape(n, 16)), bits(ocells)), k
        want = diag_from_scalars(sc, c, fluid)
        for key, val in want.items():
            assert np.float32(d[key]) == np.float32(val), (k, key, d[key], val)
        assert d["nonfinite_cells"] == 0
        vel = (ref["u"], ref["v"], ref["w"])
        old_p = ref["p"]
    pr.close()


def c_is_walls(name):
    return name.startswith("walls")


def test_reference_step_phase_drag(gpu, oracle_lib):
    """The step's viscous mobility with thermal mushy-zone drag (solver.wgsl:43-51)."""
    import mhdproj

    torch = gpu
    c = single_phase(R.wall_case((17, 13, 9), (0, 0, 0), True, False), dt=0.02)
    c["pre"] = "jacobi"
    rng = np.random.default_rng(5)
    phase = rng.uniform(0.2, 1.0, c["alpha"].shape).astype(np.float32)
    pr = make_ref_ctx(mhdproj, torch, c, "jacobi")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pr.set_phase_drag(t(phase), 1e3, c["dt"])
    u = [t(c["u"]), t(c["v"]), t(c["w"])]
    acc = np.array([0.0, 0.0, -9.81], np.float32)
    st, d = pr.fluid_step(u, c["dt"], acceleration=tuple(acc), viscosity=0.02, advection=True)
    ref, _, sc, _ = oracle_step(oracle_lib, c, (c["u"], c["v"], c["w"]), None, 0.02, acc, True, phase=phase,
                                drag_rate=1e3)
    for a, key in enumerate("uvw"):
        assert np.array_equal(bits(u[a].cpu().numpy()), bits(ref[key])), key
    assert np.float32(d["kinetic_energy_j"]) == np.float32(sc[3])
    pr.close()


def test_step_cfl_error_restores_velocity(gpu, oracle_lib):
    """A timestep beyond the velocity CFL limit is refused with the
    reference's message and the velocity is left as given."""
    import mhdproj

    torch = gpu
    c = single_phase(R.wall_case((17, 13, 9), (0, 0, 0), True, False), dt=0.02)
    pr = make_ref_ctx(mhdproj, torch, c, "jacobi")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    u = [t(c["u"]), t(c["v"]), t(c["w"])]
    before = [a.clone() for a in u]
    with pytest.raises(mhdproj.ProjectionError) as e:
        pr.fluid_step(u, 5.0, acceleration=(0.0, 0.0, -9.81), viscosity=0.0, advection=True)
    assert "Fluid timestep exceeds the velocity CFL limit; reduce" in str(e.value)
    for a, b in zip(u, before):
        assert torch.equal(a, b)
    pr.close()


def test_step_nonconvergence_rolls_back(gpu, oracle_lib):
    """A projection that fails inside the step restores the velocity."""
    import mhdproj

    torch = gpu
    c = single_phase(R.wall_case((16, 12, 8), (0, 0, 1), True, False), dt=0.02)
    per = tuple(bool(c["periodic"] & (1 << a)) for a in range(3))
    pr = mhdproj.PressureProjection(c["dims"], c["h"], periodic=per, outlet=False, solver="reference",
                                    preconditioner="jacobi", rel_tol=1e-7, abs_div_tol=0.0, two_phase=False,
                                    max_iterations=3)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pr.set_coefficients(t(c["alpha"]), t(c["solid"]), c["rho_liquid"], c["rho_air"])
    u = [t(c["u"]), t(c["v"]), t(c["w"])]
    before = [a.clone() for a in u]
    with pytest.raises(mhdproj.ProjectionError) as e:
        pr.fluid_step(u, c["dt"], acceleration=(0.0, 0.0, -9.81), viscosity=0.0, advection=True)
    assert "did not converge" in str(e.value)
    for a, b in zip(u, before):
        assert torch.equal(a, b)
    pr.close()


def test_fields_two_phase_reference(gpu, oracle_lib):
    """fields + diagnostics after a two-phase projection: density-weighted
    kinetic energy, reserved lanes, mean-free or pinned pressure."""
    import mhdproj

    torch = gpu
    c = R.wall_case((17, 13, 9), (0, 0, 0), True, False)
    per = tuple(bool(c["periodic"] & (1 << a)) for a in range(3))
    pr = mhdproj.PressureProjection(c["dims"], c["h"], periodic=per, outlet=False, solver="reference",
                                    preconditioner="jacobi", rel_tol=c["rel_tol"], abs_div_tol=c["abs_div_tol"],
                                    two_phase=True)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pr.set_coefficients(t(c["alpha"]), t(c["solid"]), c["rho_liquid"], c["rho_air"])
    (uo, vo, wo), _, _ = pr.project((t(c["u"]), t(c["v"]), t(c["w"])), c["dt"])
    acc = np.array([0.0, 0.0, -9.81], np.float32)
    cells, d = pr.fields((uo, vo, wo), c["dt"], acceleration=tuple(acc))
    ref = R.run_oracle(oracle_lib, c, preconditioner="jacobi")
    dims = c["dims"]
    n = dims[0] * dims[1] * dims[2]
    occ = np.asarray(c["alpha"], np.float32).reshape(-1)
    reserved = np.zeros((n, 4), np.float32)
    reserved[:, 2] = occ
    ocells, sc = oracle_lib.fields(ref["params"], ref["mask"], occ, ref["work"],
                                   R.soa_to_records(dims, ref["u"], ref["v"], ref["w"]), acc, reserved=reserved)
    assert np.array_equal(bits(cells.cpu().numpy().reshape(n, 16)), bits(ocells))
    assert np.float32(d["kinetic_energy_j"]) == np.float32(sc[3])
    assert np.float32(d["max_pressure_pa"]) == np.float32(sc[4])
    pr.close()


def test_gb300_step_stages(gpu, oracle_lib):
    """GB300 solver: the step equals the oracle's predict + viscous projected
    by a second context with a warm start, bit for bit; its fields equal the
    oracle's on the same velocity and potential (pressure to 1e-6)."""
    import mhdproj
    from mhdproj import synth

    torch = gpu
    c = synth.make_case("jet64", scale=0.5)  # 32^3 nozzle, single phase, top outlet
    dims = c["dims"]
    nx, ny, nz = dims
    n = nx * ny * nz
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    dt = 2e-5
    acc = np.array([0.0, 0.0, -9.81], np.float32)
    nu = 1e-6

    def ctx():
        pr = mhdproj.PressureProjection(dims, c["h"], outlet=True, precision="fp32", rel_tol=1e-8)
        pr.set_coefficients(t(c["alpha"]), t(c["solid"]), c["rho_liquid"], c["rho_liquid"])
        return pr

    a, b = ctx(), ctx()
    u = [t(c["u"]), t(c["v"]), t(c["w"])]
    st, d = a.fluid_step(u, dt, acceleration=tuple(acc), viscosity=nu, advection=True)
    # the same stages on the oracle, projected by context b
    g = oracle_lib.grid(nx, ny, nz, c["h"], c["rho_liquid"], c["rho_liquid"], 0, True)
    _, cls = oracle_lib.classify(g, c["solid"])
    mask = (cls != 0).astype(np.uint32)
    p = oracle_lib.make_params(dims, c["h"], dt, c["rho_liquid"], c["rho_liquid"], False, 0, 1e-5, 0.0,
                               int(mask.sum()), False, 1e6)
    p.physical[2] = nu
    p.flags[1] = 1
    pred = oracle_lib.predict(p, mask, R.soa_to_records(dims, c["u"], c["v"], c["w"]))
    visc = oracle_lib.viscous(p, mask, np.asarray(c["alpha"], np.float32).reshape(-1), pred, acc)
    (ub, vb, wb), _, _ = b.project(tuple(t(x) for x in R.records_to_soa(dims, visc)), dt, warm_start=True)
    for x, y in zip(u, (ub, vb, wb)):
        assert torch.equal(x, y)
    # fields of the projected velocity with b's potential
    cells, db = b.fields((ub, vb, wb), dt, acceleration=tuple(acc))
    phi = torch.empty(n, dtype=torch.float64, device="cuda")
    b._check(b._lib.mhdproj_copy_potential(b._ctx, mhdproj._ptr(phi)))
    work = np.zeros((n, 4), np.float32)
    work[:, 0] = phi.cpu().numpy().astype(np.float32)
    reserved = np.zeros((n, 4), np.float32)
    reserved[:, 2] = np.asarray(c["alpha"], np.float32).reshape(-1)
    ocells, sc = oracle_lib.fields(p, mask, np.asarray(c["alpha"], np.float32).reshape(-1), work,
                                   R.soa_to_records(dims, ub.cpu().numpy(), vb.cpu().numpy(), wb.cpu().numpy()),
                                   acc, reserved=reserved)
    got = cells.cpu().numpy().reshape(n, 16)
    same = [0, 1, 2, 3, 5, 8, 9, 10, 12, 13, 14, 15]
    assert np.array_equal(bits(got[:, same]), bits(ocells[:, same]))
    np.testing.assert_allclose(got[:, 4], ocells[:, 4], rtol=1e-6, atol=1e-6 * np.abs(ocells[:, 4]).max())
    assert np.float32(db["kinetic_energy_j"]) == np.float32(sc[3])
    assert d["max_divergence_s_inv"] == db["max_divergence_s_inv"]
    a.close()
    b.close()


def test_gb300_step_periodic_pinned(gpu, oracle_lib):
    """GB300 solver on a periodic x-y domain without an outlet (pinned gauge
    cells): the step equals the oracle's predict + viscous projected by a
    second context, bit for bit, over two chained steps."""
    import mhdproj
    from mhdproj import synth

    torch = gpu
    c = synth.make_case("jet128", scale=0.25)  # 32^3 nozzle geometry
    dims = c["dims"]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    dt, nu = 1e-5, 1e-6
    acc = np.array([0.5, 0.0, -9.81], np.float32)

    def ctx():
        pr = mhdproj.PressureProjection(dims, c["h"], periodic=(True, True, False), outlet=False, precision="fp16",
                                        rel_tol=1e-8)
        pr.set_coefficients(t(c["alpha"]), t(c["solid"]), c["rho_liquid"], c["rho_liquid"])
        return pr

    a, b = ctx(), ctx()
    u = [t(c["u"]), t(c["v"]), t(c["w"])]
    ub = [x.clone() for x in u]
    g = oracle_lib.grid(dims[0], dims[1], dims[2], c["h"], c["rho_liquid"], c["rho_liquid"], 3, False)
    _, cls = oracle_lib.classify(g, c["solid"])
    mask = (cls != 0).astype(np.uint32)
    p = oracle_lib.make_params(dims, c["h"], dt, c["rho_liquid"], c["rho_liquid"], False, 3, 1e-5, 0.0,
                               int(mask.sum()), False, 1e6)
    p.physical[2] = nu
    p.flags[1] = 1
    for k in range(2):
        a.fluid_step(u, dt, acceleration=tuple(acc), viscosity=nu, advection=True)
        pred = oracle_lib.predict(p, mask, R.soa_to_records(dims, *(x.cpu().numpy() for x in ub)))
        visc = oracle_lib.viscous(p, mask, np.asarray(c["alpha"], np.float32).reshape(-1), pred, acc)
        (u0, u1, u2), _, _ = b.project(tuple(t(x) for x in R.records_to_soa(dims, visc)), dt, warm_start=True)
        ub = [u0, u1, u2]
        for x, y in zip(u, ub):
            assert torch.equal(x, y), k
    a.close()
    b.close()


def interface_case(seed=4):
    """A 17x13x9 two-phase box of 1 mm cells: liquid fraction uniform in
    [0, 1] (interface cells everywhere), a solid wall at x = 8 with the gap
    cell (1, 1), 1000:1.2 densities, velocities N(0, 0.01 m/s), curvature
    N(0, 200 1/m)."""
    c = R.wall_case((17, 13, 9), (0, 0, 0), True, False, seed=seed)
    rng = np.random.default_rng(seed)
    c = dict(c)
    c["h"] = 1e-3
    c["rho_liquid"], c["rho_air"] = 1000.0, 1.2
    c["two_phase"] = True
    c["alpha"] = rng.uniform(0.0, 1.0, c["alpha"].shape).astype(np.float32)
    for k in "uvw":
        c[k] = (0.01 * c[k]).astype(np.float32)
    c["curvature"] = rng.normal(0.0, 200.0, c["alpha"].shape).astype(np.float32)
    c["dt"] = 1e-4
    c["rel_tol"], c["abs_div_tol"] = 1e-5, 1e-5
    return c


INTERFACE_CASES = [
    # air viscosity, expected substep path: host bound (1 Euler), GPU bound with Euler substeps, RKC stages
    ("host_bound", 1e-6, 1e-7),
    ("euler", 4e-2, 1e-6),
    ("rkc", 0.2, 1e-6),
]


@pytest.mark.parametrize("name,mu_air,nu", INTERFACE_CASES)
def test_reference_interface_step_bit_exact(gpu, oracle_lib, name, mu_air, nu):
    """The moving-interface step (no advection here, capillary force, stress
    diffusion by Euler substeps or RKC2 stages, face densities) on the
    reference solver equals the oracle's chain bit for bit over two steps."""
    import mhdproj

    torch = gpu
    c = interface_case()
    dims = c["dims"]
    nx, ny, nz = dims
    n = nx * ny * nz
    sigma = 0.07
    acc = np.array([0.0, 0.0, -9.81], np.float32)
    per = tuple(bool(c["periodic"] & (1 << a)) for a in range(3))
    pr = mhdproj.PressureProjection(dims, c["h"], periodic=per, outlet=False, solver="reference",
                                    preconditioner="jacobi", rel_tol=c["rel_tol"], abs_div_tol=c["abs_div_tol"],
                                    two_phase=True, max_iterations=20000)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pr.set_coefficients(t(c["alpha"]), t(c["solid"]), c["rho_liquid"], c["rho_air"])
    u = [t(c["u"]), t(c["v"]), t(c["w"])]
    curv = t(c["curvature"])
    cells = torch.zeros((nz, ny, nx, 16), dtype=torch.float32, device="cuda")
    p_out = torch.zeros((nz, ny, nx), dtype=torch.float32, device="cuda")
    mask01 = (np.asarray(c["solid"]).reshape(-1) == 0).astype(np.uint32)
    comps, mask = oracle_lib.anchors(mask01, dims, 0)
    fluid = int((mask != 0).sum())
    occ = np.asarray(c["alpha"], np.float32).reshape(-1)
    vel = (c["u"], c["v"], c["w"])
    old_p = np.zeros(n, np.float32)
    paths = set()
    for k in range(2):
        st, d = pr.fluid_step(u, c["dt"], acceleration=tuple(acc), viscosity=nu, advection=True, p_out=p_out,
                              cells=cells, surface_tension=sigma, air_viscosity=mu_air, curvature=curv)
        torch.cuda.synchronize()
        prm = oracle_lib.make_params(dims, c["h"], c["dt"], c["rho_liquid"], c["rho_air"], True, 0, c["rel_tol"],
                                     c["abs_div_tol"], fluid, False, 1e6)
        prm.physical[2] = nu
        prm.flags[1] = 0  # the interface transport advects the momentum
        rec = R.soa_to_records(dims, *vel)
        pred = oracle_lib.predict(prm, mask, rec)
        status, sub, gbound, pred = oracle_lib.diffuse_surface_stress(prm, mask, occ, pred, rec, mu_air, c["dt"])
        assert status == 0
        paths.add("host" if gbound < 0 else ("rkc" if sub > 0 and gbound * c["dt"] / 1.8 > 8 else "euler"))
        assert d["viscous_substeps"] == sub, (k, d["viscous_substeps"], sub)
        visc = oracle_lib.viscous_surface(prm, mask, occ, pred, acc, curvature=c["curvature"].reshape(-1),
                                          sigma=sigma)
        ref = R.run_oracle(oracle_lib, c, preconditioner="jacobi", warm_start=True, old_pressure=old_p,
                           u=R.records_to_soa(dims, visc))
        assert ref["result"].status == 0
        assert st["iterations"] == ref["result"].iterations, k
        for a, key in enumerate("uvw"):
            assert np.array_equal(bits(u[a].cpu().numpy()), bits(ref[key])), (k, key)
        assert np.array_equal(bits(p_out.cpu().numpy().reshape(-1)), bits(ref["p"])), k
        reserved = np.zeros((n, 4), np.float32)
        reserved[:, 2] = occ
        reserved[:, 3] = c["curvature"].reshape(-1)
        ocells, sc = oracle_lib.fields(ref["params"], mask, occ, ref["work"],
                                       R.soa_to_records(dims, ref["u"], ref["v"], ref["w"]), acc, reserved=reserved)
        assert np.array_equal(bits(cells.cpu().numpy().reshape(n, 16)), bits(ocells)), k
        assert np.float32(d["kinetic_energy_j"]) == np.float32(sc[3])
        vel = (ref["u"], ref["v"], ref["w"])
        old_p = ref["p"]
    want = {"host_bound": "host", "euler": "euler", "rkc": "rkc"}[name]
    assert paths == {want}, paths
    pr.close()


def test_gb300_interface_step_stages(gpu, oracle_lib):
    """GB300 solver with two densities (a moving interface): the step equals
    the oracle's predict, stress diffusion (several Euler substeps) and capillary
    viscous stages projected by a second context with a warm start, bit for
    bit; fields with the curvature in the reserved lane."""
    import mhdproj

    torch = gpu
    c = interface_case(seed=6)
    dims = c["dims"]
    nx, ny, nz = dims
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    dt, nu, mu_air, sigma = c["dt"], 1e-6, 4e-2, 0.07
    acc = np.array([0.0, 0.0, -9.81], np.float32)

    def ctx():
        pr = mhdproj.PressureProjection(dims, c["h"], outlet=True, precision="fp32", rel_tol=1e-8)
        pr.set_coefficients(t(c["alpha"]), t(c["solid"]), c["rho_liquid"], c["rho_air"])
        return pr

    a, b = ctx(), ctx()
    u = [t(c["u"]), t(c["v"]), t(c["w"])]
    st, d = a.fluid_step(u, dt, acceleration=tuple(acc), viscosity=nu, surface_tension=sigma, air_viscosity=mu_air,
                         curvature=t(c["curvature"]))
    g = oracle_lib.grid(nx, ny, nz, c["h"], c["rho_liquid"], c["rho_air"], 0, True)
    _, cls = oracle_lib.classify(g, c["solid"])
    mask = (cls != 0).astype(np.uint32)
    p = oracle_lib.make_params(dims, c["h"], dt, c["rho_liquid"], c["rho_air"], True, 0, 1e-5, 0.0,
                               int(mask.sum()), False, 1e6)
    p.physical[2] = nu
    occ = np.asarray(c["alpha"], np.float32).reshape(-1)
    rec = R.soa_to_records(dims, c["u"], c["v"], c["w"])
    pred = oracle_lib.predict(p, mask, rec)
    status, sub, _, pred = oracle_lib.diffuse_surface_stress(p, mask, occ, pred, rec, mu_air, dt)
    assert status == 0 and 1 < sub <= 8 and d["viscous_substeps"] == sub  # several Euler substeps
    visc = oracle_lib.viscous_surface(p, mask, occ, pred, acc, curvature=c["curvature"].reshape(-1), sigma=sigma)
    (u0, u1, u2), _, _ = b.project(tuple(t(x) for x in R.records_to_soa(dims, visc)), dt, warm_start=True)
    for x, y in zip(u, (u0, u1, u2)):
        assert torch.equal(x, y)
    a.close()
    b.close()


def test_interface_step_substep_limit(gpu, oracle_lib):
    """More equivalent Euler substeps than the work limit: the reference's
    message, velocity restored."""
    import mhdproj

    torch = gpu
    c = interface_case()
    pr = mhdproj.PressureProjection(c["dims"], c["h"], outlet=False, solver="reference", preconditioner="jacobi",
                                    rel_tol=1e-5, abs_div_tol=1e-5, two_phase=True)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pr.set_coefficients(t(c["alpha"]), t(c["solid"]), c["rho_liquid"], c["rho_air"])
    u = [t(c["u"]), t(c["v"]), t(c["w"])]
    before = [a.clone() for a in u]
    with pytest.raises(mhdproj.ProjectionError) as e:
        pr.fluid_step(u, c["dt"], viscosity=1e-6, surface_tension=0.07, air_viscosity=0.2, max_viscous_substeps=4)
    assert "equivalent Euler substeps, above the 4 work limit" in str(e.value)
    for a, b in zip(u, before):
        assert torch.equal(a, b)
    pr.close()


def test_export_fields_round_trip(gpu, oracle_lib, tmp_path):
    """export_fields (src/run/export.rs:9-60): fluid.bin holds the cell
    records byte for byte, metadata.json is published, and an existing frame
    directory is refused and left intact."""
    import json

    import mhdproj

    torch = gpu
    c = single_phase(R.wall_case((17, 13, 9), (0, 0, 0), True, False), dt=0.02)
    pr = make_ref_ctx(mhdproj, torch, c, "jacobi")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    u = [t(c["u"]), t(c["v"]), t(c["w"])]
    cells = torch.zeros(pr.cell_shape() + (16,), dtype=torch.float32, device="cuda")
    pr.fluid_step(u, c["dt"], acceleration=(0.0, 0.0, -9.81), viscosity=0.1, advection=True, cells=cells)
    frame = tmp_path / "run" / "frame-00000001"
    mhdproj.export_fields(c["dims"], c["h"], cells, str(frame), step=1, time_s=0.02, forcing_kind="none")
    raw = (frame / "fluid.bin").read_bytes()
    assert raw == cells.cpu().numpy().tobytes()
    meta = json.loads((frame / "metadata.json").read_text())
    n = c["dims"][0] * c["dims"][1] * c["dims"][2]
    assert meta["format_version"] == 1 and meta["step"] == 1 and meta["dims"] == list(c["dims"])
    assert meta["files"] == [{"physics": "fluid", "file": "fluid.bin", "bytes": n * 64, "f32_components_per_cell": 16}]
    assert meta["cell_order"] == "x fastest, then y, then z" and not (frame / "metadata.writing").exists()
    with pytest.raises(mhdproj.ProjectionError) as e:
        mhdproj.export_fields(c["dims"], c["h"], torch.zeros_like(cells), str(frame), step=2)
    assert "Create new frame directory" in str(e.value)
    assert (frame / "fluid.bin").read_bytes() == raw
    pr.close()


def test_step_and_fields_argument_errors(gpu, oracle_lib):
    """Invalid timesteps, viscosities and surface parameters are refused with
    the reference's validation text; nothing is touched."""
    import mhdproj

    torch = gpu
    c = single_phase(R.wall_case((17, 13, 9), (0, 0, 0), True, False), dt=0.02)
    pr = make_ref_ctx(mhdproj, torch, c, "jacobi")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    u = [t(c["u"]), t(c["v"]), t(c["w"])]
    before = [a.clone() for a in u]
    for kw in (dict(dt=0.0), dict(dt=float("nan")), dict(dt=0.02, viscosity=-1.0),
               dict(dt=0.02, surface_tension=-1.0), dict(dt=0.02, air_viscosity=float("inf"))):
        dt = kw.pop("dt")
        with pytest.raises(mhdproj.ProjectionError) as e:
            pr.fluid_step(u, dt, **kw)
        assert e.value.status == "invalid argument"
    for a, b in zip(u, before):
        assert torch.equal(a, b)
    with pytest.raises(mhdproj.ProjectionError):
        pr.fields(u, 0.0)
    pr.close()


def test_gb300_step_with_em_force(gpu, oracle_lib):
    """GB300 solver with an EM force density: the step equals the oracle's
    predict + viscous (with the force) projected by a second context."""
    import mhdproj
    from mhdproj import synth

    torch = gpu
    c = synth.make_case("jet64", scale=0.5)
    dims = c["dims"]
    nx, ny, nz = dims
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    dt, nu = 2e-5, 1e-6
    acc = np.array([0.0, 0.0, -9.81], np.float32)
    rng = np.random.default_rng(9)
    em = (rng.standard_normal((nz, ny, nx, 4)) * 1e4).astype(np.float32)

    def ctx():
        pr = mhdproj.PressureProjection(dims, c["h"], outlet=True, precision="bf16", rel_tol=1e-8)
        pr.set_coefficients(t(c["alpha"]), t(c["solid"]), c["rho_liquid"], c["rho_liquid"])
        return pr

    a, b = ctx(), ctx()
    u = [t(c["u"]), t(c["v"]), t(c["w"])]
    a.fluid_step(u, dt, acceleration=tuple(acc), viscosity=nu, advection=True, em_force=t(em))
    g = oracle_lib.grid(nx, ny, nz, c["h"], c["rho_liquid"], c["rho_liquid"], 0, True)
    _, cls = oracle_lib.classify(g, c["solid"])
    mask = (cls != 0).astype(np.uint32)
    p = oracle_lib.make_params(dims, c["h"], dt, c["rho_liquid"], c["rho_liquid"], False, 0, 1e-5, 0.0,
                               int(mask.sum()), False, 1e6)
    p.physical[2] = nu
    p.flags[1] = 1
    pred = oracle_lib.predict(p, mask, R.soa_to_records(dims, c["u"], c["v"], c["w"]))
    visc = oracle_lib.viscous(p, mask, np.asarray(c["alpha"], np.float32).reshape(-1), pred, acc,
                              em=em.reshape(-1, 4))
    (u0, u1, u2), _, _ = b.project(tuple(t(x) for x in R.records_to_soa(dims, visc)), dt, warm_start=True)
    for x, y in zip(u, (u0, u1, u2)):
        assert torch.equal(x, y)
    a.close()
    b.close()
