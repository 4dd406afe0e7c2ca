"""GPU parity of the GB300 solver against the FP64 oracle (through the C ABI).

Small seeded workloads are compared with the oracle directly; the full 256^3
workload is checked through size-independent properties (true FP64 residual,
discrete divergence, idempotence of the projection).
"""
import math

import numpy as np
import pytest

from mhdproj import synth

pytestmark = pytest.mark.gpu

CASES = [("jet64", 0.5), ("jet128", 0.25), ("column512", 0.125)]


def tensors(torch, c):
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return t(c["alpha"]), t(c["solid"]), (t(c["u"]), t(c["v"]), t(c["w"]))


def make(mhdproj, c, **kw):
    per = [bool(c["periodic"] & (1 << a)) for a in range(3)]
    return mhdproj.PressureProjection(c["dims"], c["h"], periodic=per, outlet=c["outlet"], **kw)


def ogrid(oracle, c):
    nx, ny, nz = c["dims"]
    return oracle.grid(nx, ny, nz, c["h"], c["rho_liquid"], c["rho_air"], c["periodic"], c["outlet"])


def rel_l2(a, b):
    a = np.asarray(a, np.float64).reshape(-1)
    b = np.asarray(b, np.float64).reshape(-1)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def periodic_case(scale=0.25):
    """jet128 geometry with periodic x and y (closed z, no outlet): pinned gauges."""
    c = synth.make_case("jet128", scale=scale)
    c["periodic"] = 3
    c["outlet"] = False
    return c


@pytest.mark.parametrize("name,scale", CASES)
def test_coefficients_bit_exact(gpu, oracle_lib, name, scale):
    import mhdproj

    torch = gpu
    c = synth.make_case(name, scale=scale)
    pr = make(mhdproj, c)
    a, s, _ = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    g = ogrid(oracle_lib, c)
    _, cls = oracle_lib.classify(g, c["solid"])
    coef, _ = oracle_lib.coefficients(g, c["alpha"], cls)
    got = pr.coefficients().cpu().numpy().reshape(-1, 4)
    assert np.array_equal(got.view(np.uint32), coef.view(np.uint32))
    m, comps = pr.topology()
    assert np.array_equal(m.astype(np.uint8), cls)


@pytest.mark.parametrize("gauge", [0, -1], ids=["pinned", "mean_free"])
def test_coefficients_bit_exact_periodic_closed(gpu, oracle_lib, gauge):
    """One closed component: pinned at its root with gauge 0; by default the
    mean-free gauge, with no pinned cell and so no reactions."""
    import mhdproj

    torch = gpu
    c = periodic_case()
    pr = make(mhdproj, c, gauge=gauge)
    a, s, _ = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    g = ogrid(oracle_lib, c)
    pinned, cls = oracle_lib.classify(g, c["solid"])
    assert pinned == 1
    if gauge != 0:
        cls[cls == 2] = 1
    coef, _ = oracle_lib.coefficients(g, c["alpha"], cls)
    got = pr.coefficients().cpu().numpy().reshape(-1, 4)
    assert np.array_equal(got.view(np.uint32), coef.view(np.uint32))
    m, _ = pr.topology()
    assert np.array_equal(m.astype(np.uint8), cls)


@pytest.mark.parametrize("name,scale", CASES)
def test_operator_matches_oracle(gpu, oracle_lib, name, scale):
    import mhdproj

    torch = gpu
    c = synth.make_case(name, scale=scale)
    pr = make(mhdproj, c)
    a, s, _ = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    g = ogrid(oracle_lib, c)
    _, cls = oracle_lib.classify(g, c["solid"])
    coef, _ = oracle_lib.coefficients(g, c["alpha"], cls)
    x = np.where(cls == 1, np.random.default_rng(1).standard_normal(cls.size), 0.0).astype(np.float32)
    y = pr.apply_operator(torch.from_numpy(x.reshape(pr.cell_shape())).cuda()).cpu().numpy()
    ref = oracle_lib.apply(g, coef, x.astype(np.float64))
    assert rel_l2(y, ref) < 1e-6


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("name,scale", CASES)
@pytest.mark.parametrize("tol", [1e-6, 1e-8])
def test_projection_matches_fp64_oracle(gpu, oracle_lib, precision, name, scale, tol):
    import mhdproj

    torch = gpu
    c = synth.make_case(name, scale=scale)
    pr = make(mhdproj, c, precision=precision, rel_tol=tol, compute_divergence=True)
    a, s, us = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    (uo, vo, wo), p, st = pr.project(us, c["dt"])
    assert st.true_relative_residual <= tol
    g = ogrid(oracle_lib, c)
    ref = oracle_lib.project(g, c["alpha"], c["solid"], c["u"], c["v"], c["w"], c["dt"], 1e-13)
    # Error budget: a residual of tol allows a solution error of about
    # cond * tol in the worst case; these fields stay far inside 100 * tol.
    phi = pr.potential().cpu().numpy()
    assert rel_l2(phi, ref["phi"]) < 100 * tol + 1e-6
    assert rel_l2(p.cpu().numpy(), ref["p"]) < 100 * tol + 1e-6
    for got, key in ((uo, "u"), (vo, "v"), (wo, "w")):
        assert rel_l2(got.cpu().numpy(), ref[key]) < 100 * tol + 1e-6
    _, cls = oracle_lib.classify(g, c["solid"])
    _, gtop = oracle_lib.coefficients(g, c["alpha"], cls)
    _, div0 = oracle_lib.divergence(g, cls, gtop, c["u"].astype(np.float64), c["v"].astype(np.float64),
                                    c["w"].astype(np.float64))
    assert st.rms_divergence <= max(10 * tol, 1e-6) * div0


@pytest.mark.parametrize("gauge", [0, -1], ids=["pinned", "mean_free"])
@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
def test_projection_periodic_closed(gpu, oracle_lib, precision, gauge):
    """Velocities do not depend on the gauge; the pressure of either gauge is
    zero at the component's root, like the FP64 oracle's."""
    import mhdproj

    torch = gpu
    c = periodic_case()
    pr = make(mhdproj, c, precision=precision, rel_tol=1e-8, gauge=gauge)
    a, s, us = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    (uo, vo, wo), p, st = pr.project(us, c["dt"])
    assert st.true_relative_residual <= 1e-8
    ref = oracle_lib.project(ogrid(oracle_lib, c), c["alpha"], c["solid"], c["u"], c["v"], c["w"], c["dt"], 1e-13)
    assert rel_l2(uo.cpu().numpy(), ref["u"]) < 1e-5
    assert rel_l2(p.cpu().numpy(), ref["p"]) < 1e-5


@pytest.mark.parametrize("precision", ["fp32", "fp16", "bf16"])
def test_preconditioner_is_symmetric_positive(gpu, oracle_lib, precision):
    import mhdproj

    torch = gpu
    c = synth.make_case("jet128", scale=0.25)
    pr = make(mhdproj, c, precision=precision)
    a, s, _ = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    _, cls = oracle_lib.classify(ogrid(oracle_lib, c), c["solid"])
    rng = np.random.default_rng(7)
    r = np.where(cls == 1, rng.standard_normal(cls.size), 0).astype(np.float32).reshape(pr.cell_shape())
    q = np.where(cls == 1, rng.standard_normal(cls.size), 0).astype(np.float32).reshape(pr.cell_shape())
    Mr = pr.apply_preconditioner(torch.from_numpy(r).cuda()).cpu().numpy().astype(np.float64)
    Mq = pr.apply_preconditioner(torch.from_numpy(q).cuda()).cpu().numpy().astype(np.float64)
    rr, qq = float((r * Mr).sum()), float((q * Mq).sum())
    sym = abs(float((r * Mq).sum()) - float((q * Mr).sum())) / math.sqrt(rr * qq)
    assert rr > 0 and qq > 0
    assert sym < {"fp32": 1e-5, "fp16": 3e-3, "bf16": 3e-2}[precision]
    assert np.all(Mr[(cls != 1).reshape(pr.cell_shape())] == 0)


def test_adjoint_identity_and_oracle(gpu, oracle_lib):
    """<P a, b> == <a, P^T b> on the GPU, and the GPU VJP equals the FP64 oracle's.

    Both solves stop on a relative residual; the error that reaches the
    identity is up to the condition number times that, so the solves run at
    1e-10, where both sit at the FP32 rounding floor of the outputs."""
    import mhdproj

    torch = gpu
    c = synth.make_case("jet128", scale=0.25)
    pr = make(mhdproj, c, precision="fp16", rel_tol=1e-10)
    a, s, us = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    rng = np.random.default_rng(11)
    shapes = pr.face_shapes()
    b = [rng.standard_normal(sh).astype(np.float32) for sh in shapes]
    (uo, vo, wo), _, _ = pr.project(us, c["dt"], pressure=False)
    gb = tuple(torch.from_numpy(x).cuda() for x in b)
    (ga, gbv, gc), st = pr.vjp(gb, None, c["dt"])
    lhs = sum(float((o.cpu().numpy().astype(np.float64) * x).sum()) for o, x in zip((uo, vo, wo), b))
    rhs = sum(float((gg.cpu().numpy().astype(np.float64) * x.cpu().numpy()).sum()) for gg, x in zip((ga, gbv, gc), us))
    assert abs(lhs - rhs) <= 1e-6 * (abs(lhs) + abs(rhs))
    g = ogrid(oracle_lib, c)
    _, ou, ov, ow = oracle_lib.project_vjp(g, c["alpha"], c["solid"], *b, None, c["dt"], 1e-13)
    for got, ref in zip((ga, gbv, gc), (ou, ov, ow)):
        assert rel_l2(got.cpu().numpy(), ref) < 1e-6


def test_chain_gradient_matches_oracle_and_finite_differences(gpu, oracle_lib):
    import mhdproj

    torch = gpu
    c = synth.make_case("adjoint128", scale=0.25)
    pr = make(mhdproj, c, precision="fp16", rel_tol=1e-9)
    a, s, us = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    f = tuple(torch.from_numpy(x).cuda() for x in (c["fu"], c["fv"], c["fw"]))
    steps = c["steps"]
    uf, J, st = pr.chain_forward(us, f, c["dt"], steps, c["checkpoint_every"])
    grad, st2 = pr.chain_backward(us)
    g = ogrid(oracle_lib, c)
    _, Jo, uk = oracle_lib.chain_forward(g, c["alpha"], c["solid"], c["u"], c["v"], c["w"], c["fu"], c["fv"], c["fw"],
                                         c["dt"], steps)
    assert abs(J - Jo) <= 1e-5 * abs(Jo)
    _, go = oracle_lib.chain_adjoint(g, c["alpha"], c["solid"], *uk, c["dt"], steps)
    for x, y in zip(grad, go):
        assert rel_l2(x.cpu().numpy(), y) < 1e-4
    # central differences of the oracle chain (FP64 states) along seeded directions
    rng = np.random.default_rng(21)
    fn = math.sqrt(sum(float((x.astype(np.float64) ** 2).sum()) for x in (c["fu"], c["fv"], c["fw"])))
    for _ in range(4):
        d = [rng.standard_normal(x.shape) for x in (c["fu"], c["fv"], c["fw"])]
        dn = math.sqrt(sum(float((x ** 2).sum()) for x in d))
        eps = 1e-3 * fn / dn
        fp = [(x + eps * y).astype(np.float32) for x, y in zip((c["fu"], c["fv"], c["fw"]), d)]
        fm = [(x - eps * y).astype(np.float32) for x, y in zip((c["fu"], c["fv"], c["fw"]), d)]
        _, Jp, _ = oracle_lib.chain_forward(g, c["alpha"], c["solid"], c["u"], c["v"], c["w"], *fp, c["dt"], steps)
        _, Jm, _ = oracle_lib.chain_forward(g, c["alpha"], c["solid"], c["u"], c["v"], c["w"], *fm, c["dt"], steps)
        fd = (Jp - Jm) / (2 * eps)
        ad = sum(float((x.cpu().numpy().astype(np.float64) * y).sum()) for x, y in zip(grad, d))
        assert abs(fd - ad) <= 1e-4 * abs(fd)


def test_chain_gradient_full_size_16_directions(gpu):
    """The 128^3 adjoint configuration in full: K = 8 steps, checkpoints every
    4, gradient of the outlet-plane objective against central differences of
    the GPU forward chain on 16 seeded directions.  The chain is affine in f
    for fixed coefficients, so J is quadratic and a central difference has no
    truncation error at any step: eps = 100 |f| / |d| lifts J(f + eps d) -
    J(f - eps d) far above the FP32 rounding of J (at eps = 1e-3 |f| / |d| the
    difference is about 1e-7 J, the size of that rounding; the FP64 oracle's
    chain, differenced at 1e-3 |f|, checks the same gradient on the 32^3
    case).  The comparison measures the adjoint's accuracy, to 1e-4
    relative."""
    import mhdproj

    torch = gpu
    c = synth.make_case("adjoint128")
    pr = make(mhdproj, c, precision="fp16", rel_tol=1e-10)
    a, s, us = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    f = [torch.from_numpy(x).cuda() for x in (c["fu"], c["fv"], c["fw"])]
    steps, every = c["steps"], c["checkpoint_every"]
    _, J, _ = pr.chain_forward(us, tuple(f), c["dt"], steps, every)
    grad, _ = pr.chain_backward(us)
    fn = math.sqrt(sum(float((x.double() ** 2).sum()) for x in f))
    gen = torch.Generator(device="cuda").manual_seed(16)
    worst = 0.0
    for _ in range(16):
        d = [torch.randn(x.shape, generator=gen, device="cuda", dtype=torch.float32) * (x != 0) for x in f]
        dn = math.sqrt(sum(float((x.double() ** 2).sum()) for x in d))
        eps = 100.0 * fn / dn
        fp = tuple((x + eps * y).contiguous() for x, y in zip(f, d))
        fm = tuple((x - eps * y).contiguous() for x, y in zip(f, d))
        _, Jp, _ = pr.chain_forward(us, fp, c["dt"], steps, every)
        _, Jm, _ = pr.chain_forward(us, fm, c["dt"], steps, every)
        fd = (Jp - Jm) / (2 * eps)
        ad = sum(float((g.double() * y.double()).sum()) for g, y in zip(grad, d))
        worst = max(worst, abs(fd - ad) / abs(fd))
    assert worst < 1e-4, worst


def test_chain_summed_objective_recomputes_from_checkpoints(gpu, oracle_lib):
    """The chain objective summed over the states after every step.  Its
    backward pass needs every forward state, so it recomputes each checkpoint
    segment's states from its checkpoint (8 steps, checkpoints every 3: a
    ragged last segment).  J and dJ/df match the FP64 oracle, the gradient
    matches central differences of the oracle's summed chain, the backward
    pass runs the recomputed projections on top of the adjoint solves, and
    switching back restores the final-state objective."""
    import mhdproj

    torch = gpu
    c = synth.make_case("adjoint128", scale=0.25)
    pr = make(mhdproj, c, precision="fp16", rel_tol=1e-9)
    a, s, us = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    f = tuple(torch.from_numpy(x).cuda() for x in (c["fu"], c["fv"], c["fw"]))
    steps, every = c["steps"], 3
    g = ogrid(oracle_lib, c)
    args = (g, c["alpha"], c["solid"], c["u"], c["v"], c["w"])
    _, _, st_f = pr.chain_forward(us, f, c["dt"], steps, every)
    _, st_fb = pr.chain_backward(us)
    pr.chain_set_objective("summed")
    with pytest.raises(mhdproj.ProjectionError):
        pr.chain_backward(us)  # a new objective needs a new forward chain
    _, J, st = pr.chain_forward(us, f, c["dt"], steps, every)
    grad, st2 = pr.chain_backward(us)
    _, Jo, go = oracle_lib.chain_summed(*args, c["fu"], c["fv"], c["fw"], c["dt"], steps)
    assert abs(J - Jo) <= 1e-5 * abs(Jo)
    for x, y in zip(grad, go):
        assert rel_l2(x.cpu().numpy(), y) < 1e-4
    # steps - checkpoints forward projections recomputed on top of the adjoint solves
    assert st2.iterations > st_fb.iterations
    rng = np.random.default_rng(23)
    fo = (c["fu"], c["fv"], c["fw"])
    fn = math.sqrt(sum(float((x.astype(np.float64) ** 2).sum()) for x in fo))
    for _ in range(2):
        d = [rng.standard_normal(x.shape) for x in fo]
        dn = math.sqrt(sum(float((x ** 2).sum()) for x in d))
        eps = 1e-3 * fn / dn
        fp = [(x + eps * y).astype(np.float32) for x, y in zip(fo, d)]
        fm = [(x - eps * y).astype(np.float32) for x, y in zip(fo, d)]
        _, Jp, _ = oracle_lib.chain_summed(*args, *fp, c["dt"], steps, gradient=False)
        _, Jm, _ = oracle_lib.chain_summed(*args, *fm, c["dt"], steps, gradient=False)
        fd = (Jp - Jm) / (2 * eps)
        ad = sum(float((x.cpu().numpy().astype(np.float64) * y).sum()) for x, y in zip(grad, d))
        assert abs(fd - ad) <= 1e-4 * abs(fd)
    pr.chain_set_objective("final")
    _, J2, _ = pr.chain_forward(us, f, c["dt"], steps, every)
    _, Jo2, _ = oracle_lib.chain_forward(*args, c["fu"], c["fv"], c["fw"], c["dt"], steps)
    assert abs(J2 - Jo2) <= 1e-5 * abs(Jo2)
    with pytest.raises(ValueError):
        pr.chain_set_objective("mean")
    pr.close()


def test_failures_leave_outputs_untouched(gpu):
    import mhdproj

    torch = gpu
    c = synth.make_case("jet128", scale=0.25)
    pr = make(mhdproj, c, max_iterations=1)
    a, s, us = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    out = tuple(torch.full_like(t, 7.0) for t in us)
    with pytest.raises(mhdproj.ProjectionError, match="did not converge"):
        pr.project(us, c["dt"], out=out)
    assert all(bool((o == 7.0).all()) for o in out)
    pr2 = make(mhdproj, c)
    pr2.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    bad = (us[0].clone(), us[1], us[2])
    bad[0][1, 1, 1] = float("nan")
    with pytest.raises(mhdproj.ProjectionError, match="Nonfinite"):
        pr2.project(bad, c["dt"], out=out)
    with pytest.raises(mhdproj.ProjectionError):
        mhdproj.PressureProjection((0, 4, 4), 1e-3)


def test_host_api_equals_device_api(gpu):
    import mhdproj

    torch = gpu
    c = synth.make_case("jet64", scale=0.5)
    pr = make(mhdproj, c)
    a, s, us = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    (uo, vo, wo), p, _ = pr.project(us, c["dt"])
    pr2 = make(mhdproj, c)
    (hu, hv, hw), hp, st = pr2.project_host(c["alpha"], c["solid"], c["rho_liquid"], c["rho_air"],
                                            (c["u"], c["v"], c["w"]), c["dt"])
    for x, y in ((uo, hu), (vo, hv), (wo, hw), (p, hp)):
        assert np.array_equal(x.cpu().numpy(), y)


def test_warm_start_reuses_the_previous_potential(gpu):
    import mhdproj

    torch = gpu
    c = synth.make_case("jet128", scale=0.25)
    pr = make(mhdproj, c, rel_tol=1e-8)
    a, s, us = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    (u1, _, _), _, st1 = pr.project(us, c["dt"])
    (u2, _, _), _, st2 = pr.project(us, c["dt"], warm_start=True)
    assert st2.iterations < st1.iterations
    assert rel_l2(u2.cpu().numpy(), u1.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("precision", ["fp16", "bf16", "fp32"])
def test_full_size_jet256_properties(gpu, precision):
    """The 256^3 two-phase workload: FP64 residual, divergence and idempotence."""
    import mhdproj

    torch = gpu
    c = synth.make_case("jet256")
    pr = make(mhdproj, c, precision=precision, rel_tol=1e-8, compute_divergence=True)
    a, s, us = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    (uo, vo, wo), p, st = pr.project(us, c["dt"])
    assert st.true_relative_residual <= 1e-8
    assert bool(torch.isfinite(p).all())
    # projecting a projected field changes it by no more than the tolerance
    (u2, v2, w2), _, st2 = pr.project((uo, vo, wo), c["dt"])
    num = sum(float(((x - y).double() ** 2).sum()) for x, y in ((u2, uo), (v2, vo), (w2, wo)))
    den = sum(float((y.double() ** 2).sum()) for y in (uo, vo, wo))
    assert math.sqrt(num / den) < 1e-6
    assert st.max_divergence < 1e-3 * float(torch.abs(us[2]).max()) / c["h"]


_FP64_FULL = {}


def _fp64_full(oracle_lib, c, name):
    if name not in _FP64_FULL:
        _FP64_FULL[name] = oracle_lib.project(ogrid(oracle_lib, c), c["alpha"], c["solid"], c["u"], c["v"], c["w"],
                                              c["dt"], 1e-12)
    return _FP64_FULL[name]


FULL = [("jet64", "fp32"), ("jet128", "fp32"), ("jet256", "fp16"), ("jet256", "bf16")]


@pytest.mark.parametrize("tol", [1e-6, 1e-8])
@pytest.mark.parametrize("name,precision", FULL, ids=[f"{a}-{b}" for a, b in FULL])
def test_full_size_configs_against_fp64(gpu, oracle_lib, name, precision, tol):
    """The benchmark configurations at their full sizes against the FP64
    oracle: 64^3 and 128^3 with FP32 levels (configurations 1 and 2), 256^3
    with FP16 and BF16 levels (configuration 3), each at relative residuals
    1e-6 and 1e-8.  Pressure and face velocities within 100 tol (relative
    L2, plus a 1e-6 floor for FP32 rounding of the outputs); the largest
    pointwise error within 1000 tol of the largest value."""
    import mhdproj

    torch = gpu
    c = synth.make_case(name)
    pr = make(mhdproj, c, precision=precision, rel_tol=tol)
    a, s, us = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    (uo, vo, wo), p, st = pr.project(us, c["dt"])
    assert st.true_relative_residual <= tol
    ref = _fp64_full(oracle_lib, c, name)
    assert ref["status"] == 0
    got_u = np.concatenate([x.cpu().numpy().reshape(-1).astype(np.float64) for x in (uo, vo, wo)])
    ref_u = np.concatenate([ref[k] for k in "uvw"])
    got_p = p.cpu().numpy().reshape(-1).astype(np.float64)
    assert rel_l2(got_p, ref["p"]) < 100 * tol + 1e-6
    assert rel_l2(got_u, ref_u) < 100 * tol + 1e-6
    assert np.abs(got_p - ref["p"]).max() <= (1000 * tol + 1e-6) * np.abs(ref["p"]).max()
    assert np.abs(got_u - ref_u).max() <= (1000 * tol + 1e-6) * np.abs(ref_u).max()
    pr.close()


def test_mean_free_gauge_refuses_the_adjoint(gpu):
    """One closed component takes the mean-free gauge; the adjoint is defined
    for outlets and pinned gauges and says so."""
    import mhdproj

    torch = gpu
    c = periodic_case()
    pr = make(mhdproj, c, precision="fp16", rel_tol=1e-6)
    a, s, us = tensors(torch, c)
    pr.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    with pytest.raises(mhdproj.ProjectionError, match="gauge = 0"):
        pr.vjp(us, None, c["dt"])
    pinned = make(mhdproj, c, precision="fp16", rel_tol=1e-6, gauge=0)
    pinned.set_coefficients(a, s, c["rho_liquid"], c["rho_air"])
    pinned.vjp(us, None, c["dt"])
