"""The FP64 oracle of the GB300 path's discrete problem (oracle/oracle_native.c):
self-consistency checks that do not depend on the GPU."""
import numpy as np
import pytest

from mhdproj import synth


def small(name, scale, **kw):
    c = synth.make_case(name, scale=scale, **kw)
    nx, ny, nz = c["dims"]
    return c


def grid_of(oracle, c):
    nx, ny, nz = c["dims"]
    return oracle.grid(nx, ny, nz, c["h"], c["rho_liquid"], c["rho_air"], c["periodic"], c["outlet"])


@pytest.mark.parametrize("name,scale", [("jet64", 0.25), ("jet128", 0.125), ("column512", 0.0625)])
def test_projection_is_divergence_free(oracle_lib, name, scale):
    c = small(name, scale)
    g = grid_of(oracle_lib, c)
    r = oracle_lib.project(g, c["alpha"], c["solid"], c["u"], c["v"], c["w"], c["dt"], 1e-13)
    assert r["status"] == 0 and r["residual"] <= 1e-13
    pinned, cls = oracle_lib.classify(g, c["solid"])
    _, gtop = oracle_lib.coefficients(g, c["alpha"], cls)
    mx, rms = oracle_lib.divergence(g, cls, gtop, r["u"], r["v"], r["w"])
    mx0, _ = oracle_lib.divergence(g, cls, gtop, c["u"].astype(np.float64), c["v"].astype(np.float64),
                                   c["w"].astype(np.float64))
    assert mx <= 1e-10 * mx0


def test_outlet_carries_the_net_inflow(oracle_lib):
    """With solid side walls and an outlet, mass leaves only through the top face."""
    c = small("jet64", 0.25)
    g = grid_of(oracle_lib, c)
    r = oracle_lib.project(g, c["alpha"], c["solid"], c["u"], c["v"], c["w"], c["dt"], 1e-13)
    nx, ny, nz = c["dims"]
    w = r["w"].reshape(nz + 1, ny, nx)
    assert abs(w[0].sum()) == 0.0  # closed bottom
    # The top flux equals the total source of the interior (zero divergence).
    assert np.isfinite(w[nz]).all()


def test_closed_components_are_pinned(oracle_lib):
    g = oracle_lib.grid(3, 1, 1, 1.0, 1000.0, 1000.0, 0, False)
    pinned, cls = oracle_lib.classify(g, np.array([1, 0, 1], np.uint8))
    assert pinned == 1 and list(cls) == [0, 2, 0]
    # 3 x 1 x 2 with an outlet: {0, 3} reaches the top layer, {2} does not.
    g = oracle_lib.grid(3, 1, 2, 1.0, 1000.0, 1000.0, 0, True)
    pinned, cls = oracle_lib.classify(g, np.array([0, 1, 0, 0, 1, 1], np.uint8))
    assert pinned == 1 and list(cls) == [1, 0, 2, 1, 0, 0]


def test_adjoint_identity(oracle_lib):
    """<P u, v> == <u, P^T v> for the FP64 projection and its VJP."""
    c = small("jet128", 0.125)
    g = grid_of(oracle_lib, c)
    rng = np.random.default_rng(3)
    shapes = oracle_lib.face_shapes(g)
    a = [rng.standard_normal(s).astype(np.float32) for s in shapes]
    b = [rng.standard_normal(s) for s in shapes]
    r = oracle_lib.project(g, c["alpha"], c["solid"], *a, c["dt"], 1e-13)
    st, *vt = oracle_lib.project_vjp(g, c["alpha"], c["solid"], *b, None, c["dt"], 1e-13)
    lhs = sum(float(np.dot(r[k], bb.reshape(-1))) for k, bb in zip("uvw", b))
    rhs = sum(float(np.dot(aa.reshape(-1).astype(np.float64), vv)) for aa, vv in zip(a, vt))
    assert abs(lhs - rhs) <= 1e-10 * (abs(lhs) + abs(rhs))


def test_chain_adjoint_matches_central_differences(oracle_lib):
    c = synth.make_case("adjoint128", scale=0.125)
    g = grid_of(oracle_lib, c)
    steps = 3
    st, J, uk = oracle_lib.chain_forward(g, c["alpha"], c["solid"], c["u"], c["v"], c["w"], c["fu"], c["fv"], c["fw"],
                                         c["dt"], steps)
    st2, grad = oracle_lib.chain_adjoint(g, c["alpha"], c["solid"], *uk, c["dt"], steps)
    rng = np.random.default_rng(5)
    f = [c["fu"], c["fv"], c["fw"]]
    fn = np.sqrt(sum(float((x.astype(np.float64) ** 2).sum()) for x in f))
    for _ in range(2):
        d = [rng.standard_normal(x.shape) for x in f]
        dn = np.sqrt(sum(float((x ** 2).sum()) for x in d))
        eps = 1e-3 * fn / dn
        fp = [(x + eps * y).astype(np.float32) for x, y in zip(f, d)]
        fm = [(x - eps * y).astype(np.float32) for x, y in zip(f, d)]
        _, Jp, _ = oracle_lib.chain_forward(g, c["alpha"], c["solid"], c["u"], c["v"], c["w"], *fp, c["dt"], steps)
        _, Jm, _ = oracle_lib.chain_forward(g, c["alpha"], c["solid"], c["u"], c["v"], c["w"], *fm, c["dt"], steps)
        fd = (Jp - Jm) / (2 * eps)
        ad = sum(float(np.dot(gg, dd.reshape(-1))) for gg, dd in zip(grad, d))
        assert abs(fd - ad) <= 1e-4 * abs(ad)


def test_summed_chain_adjoint_matches_central_differences(oracle_lib):
    """The chain objective summed over the states after every step: for one
    step it is the final-state objective, and its adjoint (which adds 2 w_k on
    the outlet faces after each step's VJP) matches central differences."""
    c = synth.make_case("adjoint128", scale=0.125)
    g = grid_of(oracle_lib, c)
    args = (g, c["alpha"], c["solid"], c["u"], c["v"], c["w"])
    f = [c["fu"], c["fv"], c["fw"]]
    _, J1, _ = oracle_lib.chain_forward(*args, *f, c["dt"], 1)
    _, S1, _ = oracle_lib.chain_summed(*args, *f, c["dt"], 1, gradient=False)
    assert S1 == pytest.approx(J1, rel=1e-14)
    steps = 3
    st, J, grad = oracle_lib.chain_summed(*args, *f, c["dt"], steps)
    _, Jf, _ = oracle_lib.chain_forward(*args, *f, c["dt"], steps)
    assert st == 0 and J > Jf
    rng = np.random.default_rng(6)
    fn = np.sqrt(sum(float((x.astype(np.float64) ** 2).sum()) for x in f))
    for _ in range(2):
        d = [rng.standard_normal(x.shape) for x in f]
        dn = np.sqrt(sum(float((x ** 2).sum()) for x in d))
        eps = 1e-3 * fn / dn
        fp = [(x + eps * y).astype(np.float32) for x, y in zip(f, d)]
        fm = [(x - eps * y).astype(np.float32) for x, y in zip(f, d)]
        _, Jp, _ = oracle_lib.chain_summed(*args, *fp, c["dt"], steps, gradient=False)
        _, Jm, _ = oracle_lib.chain_summed(*args, *fm, c["dt"], steps, gradient=False)
        fd = (Jp - Jm) / (2 * eps)
        ad = sum(float(np.dot(gg, dd.reshape(-1))) for gg, dd in zip(grad, d))
        assert abs(fd - ad) <= 1e-4 * abs(ad)
