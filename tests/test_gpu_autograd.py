"""The torch.autograd.Function pair over the projection and its VJP
(mhdproj.autograd_projection), through the C ABI.

The projection is linear in the face velocities for fixed coefficients and
the objectives below are quadratic in its outputs, so a central difference
has no truncation error: the comparison measures the adjoint's accuracy.
"""
import math

import numpy as np
import pytest

from mhdproj import synth

pytestmark = pytest.mark.gpu


def _case(torch, mhdproj, rel_tol=1e-10):
    c = synth.make_case("jet128", scale=0.25)  # 32^3 two-phase jet, top outlet
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pr = mhdproj.PressureProjection(c["dims"], c["h"], outlet=True, precision="fp16", rel_tol=rel_tol)
    pr.set_coefficients(t(c["alpha"]), t(c["solid"]), c["rho_liquid"], c["rho_air"])
    return c, pr, (t(c["u"]), t(c["v"]), t(c["w"]))


def _objective(torch, outs, weights):
    """J = sum over the top plane of w^2 plus weighted sums of the pressure and of u."""
    uo, vo, wo, p = outs
    wp, wu = weights
    return (wo[-1].double() ** 2).sum() + (p.double() * wp).sum() + (uo.double() * wu).sum()


def test_autograd_matches_vjp_and_central_differences(gpu):
    import mhdproj

    torch = gpu
    c, pr, us = _case(torch, mhdproj)
    fn = mhdproj.autograd_projection()
    g = torch.Generator(device="cuda").manual_seed(5)
    wp = torch.randn(pr.cell_shape(), generator=g, device="cuda", dtype=torch.float64) * 1e-7
    wu = torch.randn(pr.face_shapes()[0], generator=g, device="cuda", dtype=torch.float64)
    leaves = [x.clone().requires_grad_(True) for x in us]
    outs = fn.apply(pr, c["dt"], *leaves)
    J = _objective(torch, outs, (wp, wu))
    J.backward()
    grads = [x.grad.detach().clone() for x in leaves]
    assert all(gr.device == us[0].device and gr.dtype == torch.float32 for gr in grads)

    # the same VJP called directly
    gw = torch.zeros(pr.face_shapes()[2], device="cuda")
    gw[-1] = 2.0 * outs[2][-1].detach()
    gp = (wp).float().contiguous()
    (a, b, cc), _ = pr.vjp((wu.float().contiguous(), torch.zeros(pr.face_shapes()[1], device="cuda"), gw), gp,
                           c["dt"])
    for x, y in zip(grads, (a, b, cc)):
        assert float((x - y).abs().max()) <= 1e-6 * float(y.abs().max())

    # central differences along seeded directions
    un = math.sqrt(sum(float((x.double() ** 2).sum()) for x in us))
    for k in range(4):
        d = [torch.randn(x.shape, generator=g, device="cuda") for x in us]
        dn = math.sqrt(sum(float((x.double() ** 2).sum()) for x in d))
        eps = 0.5 * un / dn
        with torch.no_grad():
            Jp = float(_objective(torch, fn.apply(pr, c["dt"], *[(x + eps * y).contiguous() for x, y in zip(us, d)]),
                                  (wp, wu)))
            Jm = float(_objective(torch, fn.apply(pr, c["dt"], *[(x - eps * y).contiguous() for x, y in zip(us, d)]),
                                  (wp, wu)))
        fd = (Jp - Jm) / (2 * eps)
        ad = sum(float((gr.double() * y.double()).sum()) for gr, y in zip(grads, d))
        assert abs(fd - ad) <= 1e-4 * abs(fd), (k, fd, ad)


def test_autograd_refuses_after_a_coefficient_change(gpu):
    import mhdproj

    torch = gpu
    c, pr, us = _case(torch, mhdproj, rel_tol=1e-6)
    fn = mhdproj.autograd_projection()
    leaves = [x.clone().requires_grad_(True) for x in us]
    outs = fn.apply(pr, c["dt"], *leaves)
    loss = (outs[2].double() ** 2).sum()
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pr.set_coefficients(t(c["alpha"]), t(c["solid"]), c["rho_liquid"], 2.0 * c["rho_air"])
    with pytest.raises(RuntimeError, match="coefficients changed"):
        loss.backward()


def test_autograd_unused_outputs_get_zero_gradients_on_the_projection_device(gpu):
    """Only the pressure enters the loss: the velocity outputs' gradients are
    zeros and the input gradient equals the VJP of the pressure alone."""
    import mhdproj

    torch = gpu
    c, pr, us = _case(torch, mhdproj)
    fn = mhdproj.autograd_projection()
    leaves = [x.clone().requires_grad_(True) for x in us]
    outs = fn.apply(pr, c["dt"], *leaves)
    gp = torch.ones(pr.cell_shape(), device="cuda") * 1e-9
    (outs[3].double() * gp.double()).sum().backward()
    zeros = [torch.zeros(s, device=pr.device) for s in pr.face_shapes()]
    (a, b, cc), _ = pr.vjp(tuple(zeros), gp, c["dt"])
    for x, y in zip(leaves, (a, b, cc)):
        assert x.grad.device == pr.device
        assert float((x.grad - y).abs().max()) <= 1e-6 * max(float(y.abs().max()), 1e-30)
