"""The library's GPU fluid step (mhdproj_fluid_step, reference solver) on the
reference's channel acceptance tests (src/fluid/tests.rs:8-160): after every
warm-started step of the run the face velocities equal the oracle's step
chain bit for bit, so the GPU reproduces the Poiseuille errors the reference
publishes (2.130% and 0.526%, docs/FLUIDS.md:54) and the hydrostatic balance.
"""
import math

import numpy as np
import pytest

import refcases as R

pytestmark = pytest.mark.gpu


def _gpu_channel(torch, mhdproj, n, periodic):
    dims = (4, n, 4)
    h = float(np.float32(0.008 / n))
    pr = mhdproj.PressureProjection(dims, h, periodic=periodic, outlet=False, solver="reference", rel_tol=1e-5,
                                    abs_div_tol=1e-5, two_phase=False)
    alpha = torch.ones(dims[2], dims[1], dims[0], dtype=torch.float32, device="cuda")
    solid = torch.zeros(dims[2], dims[1], dims[0], dtype=torch.uint8, device="cuda")
    pr.set_coefficients(alpha, solid, 1000.0, 1000.0)
    u = [torch.zeros(s, dtype=torch.float32, device="cuda") for s in
         ((dims[2], dims[1], dims[0] + 1), (dims[2], dims[1] + 1, dims[0]), (dims[2] + 1, dims[1], dims[0]))]
    return dims, h, pr, u


def _oracle_chain(oracle, dims, h, dt, periodic_bits, acc, steps):
    cells = dims[0] * dims[1] * dims[2]
    comps, mask = oracle.anchors(np.ones(cells, np.uint32), dims, periodic_bits)
    prm = oracle.make_params(dims, h, dt, 1000.0, 1000.0, False, periodic_bits, 1e-5, 1e-5, cells, False, 1e6)
    prm.physical[2] = 1e-3
    prm.flags[1] = 1
    vel = np.zeros((prm.faces[3], 4), np.float32)
    occ = np.ones(cells, np.float32)
    old = np.zeros(cells, np.float32)
    a = np.asarray(acc, np.float32)
    work = res = None
    for _ in range(steps):
        pred = oracle.predict(prm, mask, vel)
        visc = oracle.viscous(prm, mask, occ, pred, a)
        res, vel, work, _ = oracle.ref_project(prm, mask, comps, occ, visc, warm_start=True, old_pressure=old)
        old = work[:, 0].copy()
    return prm, mask, vel, work, res


def test_gpu_poiseuille_reproduces_published_errors(gpu, oracle_lib):
    import mhdproj

    torch = gpu
    errors = []
    for n, published in ((8, 0.02130), (16, 0.00526)):
        dims, h, pr, u = _gpu_channel(torch, mhdproj, n, (True, False, True))
        dt = float(np.float32(0.12 * np.float32(h) * np.float32(h) / np.float32(0.001)))
        steps = math.ceil(0.06 / dt)
        for _ in range(steps):
            pr.fluid_step(u, dt, acceleration=(1.0, 0.0, 0.0), viscosity=1e-3, advection=True)
        torch.cuda.synchronize()
        got = [t.cpu().numpy() for t in u]
        _, _, vel, _, _ = _oracle_chain(oracle_lib, dims, h, dt, 5, (1.0, 0.0, 0.0), steps)
        want = R.records_to_soa(dims, vel)
        for g, w in zip(got, want):
            np.testing.assert_array_equal(g.view(np.uint32), np.ascontiguousarray(w).view(np.uint32))
        err = norm = 0.0
        for y in range(n):
            pos = (y + 0.5) * (0.008 / n)
            exact = pos * (0.008 - pos) / (2.0 * 0.001)
            cell = 0.5 * (float(got[0][1, y, 1]) + float(got[0][1, y, 2]))
            err += (cell - exact) ** 2
            norm += exact ** 2
        rel = math.sqrt(err / norm)
        errors.append(rel)
        assert round(100.0 * rel, 3) == pytest.approx(100.0 * published, abs=1e-9), rel
        pr.close()
    assert errors[1] < 0.015 and errors[1] < 0.45 * errors[0]


def test_gpu_closed_box_hydrostatic_balance(gpu):
    import mhdproj

    torch = gpu
    dims, h, pr, u = _gpu_channel(torch, mhdproj, 8, (False, False, False))
    p = torch.empty(dims[2], dims[1], dims[0], dtype=torch.float32, device="cuda")
    st, d = pr.fluid_step(u, 1e-4, acceleration=(0.0, -9.81, 0.0), viscosity=1e-3, advection=True, p_out=p)
    assert 0 < st["iterations"] <= 1000
    assert d["max_speed_m_s"] < 1e-5
    pc = p.cpu().numpy()
    low, high = float(pc[2, 1, 2]), float(pc[2, 6, 2])
    assert abs((low - high) / (1000.0 * 9.81 * 0.005) - 1.0) < 0.005
    pr.close()
