"""Inputs and oracle runs for the reference solver's GPU parity tests.

The GPU reference solver takes the face arrays of include/mhdproj.h (u of
(nz, ny, nx+1), v of (nz, ny+1, nx), w of (nz+1, ny, nx)); the oracle takes
the reference's face records (one vec4 per face position of the
(nx+1)(ny+1)(nz+1) face grid, lane = axis).  These helpers convert between
the two and run the oracle's FluidState::project restatement.
"""
import math

import numpy as np

from mhdproj import synth


def soa_to_records(dims, u, v, w):
    nx, ny, nz = dims
    rec = np.zeros((nz + 1, ny + 1, nx + 1, 4), np.float32)
    rec[:nz, :ny, :, 0] = np.asarray(u, np.float32).reshape(nz, ny, nx + 1)
    rec[:nz, :, :nx, 1] = np.asarray(v, np.float32).reshape(nz, ny + 1, nx)
    rec[:, :ny, :nx, 2] = np.asarray(w, np.float32).reshape(nz + 1, ny, nx)
    return rec.reshape(-1, 4)


def records_to_soa(dims, rec):
    nx, ny, nz = dims
    r = np.asarray(rec, np.float32).reshape(nz + 1, ny + 1, nx + 1, 4)
    return (np.ascontiguousarray(r[:nz, :ny, :, 0]), np.ascontiguousarray(r[:nz, :, :nx, 1]),
            np.ascontiguousarray(r[:, :ny, :nx, 2]))


def pressure_from_work(params, mask, work, meanfree):
    """fields() pressure (solver.wgsl:269-270) in FP32: potential (minus the
    gauge cell's in mean-free mode) * rho_l / dt, zero in solid cells."""
    x = work.reshape(-1, 4)[:, 0].astype(np.float32)
    anchor = (mask >> 2).astype(np.int64)
    pot = (x - x[anchor]) if meanfree else x
    rho = np.float32(params.physical[3])
    dt = np.float32(params.physical[1])
    p = (pot * rho) / dt
    return np.where(mask != 0, p, np.float32(0.0)).astype(np.float32)


def wall_case(dims, periodic, walls, reverse, seed=3):
    """The reference's multigrid fixture geometry (multigrid/tests.rs:8-63):
    1 m cells, 7000:1 density split at x = nx/2, optional walls at x = nx/2
    plus the cell (1, 1); seeded random candidate velocities."""
    nx, ny, nz = dims
    n = nx * ny * nz
    i = np.arange(n)
    x, y = i % nx, (i // nx) % ny
    if walls:
        solid = ~((x != nx // 2) & ~((x == 1) & (y == 1)))
    else:
        solid = np.zeros(n, bool)
    alpha = ((x < nx // 2) ^ reverse).astype(np.float32)
    bits = sum(1 << a for a in range(3) if periodic[a])
    rng = np.random.default_rng(seed)
    shp = ((nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx))
    u, v, w = (rng.standard_normal(s).astype(np.float32) for s in shp)
    return dict(dims=tuple(dims), h=1.0, rho_liquid=7000.0, rho_air=1.0, two_phase=True, periodic=bits,
                alpha=alpha.reshape(nz, ny, nx), solid=solid.astype(np.uint8).reshape(nz, ny, nx), u=u, v=v, w=w,
                dt=1e-5, rel_tol=1e-5, abs_div_tol=1e-5)


def cosine_case(n=16):
    """Periodic mean-free gradient (pressure_tests.rs:4-71): 16^3, h = 1 mm,
    rho 1000 single phase, phi = 0.001 cos(2 pi x/n + pi/n)."""
    h = 1e-3
    phi = lambda x: 0.001 * math.cos(2 * math.pi * (x % n) / n + math.pi / n)
    u = np.zeros((n, n, n + 1), np.float32)
    for x in range(n + 1):
        u[:, :, x] = np.float32((phi(x) - phi((x + n - 1) % n)) / h)
    return dict(dims=(n, n, n), h=h, rho_liquid=1000.0, rho_air=1000.0, two_phase=False, periodic=7,
                alpha=np.ones((n, n, n), np.float32), solid=np.zeros((n, n, n), np.uint8), u=u,
                v=np.zeros((n, n + 1, n), np.float32), w=np.zeros((n + 1, n, n), np.float32), dt=1e-5,
                rel_tol=1e-5, abs_div_tol=1e-7)


def jet_case(name, scale, rel_tol=1e-5):
    """A synthetic jet workload with closed walls (the reference's boundary)."""
    c = synth.make_case(name, scale=scale)
    return dict(dims=tuple(c["dims"]), h=c["h"], rho_liquid=c["rho_liquid"], rho_air=c["rho_air"], two_phase=True,
                periodic=0, alpha=c["alpha"], solid=c["solid"], u=c["u"], v=c["v"], w=c["w"], dt=c["dt"],
                rel_tol=rel_tol, abs_div_tol=0.0)


def run_oracle(oracle, c, preconditioner="auto", gauge=-1, max_iterations=1000, warm_start=False,
               old_pressure=None, phase=None, drag_rate=1e6, u=None):
    """oracle FluidState::project on case c; returns dict(result, u, v, w, p, work, mask, comps)."""
    dims = c["dims"]
    mask01 = (np.asarray(c["solid"]).reshape(-1) == 0).astype(np.uint32)
    comps, mask = oracle.anchors(mask01, dims, c["periodic"])
    fluid = int((mask != 0).sum())
    p = oracle.make_params(dims, c["h"], c["dt"], c["rho_liquid"], c["rho_air"], c["two_phase"], c["periodic"],
                           c["rel_tol"], c["abs_div_tol"], fluid, phase is not None, drag_rate)
    faces = soa_to_records(dims, *(u if u is not None else (c["u"], c["v"], c["w"])))
    force_mg = {"auto": -1, "jacobi": 0, "multigrid": 1}[preconditioner]
    res, vel, work, _ = oracle.ref_project(p, mask, comps, np.asarray(c["alpha"]).reshape(-1), faces,
                                           max_iterations=max_iterations, warm_start=warm_start,
                                           old_pressure=None if old_pressure is None else
                                           np.asarray(old_pressure, np.float32).reshape(-1),
                                           phase=None if phase is None else np.asarray(phase).reshape(-1),
                                           force_mg=force_mg, force_meanfree=gauge)
    uo, vo, wo = records_to_soa(dims, vel)
    meanfree = bool(res.meanfree)
    # the gauge configuration the projection used (configure_pressure_projection)
    p.initial[3] = float(np.float32(1.0) / np.float32(max(fluid, 1))) if meanfree else 0.0
    p.solve[2] = 1.0 if meanfree else float(fluid)
    pr = pressure_from_work(p, mask, work, meanfree)
    return dict(result=res, u=uo, v=vo, w=wo, p=pr, work=work.reshape(-1, 4), mask=mask, comps=comps,
                params=p)
