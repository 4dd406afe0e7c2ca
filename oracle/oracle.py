"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by bench.py's CPU-baseline leg, and there only as the expected results the
GPU path is compared with or as the timed CPU baseline.  The product library never loads it.

``oref_*`` restates the reference projection in FP32 with the reference's
buffer layout (vec4 per (n+1)^3 face-cell); ``onat_*`` solves the GB300
path's discrete problem in FP64.  See mhd_oracle.h for the citations.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


class OrefParams(C.Structure):
    _fields_ = [
        ("dims", C.c_uint32 * 4),
        ("faces", C.c_uint32 * 4),
        ("flags", C.c_uint32 * 4),
        ("physical", C.c_float * 4),
        ("initial", C.c_float * 4),
        ("solve", C.c_float * 4),
        ("surface", C.c_float * 4),
    ]


class OrefResult(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("iterations", C.c_uint32),
        ("residual", C.c_float),
        ("meanfree", C.c_int32),
        ("multigrid", C.c_int32),
        ("levels", C.c_uint32),
        ("coarse_cells", C.c_uint64),
    ]


class OnatGrid(C.Structure):
    _fields_ = [
        ("nx", C.c_uint32),
        ("ny", C.c_uint32),
        ("nz", C.c_uint32),
        ("periodic", C.c_uint32),
        ("outlet", C.c_int32),
        ("h", C.c_float),
        ("rho_liquid", C.c_float),
        ("rho_air", C.c_float),
        ("single", C.c_int32),
        ("drag_rate", C.c_float),
        ("dt", C.c_float),
        ("phase", C.c_void_p),
    ]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile recipe next to this file."""
    if force or not os.path.exists(LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(LIB_PATH)
    return any(
        os.path.getmtime(os.path.join(HERE, f)) > t
        for f in ("oracle_ref.c", "oracle_native.c", "oracle_em.c", "mhd_oracle.h", "Makefile")
    )


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.oref_anchors.argtypes = [_u32p, C.POINTER(C.c_uint32), C.c_uint32]
        L.oref_anchors.restype = C.c_uint32
        L.oref_hierarchy.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint64),
                                     C.c_void_p, C.c_uint32]
        L.oref_hierarchy.restype = C.c_int
        L.oref_make_params.argtypes = [C.POINTER(OrefParams), C.POINTER(C.c_uint32), C.c_float, C.c_float,
                                       C.c_float, C.c_float, C.c_int, C.c_uint32, C.c_float, C.c_float,
                                       C.c_uint32, C.c_int, C.c_float]
        L.oref_project.argtypes = [C.POINTER(OrefParams), _u32p, C.c_uint32, _f32p, C.c_void_p, C.c_void_p,
                                   _f32p, _f32p, _f32p, C.c_uint32, C.c_int, C.c_int, C.c_int,
                                   C.POINTER(OrefResult)]
        L.oref_coefficients.argtypes = [C.POINTER(OrefParams), _u32p, _f32p, C.c_void_p, _f32p]
        L.oref_apply_cached.argtypes = [C.POINTER(OrefParams), _u32p, _f32p, _f32p, C.c_uint32, _f32p]
        L.oref_apply_uncached.argtypes = [C.POINTER(OrefParams), _u32p, _f32p, C.c_void_p, _f32p, C.c_uint32,
                                          _f32p, _f32p]
        L.oref_predict.argtypes = [C.POINTER(OrefParams), _u32p, _f32p, _f32p]
        L.oref_viscous.argtypes = [C.POINTER(OrefParams), _u32p, _f32p, C.c_void_p, C.c_void_p, _f32p, _f32p,
                                   _f32p]
        L.oref_viscous_surface.argtypes = [C.POINTER(OrefParams), _u32p, _f32p, C.c_void_p, C.c_void_p, _f32p,
                                           C.c_void_p, C.c_float, _f32p, _f32p]
        L.oref_diffuse_surface_stress.argtypes = [C.POINTER(OrefParams), _u32p, _f32p, C.c_void_p, C.c_float,
                                                  C.c_float, C.c_uint32, _f32p, _f32p, C.POINTER(C.c_uint32),
                                                  C.POINTER(C.c_float)]
        L.oref_diffuse_surface_stress.restype = C.c_int
        L.oref_rkc_schedule.argtypes = [C.c_double, C.c_uint32, _f32p, C.c_uint32]
        L.oref_rkc_schedule.restype = C.c_uint32
        L.oref_fields.argtypes = [C.POINTER(OrefParams), _u32p, _f32p, _f32p, _f32p, C.c_void_p, _f32p,
                                  C.c_void_p, C.c_void_p, _f32p]
        L.oref_mg_create.argtypes = [C.POINTER(OrefParams), _u32p, _f32p, C.c_int]
        L.oref_mg_create.restype = C.c_void_p
        L.oref_mg_destroy.argtypes = [C.c_void_p]
        L.oref_mg_levels.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oref_mg_levels.restype = C.c_uint32
        L.oref_mg_build.argtypes = [C.c_void_p]
        L.oref_mg_apply.argtypes = [C.c_void_p, _f32p]
        L.oref_mg_coeff.argtypes = [C.c_void_p]
        L.oref_mg_coeff.restype = C.POINTER(C.c_float)
        L.oref_mg_value.argtypes = [C.c_void_p]
        L.oref_mg_value.restype = C.POINTER(C.c_float)
        L.oref_mg_probe_action.argtypes = [C.c_void_p, C.c_uint32, _f32p, _f32p]
        L.oref_mg_coarse_solve.argtypes = [C.c_void_p, _f32p]
        L.oref_mg_coarse_jacobi_sequence.argtypes = [C.c_void_p, _f32p]

        g = C.POINTER(OnatGrid)
        L.onat_classify.argtypes = [g, _u8p, _u8p]
        L.onat_classify.restype = C.c_uint32
        L.onat_coefficients.argtypes = [g, _f32p, _u8p, _f32p, _f32p]
        L.onat_rhs.argtypes = [g, _u8p, _f32p, _f32p, _f32p, _f32p, _f64p]
        L.onat_apply.argtypes = [g, _f32p, _f64p, _f64p]
        L.onat_solve.argtypes = [g, _f32p, _u8p, _f64p, _f64p, C.c_double, C.c_int, C.POINTER(C.c_int),
                                 C.POINTER(C.c_double)]
        L.onat_correct.argtypes = [g, _f32p, _u8p, _f32p, _f64p, _f32p, _f32p, _f32p, _f64p, _f64p, _f64p]
        L.onat_project.argtypes = [g, _f32p, _u8p, _f32p, _f32p, _f32p, C.c_float, C.c_double, _f64p, _f64p,
                                   _f64p, _f64p, _f64p, C.POINTER(C.c_int), C.POINTER(C.c_double)]
        L.onat_project_vjp.argtypes = [g, _f32p, _u8p, _f64p, _f64p, _f64p, C.c_void_p, C.c_float, C.c_double,
                                       _f64p, _f64p, _f64p]
        L.onat_divergence.argtypes = [g, _u8p, _f32p, _f64p, _f64p, _f64p, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]
        L.onat_chain_forward.argtypes = [g, _f32p, _u8p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, C.c_float,
                                         C.c_int, C.c_double, _f64p, _f64p, _f64p, C.POINTER(C.c_double)]
        L.onat_chain_adjoint.argtypes = [g, _f32p, _u8p, _f64p, _f64p, _f64p, C.c_float, C.c_int, C.c_double,
                                         _f64p, _f64p, _f64p]
        L.onat_chain_summed.argtypes = [g, _f32p, _u8p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, C.c_float, C.c_int,
                                        C.c_double, C.POINTER(C.c_double), C.c_void_p, C.c_void_p, C.c_void_p]
        L.oref_classify_cells.argtypes = [C.c_uint32, _u32p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p,
                                          C.c_uint32, _u32p, _f32p]
        L.oref_classify_cells.restype = C.c_uint32
        L.oem_new.argtypes = [C.POINTER(C.c_uint32), C.c_float, C.POINTER(C.c_float), C.c_double, C.c_float,
                              C.c_uint32, C.c_int]
        L.oem_new.restype = C.c_void_p
        L.oem_free.argtypes = [C.c_void_p]
        L.oem_sizes.argtypes = [C.c_void_p, _u32p]
        L.oem_set_materials.argtypes = [C.c_void_p, _u32p, _f32p, C.c_uint32, _f32p]
        L.oem_set_materials.restype = C.c_int
        L.oem_set_motional.argtypes = [C.c_void_p, C.c_void_p]
        L.oem_set_reaction.argtypes = [C.c_void_p, _f32p]
        L.oem_set_motion.argtypes = [C.c_void_p, _f32p]
        L.oem_set_nodal_switch.argtypes = [C.c_void_p, C.c_uint32]
        L.oem_update_config.argtypes = [C.c_void_p, C.c_double, C.c_float, C.c_uint32]
        L.oem_set_predict.argtypes = [C.c_void_p, C.c_int]
        L.oem_set_previous.argtypes = [C.c_void_p, _f32p]
        L.oem_apply_nodal.argtypes = [C.c_void_p, _f32p, _f32p]
        L.oem_prediction.argtypes = [C.c_void_p, _f32p]
        L.oem_time.argtypes = [C.c_void_p, _f64p]
        L.oem_evaluate_sources.argtypes = [C.c_void_p, _f32p, C.c_uint32, _f32p]
        L.oem_body_forces.argtypes = [C.c_void_p, _u32p, C.c_uint32, _f32p]
        L.oem_energy.argtypes = [C.c_void_p, _f64p]
        L.oem_energy.restype = C.c_int
        L.oem_get.argtypes = [C.c_void_p, C.c_int, _f32p]
        L.oem_apply_operator.argtypes = [C.c_void_p, _f32p, _f32p, C.c_int]
        L.oem_advance.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_void_p, _f32p, _f32p]
        L.oem_advance.restype = C.c_int
        _lib = L
    return _lib


# ----------------------------------------------------------------- reference
def anchors(mask, dims, periodic_bits=0):
    """anchors() of src/fluid/mod.rs:1447-1493: returns (components, encoded mask)."""
    m = np.ascontiguousarray(mask, dtype=np.uint32).copy()
    d = (C.c_uint32 * 3)(*dims)
    comps = lib().oref_anchors(m, d, periodic_bits)
    return int(comps), m


def hierarchy(dims4):
    """hierarchy() of src/fluid/multigrid.rs:25-65: (levels, coarse cells) or None if rejected."""
    d = (C.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in dims4])
    nl = C.c_uint32()
    cc = C.c_uint64()
    buf = (C.c_uint32 * (4 * 64))()
    rc = lib().oref_hierarchy(d, C.byref(nl), C.byref(cc), C.cast(buf, C.c_void_p), 64)
    if rc:
        return None
    levels = [tuple(buf[4 * l:4 * l + 4]) for l in range(nl.value)]
    return levels, cc.value


def make_params(dims, h, dt, rho_liquid, rho_air=None, two_phase=False, periodic_bits=0, rel_tol=1e-5,
                abs_div_tol=1e-5, fluid_cells=0, thermal_drag=False, drag_rate=1e6):
    p = OrefParams()
    d = (C.c_uint32 * 3)(*dims)
    lib().oref_make_params(C.byref(p), d, h, dt, rho_liquid, rho_liquid if rho_air is None else rho_air,
                           int(two_phase), periodic_bits, rel_tol, abs_div_tol, fluid_cells, int(thermal_drag),
                           drag_rate)
    return p


def ref_project(params, mask, components, occupancy, predicted, max_iterations=1000, warm_start=False,
                old_pressure=None, phase=None, force_mg=-1, force_meanfree=-1):
    """FluidState::project on the restated FP32 pipeline.

    predicted: float32 (nf, 4) candidate velocities; returns (result, velocity (nf,4), work (n,4))."""
    n = params.dims[3]
    nf = params.faces[3]
    pred = np.ascontiguousarray(predicted, dtype=np.float32).reshape(nf, 4).copy()
    vel = np.zeros((nf, 4), np.float32)
    work = np.zeros((n, 4), np.float32)
    res = OrefResult()
    ph = None if phase is None else np.ascontiguousarray(phase, dtype=np.float32)
    op = None if old_pressure is None else np.ascontiguousarray(old_pressure, dtype=np.float32)
    lib().oref_project(C.byref(params), np.ascontiguousarray(mask, dtype=np.uint32), components,
                       np.ascontiguousarray(occupancy, dtype=np.float32),
                       None if ph is None else ph.ctypes.data_as(C.c_void_p),
                       None if op is None else op.ctypes.data_as(C.c_void_p),
                       pred.reshape(-1), vel.reshape(-1), work.reshape(-1), max_iterations, int(warm_start),
                       force_mg, force_meanfree, C.byref(res))
    return res, vel, work, pred


def _opt(a, dtype=np.float32):
    if a is None:
        return None, None
    a = np.ascontiguousarray(a, dtype=dtype)
    return a, a.ctypes.data_as(C.c_void_p)


def predict(params, mask, velocity):
    """predict (solver.wgsl:127-141): vec4[nf] face records -> predicted vec4[nf]."""
    vel = np.ascontiguousarray(velocity, np.float32).reshape(-1)
    out = np.zeros_like(vel)
    lib().oref_predict(C.byref(params), np.ascontiguousarray(mask, np.uint32), vel, out)
    return out.reshape(-1, 4)


def viscous(params, mask, occupancy, predicted, acceleration, em=None, phase=None):
    """viscous (solver.wgsl:143-163, no moving interface): predicted vec4[nf] -> velocity vec4[nf]."""
    pred = np.ascontiguousarray(predicted, np.float32).reshape(-1)
    out = np.zeros_like(pred)
    em_a, em_p = _opt(em)
    ph_a, ph_p = _opt(phase)
    acc = np.ascontiguousarray(acceleration, np.float32)
    lib().oref_viscous(C.byref(params), np.ascontiguousarray(mask, np.uint32),
                       np.ascontiguousarray(occupancy, np.float32), ph_p, em_p, acc, pred, out)
    return out.reshape(-1, 4)


def viscous_surface(params, mask, occupancy, predicted, acceleration, curvature=None, sigma=0.0, em=None,
                    phase=None):
    """viscous with a moving interface (capillary force, face densities)."""
    pred = np.ascontiguousarray(predicted, np.float32).reshape(-1)
    out = np.zeros_like(pred)
    em_a, em_p = _opt(em)
    ph_a, ph_p = _opt(phase)
    cv_a, cv_p = _opt(curvature)
    acc = np.ascontiguousarray(acceleration, np.float32)
    lib().oref_viscous_surface(C.byref(params), np.ascontiguousarray(mask, np.uint32),
                               np.ascontiguousarray(occupancy, np.float32), ph_p, em_p, acc, cv_p, sigma, pred, out)
    return out.reshape(-1, 4)


def diffuse_surface_stress(params, mask, occupancy, predicted, velocity, mu_air, dt, max_substeps=4096,
                           phase=None):
    """FluidState::diffuse_surface_stress: returns (status, substeps, gpu bound or -1,
    diffused predicted vec4[nf])."""
    pred = np.ascontiguousarray(predicted, np.float32).reshape(-1).copy()
    vel = np.ascontiguousarray(velocity, np.float32).reshape(-1).copy()
    ph_a, ph_p = _opt(phase)
    sub = C.c_uint32()
    bound = C.c_float()
    st = lib().oref_diffuse_surface_stress(C.byref(params), np.ascontiguousarray(mask, np.uint32),
                                           np.ascontiguousarray(occupancy, np.float32), ph_p, mu_air, dt,
                                           max_substeps, pred, vel, C.byref(sub), C.byref(bound))
    return st, sub.value, bound.value, pred.reshape(-1, 4)


def rkc_schedule(dt, euler_steps):
    """stabilized::schedule rows (n, 8)."""
    cap = int(np.ceil(3.0 * np.sqrt(euler_steps))) + 2
    rows = np.zeros(8 * cap, np.float32)
    n = lib().oref_rkc_schedule(dt, euler_steps, rows, cap)
    return rows.reshape(cap, 8)[:n]


def fields(params, mask, occupancy, work, velocity, acceleration, em=None, reserved=None, cells=True):
    """fields + diagnostics (solver.wgsl:256-291): returns (cells (n,16) or None, scalars (12,))."""
    n = params.dims[3]
    em_a, em_p = _opt(em)
    rs_a, rs_p = _opt(reserved)
    out = np.zeros((n, 16), np.float32) if cells else None
    sc = np.zeros(12, np.float32)
    lib().oref_fields(C.byref(params), np.ascontiguousarray(mask, np.uint32),
                      np.ascontiguousarray(occupancy, np.float32), np.ascontiguousarray(work, np.float32).reshape(-1),
                      np.ascontiguousarray(velocity, np.float32).reshape(-1), em_p,
                      np.ascontiguousarray(acceleration, np.float32), rs_p,
                      None if out is None else out.ctypes.data_as(C.c_void_p), sc)
    return out, sc


# -------------------------------------------------------------------- native
def grid(nx, ny, nz, h, rho_liquid, rho_air, periodic=0, outlet=True, single=False, phase=None, drag_rate=0.0,
         dt=0.0):
    """The FP64 oracle's problem description.  single: one phase (mobility 1);
    phase (cells, float32) with drag_rate and dt: thermal phase drag."""
    ph = None if phase is None else np.ascontiguousarray(phase, dtype=np.float32).reshape(-1)
    g = OnatGrid(nx, ny, nz, periodic, int(outlet), h, rho_liquid, rho_air, int(bool(single)), drag_rate, dt,
                 None if ph is None else ph.ctypes.data)
    g._phase = ph  # keeps the array alive while the grid is used
    return g


def classify(g, solid):
    cls = np.zeros(g.nx * g.ny * g.nz, np.uint8)
    pinned = lib().onat_classify(C.byref(g), np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1), cls)
    return int(pinned), cls


def coefficients(g, alpha, cls):
    n = g.nx * g.ny * g.nz
    coef = np.zeros(4 * n, np.float32)
    gtop = np.zeros(g.nx * g.ny, np.float32)
    lib().onat_coefficients(C.byref(g), np.ascontiguousarray(alpha, dtype=np.float32).reshape(-1), cls, coef,
                            gtop)
    return coef.reshape(n, 4), gtop


def rhs(g, cls, gtop, u, v, w):
    b = np.zeros(g.nx * g.ny * g.nz, np.float64)
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    lib().onat_rhs(C.byref(g), cls, gtop, f(u), f(v), f(w), b)
    return b


def apply(g, coef, x):
    y = np.zeros_like(x, dtype=np.float64)
    lib().onat_apply(C.byref(g), np.ascontiguousarray(coef, dtype=np.float32).reshape(-1),
                     np.ascontiguousarray(x, dtype=np.float64), y)
    return y


def face_shapes(g):
    return ((g.nz, g.ny, g.nx + 1), (g.nz, g.ny + 1, g.nx), (g.nz + 1, g.ny, g.nx))


def project(g, alpha, solid, u, v, w, dt, rtol=1e-13):
    """FP64 projection: returns dict(phi, u, v, w, p, iterations, residual, status)."""
    n = g.nx * g.ny * g.nz
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    su, sv, sw = face_shapes(g)
    phi = np.zeros(n)
    uo, vo, wo = np.zeros(int(np.prod(su))), np.zeros(int(np.prod(sv))), np.zeros(int(np.prod(sw)))
    p = np.zeros(n)
    it = C.c_int()
    rel = C.c_double()
    st = lib().onat_project(C.byref(g), f(alpha), np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1),
                            f(u), f(v), f(w), dt, rtol, phi, uo, vo, wo, p, C.byref(it), C.byref(rel))
    return dict(phi=phi, u=uo, v=vo, w=wo, p=p, iterations=it.value, residual=rel.value, status=st)


def project_vjp(g, alpha, solid, gu, gv, gw, gp, dt, rtol=1e-13):
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    d = lambda a: np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    su, sv, sw = face_shapes(g)
    ou, ov, ow = np.zeros(int(np.prod(su))), np.zeros(int(np.prod(sv))), np.zeros(int(np.prod(sw)))
    gpp = None if gp is None else d(gp)
    st = lib().onat_project_vjp(C.byref(g), f(alpha), np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1),
                                d(gu), d(gv), d(gw), None if gpp is None else gpp.ctypes.data_as(C.c_void_p), dt,
                                rtol, ou, ov, ow)
    return st, ou, ov, ow


def divergence(g, cls, gtop, u, v, w):
    mx = C.c_double()
    rms = C.c_double()
    d = lambda a: np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    lib().onat_divergence(C.byref(g), cls, gtop, d(u), d(v), d(w), C.byref(mx), C.byref(rms))
    return mx.value, rms.value


def chain_forward(g, alpha, solid, u0, v0, w0, fu, fv, fw, dt, steps, rtol=1e-13):
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    su, sv, sw = face_shapes(g)
    uk, vk, wk = np.zeros(int(np.prod(su))), np.zeros(int(np.prod(sv))), np.zeros(int(np.prod(sw)))
    J = C.c_double()
    st = lib().onat_chain_forward(C.byref(g), f(alpha), np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1),
                                  f(u0), f(v0), f(w0), f(fu), f(fv), f(fw), dt, steps, rtol, uk, vk, wk,
                                  C.byref(J))
    return st, J.value, (uk, vk, wk)


def chain_adjoint(g, alpha, solid, uk, vk, wk, dt, steps, rtol=1e-13):
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    d = lambda a: np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    su, sv, sw = face_shapes(g)
    gu, gv, gw = np.zeros(int(np.prod(su))), np.zeros(int(np.prod(sv))), np.zeros(int(np.prod(sw)))
    st = lib().onat_chain_adjoint(C.byref(g), f(alpha), np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1),
                                  d(uk), d(vk), d(wk), dt, steps, rtol, gu, gv, gw)
    return st, (gu, gv, gw)


def chain_summed(g, alpha, solid, u0, v0, w0, fu, fv, fw, dt, steps, gradient=True, rtol=1e-13):
    """The chain with J summed over the states after every step (FP64):
    returns (status, J, (gu, gv, gw) or None)."""
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    su, sv, sw = face_shapes(g)
    grads = [np.zeros(int(np.prod(s))) for s in (su, sv, sw)] if gradient else None
    ptr = lambda a: a.ctypes.data_as(C.c_void_p) if a is not None else None
    J = C.c_double()
    st = lib().onat_chain_summed(C.byref(g), f(alpha), np.ascontiguousarray(solid, dtype=np.uint8).reshape(-1),
                                 f(u0), f(v0), f(w0), f(fu), f(fv), f(fw), dt, steps, rtol, C.byref(J),
                                 *([ptr(x) for x in grads] if grads else [None, None, None]))
    return st, J.value, (tuple(grads) if grads else None)


def classify_cells(materials, liquid_material, mask, cells, thermal=None, thermal_stride=1, interface=None,
                   interface_stride=2):
    """phase/surface passes in place on `mask` (uint32) and `cells` (n x 16
    float32); returns the changed flags."""
    m = np.ascontiguousarray(materials, np.uint32).reshape(-1)
    th = None if thermal is None else np.ascontiguousarray(thermal, np.float32).reshape(-1)
    it = None if interface is None else np.ascontiguousarray(interface, np.float32).reshape(-1)
    return int(lib().oref_classify_cells(m.size, m, int(liquid_material), None if th is None else th.ctypes.data,
                                         int(thermal_stride), None if it is None else it.ctypes.data,
                                         int(interface_stride), mask, cells.reshape(-1)))


class EmSolve:
    """The EM induction step restated in FP32 (oracle_em.c): one instance per
    grid, mirroring EmState (src/em/mod.rs) without its source summation."""

    OK, NOT_CONVERGED, NONFINITE = 0, 1, 2

    def __init__(self, dims, h, dt=1e-5, rel_tol=1e-5, max_iterations=1000, origin=(0.0, 0.0, 0.0), vacuum=False,
                 nodal_switch_after=1024):
        L = lib()
        d = (C.c_uint32 * 3)(*dims)
        o = (C.c_float * 3)(*origin)
        self._p = L.oem_new(d, float(h), o, float(dt), float(rel_tol), int(max_iterations), int(bool(vacuum)))
        if not self._p:
            raise MemoryError("oem_new")
        sz = np.zeros(8, np.uint32)
        L.oem_sizes(self._p, sz)
        self.dims = tuple(int(v) for v in sz[:3])
        self.cells = int(sz[3])
        self.edge_counts = tuple(int(v) for v in sz[4:7])
        self.edges = int(sz[7])
        L.oem_set_nodal_switch(self._p, int(nodal_switch_after))

    def close(self):
        if self._p:
            lib().oem_free(self._p)
            self._p = None

    def __del__(self):
        self.close()

    def set_materials(self, materials, properties):
        m = np.ascontiguousarray(materials, np.uint32).reshape(-1)
        pr = np.ascontiguousarray(properties, np.float32).reshape(-1, 2)
        check = np.zeros(4, np.float32)
        rc = lib().oem_set_materials(self._p, m, pr.reshape(-1), pr.shape[0], check)
        if rc != 0:
            raise ValueError("material id without a property row")
        return check

    def set_motional(self, emf=None):
        e = None if emf is None else np.ascontiguousarray(emf, np.float32)
        lib().oem_set_motional(self._p, None if e is None else e.ctypes.data)
        self._keep = e

    def set_reaction(self, a):
        lib().oem_set_reaction(self._p, np.ascontiguousarray(a, np.float32))

    def update_config(self, dt, rel_tol, max_iterations):
        lib().oem_update_config(self._p, float(dt), float(rel_tol), int(max_iterations))

    def apply_nodal(self, r):
        out = np.zeros(self.edges, np.float32)
        lib().oem_apply_nodal(self._p, np.ascontiguousarray(r, np.float32), out)
        return out

    def set_previous(self, a):
        lib().oem_set_previous(self._p, np.ascontiguousarray(a, np.float32))

    def set_predict(self, on):
        lib().oem_set_predict(self._p, int(bool(on)))

    def prediction(self):
        out = np.zeros(3, np.float32)
        lib().oem_prediction(self._p, out)
        return out

    def time(self):
        out = np.zeros(2, np.float64)
        lib().oem_time(self._p, out)
        return float(out[0]), float(out[1])

    def evaluate_sources(self, elements):
        el = np.ascontiguousarray(elements, np.float32).reshape(-1, 12)
        out = np.zeros(self.edges, np.float32)
        lib().oem_evaluate_sources(self._p, el.reshape(-1) if el.size else np.zeros(12, np.float32), el.shape[0],
                                   out)
        return out

    ENERGY_KEYS = ("magnetic_j", "delta_magnetic_j", "backward_euler_j", "joule_j", "mechanical_j", "external_j",
                   "balance_error_j")

    def energy(self):
        out = np.zeros(7, np.float64)
        if lib().oem_energy(self._p, out) != 0:
            raise ValueError("Nonfinite EM energy integral")
        return dict(zip(self.ENERGY_KEYS, out.tolist()))

    def body_forces(self, masks, bodies):
        out = np.zeros((bodies, 4), np.float32)
        lib().oem_body_forces(self._p, np.ascontiguousarray(masks, np.uint32).reshape(-1), bodies, out.reshape(-1))
        return out

    def set_motion(self, fluid_cells):
        lib().oem_set_motion(self._p, np.ascontiguousarray(fluid_cells, np.float32).reshape(-1))

    def work(self):
        out = np.zeros((self.edges, 4), np.float32)
        lib().oem_get(self._p, 0, out)
        return out

    def reaction(self):
        return self.work()[:, 0].copy()

    def previous(self):
        out = np.zeros(self.edges, np.float32)
        lib().oem_get(self._p, 1, out)
        return out

    def source(self):
        out = np.zeros((2 * self.edges, 4), np.float32)
        lib().oem_get(self._p, 2, out)
        return out

    def results(self):
        out = np.zeros((self.cells, 16), np.float32)
        lib().oem_get(self._p, 3, out)
        return out

    def scalars(self):
        out = np.zeros(32, np.float32)
        lib().oem_get(self._p, 4, out)
        return out

    def apply_operator(self, p, use_air=True):
        q = np.zeros(self.edges, np.float32)
        lib().oem_apply_operator(self._p, np.ascontiguousarray(p, np.float32), q, int(bool(use_air)))
        return q

    def advance(self, time_s, initial=False, applied=None):
        """Returns (code, status[8], stats[16])."""
        a = None if applied is None else np.ascontiguousarray(applied, np.float32)
        st = np.zeros(8, np.float32)
        stats = np.zeros(16, np.float32)
        rc = lib().oem_advance(self._p, float(time_s), int(bool(initial)), None if a is None else a.ctypes.data,
                               st, stats)
        return rc, st, stats


def em_edge_dims(dims, axis):
    d = [v + 1 for v in dims]
    d[axis] -= 1
    return tuple(d)
