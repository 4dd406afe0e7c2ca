"""Python mirror of the projection interface, over the C ABI of libmhdproj.so.

The reference's projection is a private Rust method,
``FluidState::project(warm_start) -> Result<(u32 iterations, f32 residual), String>``
(src/fluid/mod.rs:1015-1115), working on buffers its ``FluidState`` owns.  This
module keeps that shape: a :class:`PressureProjection` owns the solver state,
:meth:`PressureProjection.set_coefficients` plays the part of the coefficient
cache and gauge set-up (pressure_coefficients, anchors), and
:meth:`PressureProjection.project` returns ``(iterations, residual)`` or raises
:class:`ProjectionError` with the reference's messages.

Device memory comes from torch (CUDA tensors, passed as raw pointers); the
CUDA work is the library's own kernels.  There is no CPU fallback: without a
built library or a GPU every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmhdproj.so")

SOLVERS = {"reference": 0, "gb300": 1}
PRECISIONS = {"fp32": 0, "fp16": 1, "bf16": 2}
PRECONDITIONERS = {"auto": -1, "jacobi": 0, "multigrid": 1}
STATUS = {
    0: "ok",
    1: "invalid argument",
    2: "CUDA error",
    3: "not converged",
    4: "non-finite residual",
    5: "no progress",
    6: "call order",
    7: "out of memory",
    8: "timeout",
}


class Grid(C.Structure):
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32), ("h", C.c_float),
                ("periodic", C.c_uint32), ("boundary", C.c_int32)]


class Options(C.Structure):
    _fields_ = [("solver", C.c_int32), ("precision", C.c_int32), ("preconditioner", C.c_int32),
                ("rel_tol", C.c_float), ("abs_div_tol", C.c_float), ("max_iterations", C.c_uint32),
                ("max_refinements", C.c_int32), ("two_phase", C.c_int32), ("gauge", C.c_int32),
                ("compute_divergence", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("iterations", C.c_uint32), ("refinements", C.c_uint32), ("relative_residual", C.c_float),
                ("true_relative_residual", C.c_double), ("max_divergence", C.c_double),
                ("rms_divergence", C.c_double), ("elapsed_ms", C.c_float), ("meanfree", C.c_int32),
                ("multigrid", C.c_int32), ("levels", C.c_uint32), ("coarse_cells", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Diagnostics(C.Structure):
    """mhdproj_diagnostics: FluidDiagnostics plus the CFL inputs of the next step."""
    _fields_ = [("max_speed_m_s", C.c_float), ("max_divergence_s_inv", C.c_float),
                ("rms_divergence_s_inv", C.c_float), ("max_pressure_pa", C.c_float),
                ("kinetic_energy_j", C.c_float), ("fluid_mass_kg", C.c_float), ("net_flux_m3_s", C.c_float),
                ("max_force_density", C.c_float), ("max_face_speed_m_s", C.c_float),
                ("nonfinite_cells", C.c_uint32), ("viscous_substeps", C.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class StepParams(C.Structure):
    _fields_ = [("dt", C.c_float), ("acceleration", C.c_float * 3), ("kinematic_viscosity", C.c_float),
                ("advection", C.c_int32), ("surface_tension", C.c_float), ("air_viscosity", C.c_float),
                ("max_viscous_substeps", C.c_uint32), ("curvature", C.c_void_p)]


class EmConfig(C.Structure):
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32), ("cell_m", C.c_float),
                ("origin_m", C.c_float * 3), ("dt_s", C.c_double), ("relative_tolerance", C.c_float),
                ("max_iterations", C.c_uint32), ("mode", C.c_int32), ("nodal_switch_after", C.c_uint32)]


class EmDiagnostics(C.Structure):
    _fields_ = [("maxima", C.c_float * 4), ("force_n", C.c_float * 3), ("power_w", C.c_float),
                ("divergence_j_scaled", C.c_float), ("max_edge_j", C.c_float), ("divergence_b_scaled", C.c_float),
                ("magnetic_energy_j", C.c_float), ("applied_max_t", C.c_float), ("reaction_max_t", C.c_float),
                ("iterations", C.c_uint32), ("relative_residual", C.c_float), ("conductivity_range", C.c_float * 2),
                ("device_ms", C.c_float), ("elapsed_ms", C.c_double), ("status", C.c_float * 8)]

    def stats(self):
        """The 16 field statistics in the reference's scalars[2..5] order."""
        return np.array(list(self.maxima) + list(self.force_n) + [self.power_w, self.divergence_j_scaled,
                        self.max_edge_j, self.divergence_b_scaled, self.magnetic_energy_j, self.applied_max_t,
                        self.reaction_max_t, 0.0, 0.0], np.float32)


class KernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("ms", C.c_float), ("bytes", C.c_double), ("per_iteration", C.c_int)]


class ProjectionError(RuntimeError):
    """A failed projection; ``code`` is the mhdproj_status value."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code
        self.status = STATUS.get(code, "unknown")


_lib = None
_vp = C.c_void_p


def load():
    """Load libmhdproj.so (built by ``mhdproj.build.build()``).  Raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with mhdproj.build.build() (needs nvcc)")
    L = C.CDLL(LIB_PATH)
    L.mhdproj_default_options.argtypes = [C.POINTER(Options)]
    L.mhdproj_create.argtypes = [C.POINTER(Grid), C.POINTER(Options), C.POINTER(_vp)]
    L.mhdproj_destroy.argtypes = [_vp]
    L.mhdproj_last_error.argtypes = [_vp]
    L.mhdproj_last_error.restype = C.c_char_p
    L.mhdproj_set_stream.argtypes = [_vp, _vp]
    L.mhdproj_set_coefficients.argtypes = [_vp, _vp, _vp, C.c_float, C.c_float]
    L.mhdproj_set_phase_drag.argtypes = [_vp, _vp, C.c_float, C.c_float]
    L.mhdproj_project.argtypes = [_vp] + [_vp] * 7 + [C.c_float, C.c_int, C.POINTER(Stats)]
    L.mhdproj_project_host.argtypes = [_vp, _vp, _vp, C.c_float, C.c_float] + [_vp] * 7 + [C.c_float, C.c_int,
                                                                                          C.POINTER(Stats)]
    L.mhdproj_project_vjp.argtypes = [_vp] + [_vp] * 4 + [C.c_float] + [_vp] * 3 + [C.POINTER(Stats)]
    L.mhdproj_chain_forward.argtypes = [_vp] + [_vp] * 6 + [C.c_float, C.c_int, C.c_int] + [_vp] * 3 + [
        C.POINTER(C.c_double), C.POINTER(Stats)]
    L.mhdproj_chain_backward.argtypes = [_vp, _vp, _vp, _vp, C.POINTER(Stats)]
    L.mhdproj_chain_set_objective.argtypes = [_vp, C.c_int]
    L.mhdproj_apply_operator.argtypes = [_vp, _vp, _vp]
    L.mhdproj_apply_preconditioner.argtypes = [_vp, _vp, _vp]
    L.mhdproj_copy_coefficients.argtypes = [_vp, _vp]
    L.mhdproj_copy_potential.argtypes = [_vp, _vp]
    L.mhdproj_copy_topology.argtypes = [_vp, _vp, C.POINTER(C.c_uint32)]
    L.mhdproj_profile_kernels.argtypes = [_vp, C.c_int, C.POINTER(KernelTime), C.c_int, C.POINTER(C.c_int)]
    L.mhdproj_divergence_noalloc.argtypes = [C.POINTER(Grid), _vp, _vp, _vp, _vp, C.POINTER(C.c_double), _vp]
    L.mhdproj_kernel_launches.argtypes = [_vp, C.POINTER(C.c_uint64)]
    L.mhdproj_hierarchy.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)]
    L.mhdproj_anchors.argtypes = [_vp, C.POINTER(C.c_uint32), C.c_uint32]
    L.mhdproj_anchors.restype = C.c_uint32
    L.mhdproj_fields.argtypes = [_vp] + [_vp] * 4 + [C.POINTER(C.c_float * 3), C.c_float, _vp,
                                                     C.POINTER(Diagnostics)]
    L.mhdproj_fluid_step.argtypes = [_vp] + [_vp] * 4 + [C.POINTER(StepParams), _vp, _vp, C.POINTER(Stats),
                                                         C.POINTER(Diagnostics)]
    L.mhdproj_export_fields.argtypes = [C.POINTER(Grid), _vp, C.c_char_p, C.c_uint64, C.c_double,
                                        C.POINTER(C.c_float * 3), C.c_int, C.c_char_p]
    L.mhdproj_classify_cells.argtypes = [C.POINTER(Grid), _vp, C.c_uint32, _vp, C.c_uint32, _vp, C.c_uint32, _vp,
                                         _vp, _vp, C.POINTER(C.c_uint32), _vp]
    L.mhdproj_classify_last_error.argtypes = []
    L.mhdproj_classify_last_error.restype = C.c_char_p
    L.mhdproj_em_create.argtypes = [C.POINTER(EmConfig), C.POINTER(_vp)]
    L.mhdproj_em_destroy.argtypes = [_vp]
    L.mhdproj_em_update_config.argtypes = [_vp, C.POINTER(EmConfig)]
    L.mhdproj_em_last_error.argtypes = [_vp]
    L.mhdproj_em_last_error.restype = C.c_char_p
    L.mhdproj_em_set_stream.argtypes = [_vp, _vp]
    L.mhdproj_em_sizes.argtypes = [_vp, C.POINTER(C.c_uint64 * 8)]
    L.mhdproj_em_set_materials.argtypes = [_vp, _vp, _vp, C.c_uint32, C.POINTER(C.c_float * 2)]
    L.mhdproj_em_set_motional_emf.argtypes = [_vp, _vp]
    L.mhdproj_em_set_reaction.argtypes = [_vp, _vp]
    L.mhdproj_em_set_motion.argtypes = [_vp, _vp]
    L.mhdproj_em_evaluate_sources.argtypes = [_vp, _vp, C.c_uint32, _vp]
    L.mhdproj_em_body_forces.argtypes = [_vp, _vp, C.c_uint32, _vp]
    L.mhdproj_em_energy.argtypes = [_vp, _vp]
    L.mhdproj_em_advance.argtypes = [_vp, C.c_double, C.c_int, _vp, C.POINTER(EmDiagnostics)]
    L.mhdproj_em_copy.argtypes = [_vp, C.c_int, _vp]
    L.mhdproj_em_apply_operator.argtypes = [_vp, _vp, _vp, C.c_int]
    L.mhdproj_em_kernel_launches.argtypes = [_vp, C.POINTER(C.c_uint64)]
    _lib = L
    return L


EXPORTED = [
    "mhdproj_default_options", "mhdproj_create", "mhdproj_destroy", "mhdproj_last_error", "mhdproj_set_stream",
    "mhdproj_set_coefficients", "mhdproj_set_phase_drag", "mhdproj_project", "mhdproj_project_host",
    "mhdproj_project_vjp", "mhdproj_chain_forward", "mhdproj_chain_backward", "mhdproj_chain_set_objective",
    "mhdproj_apply_operator",
    "mhdproj_apply_preconditioner", "mhdproj_copy_coefficients", "mhdproj_copy_potential", "mhdproj_copy_topology",
    "mhdproj_hierarchy", "mhdproj_anchors", "mhdproj_profile_kernels", "mhdproj_divergence_noalloc",
    "mhdproj_kernel_launches", "mhdproj_fields", "mhdproj_fluid_step", "mhdproj_export_fields",
    "mhdproj_classify_cells", "mhdproj_classify_last_error",
    "mhdproj_em_create", "mhdproj_em_update_config", "mhdproj_em_destroy", "mhdproj_em_last_error", "mhdproj_em_set_stream", "mhdproj_em_sizes",
    "mhdproj_em_set_materials", "mhdproj_em_set_motional_emf", "mhdproj_em_set_motion", "mhdproj_em_evaluate_sources", "mhdproj_em_body_forces", "mhdproj_em_energy", "mhdproj_em_set_reaction", "mhdproj_em_advance",
    "mhdproj_em_copy", "mhdproj_em_apply_operator", "mhdproj_em_kernel_launches",
]


def divergence_noalloc(dims, h, solid, u, v, w, stream=None, periodic=0):
    """Max and RMS divergence (1/s) of a face field over non-solid cells, with
    no device allocation (mhdproj_divergence_noalloc).  periodic: bit a set
    reads the high face of the last cell on axis a at face 0."""
    import torch

    L = load()
    nx, ny, nz = (int(d) for d in dims)
    want = (("solid", solid, (nz, ny, nx), torch.uint8), ("u", u, (nz, ny, nx + 1), torch.float32),
            ("v", v, (nz, ny + 1, nx), torch.float32), ("w", w, (nz + 1, ny, nx), torch.float32))
    for name, a, shape, dtype in want:
        if not (a.is_cuda and a.is_contiguous()) or a.dtype != dtype or a.numel() != shape[0] * shape[1] * shape[2]:
            raise ValueError(f"divergence_noalloc: {name} must be a contiguous CUDA {dtype} tensor of shape {shape}")
        if a.dim() == 3 and tuple(a.shape) != shape:
            raise ValueError(f"divergence_noalloc: {name} has shape {tuple(a.shape)}, expected {shape}")
    g = Grid(nx, ny, nz, float(h), int(periodic), 0)
    out = (C.c_double * 2)()
    s = stream if stream is not None else torch.cuda.current_stream()
    s.synchronize()
    rc = L.mhdproj_divergence_noalloc(C.byref(g), _ptr(solid), _ptr(u), _ptr(v), _ptr(w), out,
                                      C.c_void_p(s.cuda_stream))
    if rc:
        raise ProjectionError(rc, L.mhdproj_last_error(None).decode())
    return out[0], out[1]


def export_fields(dims, h, cells, directory, step=0, time_s=0.0, origin_m=(0.0, 0.0, 0.0), moving_interface=False,
                  forcing_kind="none"):
    """Write a frame directory (fluid.bin + metadata.json) from device cell
    records (mhdproj_export_fields); raises ProjectionError on failure."""
    L = load()
    g = Grid(int(dims[0]), int(dims[1]), int(dims[2]), float(h), 0, 0)
    o = (C.c_float * 3)(*origin_m)
    rc = L.mhdproj_export_fields(C.byref(g), _ptr(cells), os.fsencode(directory), int(step), float(time_s),
                                 C.byref(o), int(bool(moving_interface)), forcing_kind.encode())
    if rc:
        raise ProjectionError(rc, L.mhdproj_last_error(None).decode())


def classify_cells(dims, materials, liquid_material, mask, cells, thermal=None, thermal_stride=1, interface=None,
                   interface_stride=2, stream=None):
    """The phase/surface passes of FluidState::update_cells
    (src/fluid/phase.wgsl:10-31) on CUDA tensors: updates the 0/1 mobility
    ``mask`` (int32/uint32 storage, one per cell) and the FluidCell
    ``cells`` records (16 floats per cell) in place; returns the changed
    flags (bit 0: some cell's mobility changed).  Raises ProjectionError with
    the reference's message for an interface fraction out of [0, 1]."""
    import torch

    L = load()
    g = Grid(int(dims[0]), int(dims[1]), int(dims[2]), 1.0, 0, 0)
    scratch = torch.zeros(1, dtype=torch.int32, device=mask.device)
    changed = C.c_uint32()
    s = torch.cuda.current_stream() if stream is None else stream
    rc = L.mhdproj_classify_cells(C.byref(g), _ptr(materials), int(liquid_material), _ptr(thermal),
                                  int(thermal_stride), _ptr(interface), int(interface_stride), _ptr(mask),
                                  _ptr(cells), _ptr(scratch), C.byref(changed), C.c_void_p(s.cuda_stream))
    if rc:
        raise ProjectionError(rc, L.mhdproj_classify_last_error().decode())
    return int(changed.value)


def hierarchy(dims4):
    """hierarchy() of src/fluid/multigrid.rs:25-65: (levels, coarse cells); raises on rejected grids."""
    L = load()
    d = (C.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in dims4])
    nl, cc = C.c_uint32(), C.c_uint64()
    if L.mhdproj_hierarchy(d, C.byref(nl), C.byref(cc)):
        raise ValueError("Invalid pressure grid dimensions")
    return nl.value, cc.value


def anchors(mask, dims, periodic_bits=0):
    """anchors() of src/fluid/mod.rs:1447-1493 on a 0/1 mask: (components, encoded mask)."""
    L = load()
    m = np.ascontiguousarray(mask, dtype=np.uint32).reshape(-1).copy()
    comps = L.mhdproj_anchors(m.ctypes.data_as(_vp), (C.c_uint32 * 3)(*dims), periodic_bits)
    return int(comps), m


def _ptr(t):
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return C.c_void_p(t.data_ptr())


def _host_ptr(a):
    return None if a is None else a.ctypes.data_as(_vp)


class PressureProjection:
    """One projection context (mhdproj_ctx) on the current CUDA device.

    dims = (nx, ny, nz); h the cell size in metres; periodic a triple of
    booleans; outlet selects a Dirichlet p = 0 top z-face.  Face velocity
    tensors have shapes (nz, ny, nx+1), (nz, ny+1, nx), (nz+1, ny, nx); cell
    tensors (nz, ny, nx).
    """

    def __init__(self, dims, h, periodic=(False, False, False), outlet=True, solver="gb300", precision="fp16",
                 preconditioner="auto", rel_tol=1e-6, abs_div_tol=0.0, max_iterations=20000, max_refinements=4,
                 two_phase=True, gauge=-1, compute_divergence=False, stream=None):
        import torch

        self._torch = torch
        L = load()
        self.dims = tuple(int(d) for d in dims)
        self.h = float(h)
        bits = sum(1 << a for a, p in enumerate(periodic) if p)
        self.periodic_bits = bits
        g = Grid(self.dims[0], self.dims[1], self.dims[2], self.h, bits, 1 if outlet else 0)
        o = Options()
        L.mhdproj_default_options(C.byref(o))
        o.solver = SOLVERS[solver]
        o.precision = PRECISIONS[precision]
        o.preconditioner = PRECONDITIONERS[preconditioner]
        o.rel_tol = rel_tol
        o.abs_div_tol = abs_div_tol
        o.max_iterations = max_iterations
        o.max_refinements = max_refinements
        o.two_phase = int(two_phase)
        o.gauge = gauge
        o.compute_divergence = int(compute_divergence)
        self.options = o
        h_ = C.c_void_p()
        rc = L.mhdproj_create(C.byref(g), C.byref(o), C.byref(h_))
        if rc:
            raise ProjectionError(rc, L.mhdproj_last_error(None).decode())
        self._ctx = h_
        self._lib = L
        # The library works on a non-default stream (CUDA graphs cannot be
        # captured on the legacy default stream); every call first orders it
        # after torch's current stream, and returns with its own stream idle.
        if stream is None or stream.cuda_stream == 0:
            stream = torch.cuda.Stream()
        self.stream = stream
        self._check(L.mhdproj_set_stream(self._ctx, C.c_void_p(stream.cuda_stream)))
        self.solver = solver
        self.device = torch.device("cuda", torch.cuda.current_device())
        # bumped by every coefficient change; the autograd pair checks it
        self.coefficient_generation = 0

    # ------------------------------------------------------------ helpers
    def _order(self):
        cur = self._torch.cuda.current_stream()
        if cur.cuda_stream != self.stream.cuda_stream:
            self.stream.wait_stream(cur)

    def _check(self, rc):
        if rc:
            raise ProjectionError(rc, self._lib.mhdproj_last_error(self._ctx).decode())

    def face_shapes(self):
        nx, ny, nz = self.dims
        return (nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx)

    def cell_shape(self):
        nx, ny, nz = self.dims
        return (nz, ny, nx)

    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.mhdproj_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------- interface
    def set_coefficients(self, alpha, solid, rho_liquid, rho_air):
        self._order()
        self.coefficient_generation += 1
        self._check(self._lib.mhdproj_set_coefficients(self._ctx, _ptr(alpha), _ptr(solid), rho_liquid, rho_air))

    def set_phase_drag(self, phase, drag_rate, dt):
        self._order()
        self.coefficient_generation += 1
        self._check(self._lib.mhdproj_set_phase_drag(self._ctx, _ptr(phase), drag_rate, dt))

    def project(self, u_star, dt, warm_start=False, out=None, pressure=True):
        """Project (u*, v*, w*) -> ((u, v, w), p, stats)."""
        self._order()
        torch = self._torch
        if out is None:
            out = tuple(torch.empty_like(t) for t in u_star)
        p = torch.empty(self.cell_shape(), dtype=torch.float32, device=u_star[0].device) if pressure else None
        st = Stats()
        self._check(self._lib.mhdproj_project(self._ctx, *[_ptr(t) for t in u_star], *[_ptr(t) for t in out],
                                              _ptr(p), dt, int(warm_start), C.byref(st)))
        return out, p, st

    def project_host(self, alpha, solid, rho_liquid, rho_air, u_star, dt, warm_start=False, out=None, p_out=None):
        """The same call on numpy host arrays (copies inside the call)."""
        if out is None:
            out = tuple(np.empty_like(a) for a in u_star)
        if p_out is None:
            p_out = np.empty(self.cell_shape(), np.float32)
        st = Stats()
        self._check(self._lib.mhdproj_project_host(self._ctx, _host_ptr(alpha), _host_ptr(solid), rho_liquid, rho_air,
                                                   *[_host_ptr(a) for a in u_star], *[_host_ptr(a) for a in out],
                                                   _host_ptr(p_out), dt, int(warm_start), C.byref(st)))
        return out, p_out, st

    def vjp(self, grad_u, grad_p, dt):
        self._order()
        torch = self._torch
        out = tuple(torch.empty_like(t) for t in grad_u)
        st = Stats()
        self._check(self._lib.mhdproj_project_vjp(self._ctx, *[_ptr(t) for t in grad_u], _ptr(grad_p), dt,
                                                  *[_ptr(t) for t in out], C.byref(st)))
        return out, st

    def chain_forward(self, u0, force, dt, steps, checkpoint_every=4):
        self._order()
        torch = self._torch
        uf = tuple(torch.empty_like(t) for t in u0)
        J = C.c_double()
        st = Stats()
        self._check(self._lib.mhdproj_chain_forward(self._ctx, *[_ptr(t) for t in u0], *[_ptr(t) for t in force], dt,
                                                    steps, checkpoint_every, *[_ptr(t) for t in uf], C.byref(J),
                                                    C.byref(st)))
        return uf, J.value, st

    CHAIN_OBJECTIVES = {"final": 0, "summed": 1}

    def chain_set_objective(self, kind):
        """'final': J = sum of w^2 over the outlet faces of the final state
        (the default); 'summed': that sum over the states after every step,
        whose backward pass recomputes the states between checkpoints."""
        if kind not in self.CHAIN_OBJECTIVES:
            raise ValueError(f"chain objective must be one of {sorted(self.CHAIN_OBJECTIVES)}")
        self._check(self._lib.mhdproj_chain_set_objective(self._ctx, self.CHAIN_OBJECTIVES[kind]))

    def chain_backward(self, like):
        self._order()
        torch = self._torch
        g = tuple(torch.empty_like(t) for t in like)
        st = Stats()
        self._check(self._lib.mhdproj_chain_backward(self._ctx, *[_ptr(t) for t in g], C.byref(st)))
        return g, st

    def apply_operator(self, x):
        self._order()
        y = self._torch.empty_like(x)
        self._check(self._lib.mhdproj_apply_operator(self._ctx, _ptr(x), _ptr(y)))
        return y

    def apply_preconditioner(self, r):
        self._order()
        z = self._torch.empty_like(r)
        self._check(self._lib.mhdproj_apply_preconditioner(self._ctx, _ptr(r), _ptr(z)))
        return z

    def coefficients(self):
        self._order()
        torch = self._torch
        c = torch.empty(self.cell_shape() + (4,), dtype=torch.float32, device=self.device)
        self._check(self._lib.mhdproj_copy_coefficients(self._ctx, _ptr(c)))
        return c

    def potential(self):
        self._order()
        torch = self._torch
        phi = torch.empty(self.cell_shape(), dtype=torch.float64, device=self.device)
        self._check(self._lib.mhdproj_copy_potential(self._ctx, _ptr(phi)))
        return phi

    def kernel_launches(self):
        """Kernels this context has launched since creation (mhdproj_kernel_launches)."""
        n = C.c_uint64()
        self._check(self._lib.mhdproj_kernel_launches(self._ctx, C.byref(n)))
        return int(n.value)

    def profile_kernels(self, reps=20):
        """Per-kernel mean launch time (ms), algorithmic bytes and launches per CG iteration."""
        buf = (KernelTime * 16)()
        n = C.c_int()
        self._check(self._lib.mhdproj_profile_kernels(self._ctx, reps, buf, 16, C.byref(n)))
        return [dict(name=buf[i].name.decode(), ms=buf[i].ms, bytes=buf[i].bytes, per_iteration=buf[i].per_iteration)
                for i in range(n.value)]

    def fields(self, u, dt, em_force=None, acceleration=(0.0, 0.0, 0.0), cells=True):
        """fields + diagnostics (mhdproj_fields) of face velocities u = (u, v, w)
        with the last pressure potential: returns (cells (nz, ny, nx, 16) or
        None, diagnostics dict).  em_force: (nz, ny, nx, 4) force density."""
        self._order()
        torch = self._torch
        out = torch.empty(self.cell_shape() + (16,), dtype=torch.float32, device=u[0].device) if cells else None
        d = Diagnostics()
        acc = (C.c_float * 3)(*acceleration)
        self._check(self._lib.mhdproj_fields(self._ctx, _ptr(u[0]), _ptr(u[1]), _ptr(u[2]),
                                             None if em_force is None else _ptr(em_force), C.byref(acc), dt,
                                             None if out is None else _ptr(out), C.byref(d)))
        return out, d.as_dict()

    def fluid_step(self, u, dt, acceleration=(0.0, 0.0, -9.81), viscosity=0.0, advection=True, em_force=None,
                   p_out=None, cells=None, surface_tension=0.0, air_viscosity=0.0, max_viscous_substeps=4096,
                   curvature=None):
        """One FluidState::step (mhdproj_fluid_step) in place on u = (u, v, w):
        returns (stats dict, diagnostics dict).  p_out / cells: optional
        device outputs (cells shaped (nz, ny, nx, 16)).  surface_tension,
        air_viscosity, max_viscous_substeps and curvature (a cell tensor)
        apply with a moving interface."""
        self._order()
        sp = StepParams(dt, (C.c_float * 3)(*acceleration), viscosity, int(bool(advection)), surface_tension,
                        air_viscosity, max_viscous_substeps,
                        None if curvature is None else _ptr(curvature).value)
        st = Stats()
        d = Diagnostics()
        self._check(self._lib.mhdproj_fluid_step(self._ctx, _ptr(u[0]), _ptr(u[1]), _ptr(u[2]),
                                                 None if em_force is None else _ptr(em_force), C.byref(sp),
                                                 None if p_out is None else _ptr(p_out),
                                                 None if cells is None else _ptr(cells), C.byref(st), C.byref(d)))
        return st.as_dict(), d.as_dict()

    def topology(self):
        n = self.dims[0] * self.dims[1] * self.dims[2]
        m = np.zeros(n, np.uint32)
        comps = C.c_uint32()
        self._check(self._lib.mhdproj_copy_topology(self._ctx, m.ctypes.data_as(_vp), C.byref(comps)))
        return m, comps.value


def autograd_projection():
    """torch.autograd.Function pair over forward projection and its VJP:
    ``ProjectFn.apply(proj, dt, u, v, w) -> (u', v', w', p)``.

    The projection is linear in (u, v, w) for fixed coefficients, so the
    backward pass needs only the coefficients the forward pass used.  It
    refuses (RuntimeError) when the context's coefficients changed between
    forward and backward, instead of returning the VJP of another operator.
    Missing output gradients are zeros on the projection's device."""
    import torch

    class ProjectFn(torch.autograd.Function):
        @staticmethod
        def forward(ctx, proj, dt, u, v, w):
            (uo, vo, wo), p, _ = proj.project((u.contiguous(), v.contiguous(), w.contiguous()), dt)
            ctx.proj = proj
            ctx.dt = dt
            ctx.generation = proj.coefficient_generation
            return uo, vo, wo, p

        @staticmethod
        def backward(ctx, gu, gv, gw, gp):
            proj = ctx.proj
            if proj.coefficient_generation != ctx.generation:
                raise RuntimeError("the projection's coefficients changed between forward and backward; "
                                   "the VJP would belong to another operator")
            grads = [g.contiguous() if g is not None else None for g in (gu, gv, gw)]
            shapes = proj.face_shapes()
            grads = [g if g is not None else torch.zeros(s, dtype=torch.float32, device=proj.device)
                     for g, s in zip(grads, shapes)]
            (a, b, c), _ = proj.vjp(tuple(grads), gp.contiguous() if gp is not None else None, ctx.dt)
            return None, None, a, b, c

    return ProjectFn


EM_MODES = {"induction": 0, "applied": 1}
EM_ARRAYS = {"reaction": 0, "previous": 1, "applied": 2, "cells": 3, "work": 4, "coefficients": 5}


class EmInduction:
    """The EM induction state (mhdproj_em_ctx), mirroring EmState
    (src/em/mod.rs): :meth:`set_materials` is the coefficient build of
    ``EmState::new`` / ``update_material_geometry``, :meth:`advance` is
    ``advance_to`` with the applied potential A_s supplied by the caller,
    :meth:`step` is ``EmState::step`` (one ``dt_s`` further).

    Edge arrays are flat float32 CUDA tensors of ``edges`` entries (x-edges,
    y-edges, z-edges, each x-fastest); cell results are ``(cells, 16)``.
    """

    def __init__(self, dims, cell_m, dt_s=1e-5, relative_tolerance=1e-5, max_iterations=1000,
                 origin_m=(0.0, 0.0, 0.0), mode="induction", nodal_switch_after=1024, stream=None):
        import torch

        self._torch = torch
        L = load()
        cfg = EmConfig(int(dims[0]), int(dims[1]), int(dims[2]), float(cell_m), (C.c_float * 3)(*origin_m),
                       float(dt_s), float(relative_tolerance), int(max_iterations), EM_MODES[mode],
                       int(nodal_switch_after))
        h_ = C.c_void_p()
        rc = L.mhdproj_em_create(C.byref(cfg), C.byref(h_))
        if rc:
            raise ProjectionError(rc, L.mhdproj_em_last_error(None).decode())
        self._ctx = h_
        self._lib = L
        self.config = cfg
        self.dt_s = float(dt_s)
        self.time_s = 0.0
        if stream is None or stream.cuda_stream == 0:
            stream = torch.cuda.Stream()
        self.stream = stream
        self._check(L.mhdproj_em_set_stream(self._ctx, C.c_void_p(stream.cuda_stream)))
        sz = (C.c_uint64 * 8)()
        self._check(L.mhdproj_em_sizes(self._ctx, C.byref(sz)))
        self.dims = tuple(int(v) for v in sz[:3])
        self.cells = int(sz[3])
        self.edge_counts = tuple(int(v) for v in sz[4:7])
        self.edges = int(sz[7])

    def _order(self):
        cur = self._torch.cuda.current_stream()
        if cur.cuda_stream != self.stream.cuda_stream:
            self.stream.wait_stream(cur)

    def _check(self, rc):
        if rc:
            raise ProjectionError(rc, self._lib.mhdproj_em_last_error(self._ctx).decode())

    def update_config(self, dt_s=None, relative_tolerance=None, max_iterations=None, nodal_switch_after=None):
        """Changes the EmConfig fields the reference lets a caller change."""
        c = self.config
        if dt_s is not None:
            c.dt_s = float(dt_s)
        if relative_tolerance is not None:
            c.relative_tolerance = float(relative_tolerance)
        if max_iterations is not None:
            c.max_iterations = int(max_iterations)
        if nodal_switch_after is not None:
            c.nodal_switch_after = int(nodal_switch_after)
        self._check(self._lib.mhdproj_em_update_config(self._ctx, C.byref(c)))
        self.dt_s = float(c.dt_s)

    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.mhdproj_em_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_materials(self, materials, properties):
        """materials: uint32-valued CUDA tensor (cells), int32 accepted;
        properties: rows of (conductivity S/m, relative permeability) per id.
        Returns the conducting-edge conductivity range."""
        self._order()
        m = materials.contiguous()
        pr = np.ascontiguousarray(properties, np.float32).reshape(-1, 2)
        rng = (C.c_float * 2)()
        self._check(self._lib.mhdproj_em_set_materials(self._ctx, _ptr(m), _host_ptr(pr), pr.shape[0],
                                                       C.byref(rng)))
        self._materials = m
        return float(rng[0]), float(rng[1])

    def set_motional_emf(self, emf=None):
        self._order()
        self._check(self._lib.mhdproj_em_set_motional_emf(self._ctx, _ptr(emf)))

    def set_reaction(self, a):
        self._order()
        self._check(self._lib.mhdproj_em_set_reaction(self._ctx, _ptr(a.contiguous())))

    def evaluate_sources(self, elements):
        """The applied potential (edges) of source elements, an (n, 12)
        float32 array on the host (EmConfig::elements records)."""
        el = np.ascontiguousarray(elements, np.float32).reshape(-1, 12)
        out = self._torch.empty(self.edges, dtype=self._torch.float32, device="cuda")
        self._order()
        self._check(self._lib.mhdproj_em_evaluate_sources(self._ctx, _host_ptr(el) if el.size else None, el.shape[0],
                                                          _ptr(out)))
        return out

    ENERGY_KEYS = ("magnetic_j", "delta_magnetic_j", "backward_euler_j", "joule_j", "mechanical_j", "external_j",
                   "balance_error_j")

    def energy(self):
        """EmState::energy_step: the energy ledger of the last step (J)."""
        out = np.zeros(7, np.float64)
        self._order()
        self._check(self._lib.mhdproj_em_energy(self._ctx, _host_ptr(out)))
        return dict(zip(self.ENERGY_KEYS, out.tolist()))

    def body_forces(self, masks, bodies):
        """(bodies, 4) float32: force xyz (N) and Joule power (W) of the last
        step for the cells with bit z of ``masks`` (int32 CUDA tensor)."""
        out = np.zeros((bodies, 4), np.float32)
        self._order()
        self._check(self._lib.mhdproj_em_body_forces(self._ctx, _ptr(masks.contiguous()), int(bodies),
                                                     _host_ptr(out)))
        return out

    def set_motion(self, fluid_cells):
        """EmState::set_velocity: the motional EMF from the fluid's
        (cells, 16) FluidCell records and this state's last B."""
        self._order()
        self._check(self._lib.mhdproj_em_set_motion(self._ctx, _ptr(fluid_cells.contiguous())))

    def advance(self, time_s, initial=False, applied=None):
        """One step to ``time_s``; returns :class:`EmDiagnostics`."""
        self._order()
        d = EmDiagnostics()
        a = None if applied is None else applied.contiguous()
        self._check(self._lib.mhdproj_em_advance(self._ctx, float(time_s), int(bool(initial)), _ptr(a),
                                                 C.byref(d)))
        self.time_s = float(time_s)
        return d

    def step(self, applied=None):
        return self.advance(self.time_s + self.dt_s, False, applied)

    def copy(self, which):
        torch = self._torch
        k = EM_ARRAYS[which]
        n = self.cells * 16 if k == 3 else self.edges * 4 if k in (4, 5) else self.edges
        out = torch.empty(n, dtype=torch.float32, device="cuda")
        self._order()
        self._check(self._lib.mhdproj_em_copy(self._ctx, k, _ptr(out)))
        if k == 3:
            return out.view(self.cells, 16)
        if k in (4, 5):
            return out.view(self.edges, 4)
        return out

    def apply_operator(self, p, air_stencil=True):
        q = self._torch.empty_like(p)
        self._order()
        self._check(self._lib.mhdproj_em_apply_operator(self._ctx, _ptr(p.contiguous()), _ptr(q),
                                                        int(bool(air_stencil))))
        return q

    def kernel_launches(self):
        n = C.c_uint64()
        self._check(self._lib.mhdproj_em_kernel_launches(self._ctx, C.byref(n)))
        return int(n.value)
