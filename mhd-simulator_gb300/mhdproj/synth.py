"""Seeded synthetic inputs for the projection workloads.

The reference measures no public benchmark or dataset for this path, so every
workload is a deterministic synthetic field: a counter-based splitmix64
stream per field (seed, field id), uniform doubles from the top 53 bits,
Box-Muller normals in double, cast to FP32.

Workloads (grid sizes at scale 1):
  jet64        64^3, h=0.1 mm, single-phase liquid rho=6440, solid outside a
               z-aligned cylinder of radius 28 cells, outlet on the top z-face,
               face velocities N(0, 0.05 m/s) zeroed on closed faces.
  jet128       128^3, h=0.05 mm, rho 6440:1.2.  Liquid fraction: tanh-smoothed
               (width 1.5 cells) union of a z-cylinder jet of radius 10 cells and
               a sphere drop of radius 16 cells at seeded offsets.  Solid nozzle:
               tapered annulus in the bottom 32 layers, inner radius 24 -> 12
               cells, outer radius = inner + 8 cells.  Velocities N(0, 0.2) where
               the face liquid fraction >= 1/2, N(0, 0.02) elsewhere.
  jet256       jet128 scaled 2x (h=0.025 mm, radii 20/32, width 3, annulus
               48 -> 24 over 64 layers, outer = inner + 16).
  adjoint128   jet128 plus a face body force N(0, 1e5 N/m^3) on liquid faces,
               dt = 1e-6 s.
  column512    512x256x256, h=0.025 mm, liquid column of radius 20 cells along
               x plus 4 seeded drops of radius 8..14 cells, no solids.
A ``scale`` argument shrinks a workload geometrically for oracle-sized tests.

EM workload (:func:`em_ring`): an n^3 box of 1 mm cells (origin at the box
centre) holding a conducting annulus about the z axis (radii 0.19 n and
0.38 n cells, the middle third of the height; conductivity 40 x 316
stainless, 5.33e7 S/m, relative permeability 1) in air, driven by a uniform
applied field B_z = 0.02 T sin(2 pi 1 kHz t) whose potential A_s = B x r / 2
is evaluated at the edge midpoints, dt = 1e-5 s -- the induction-heating
setting of the reference's EM tests (a conductor in a 16 mm box driven by a
uniform source) scaled to n.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix(z):
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform(seed: int, field: int, count: int) -> np.ndarray:
    """Uniform doubles in (0, 1) from a counter-based splitmix64 stream."""
    with np.errstate(over="ignore"):
        base = _mix(np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + np.uint64(field) * np.uint64(0xD1B54A32D192ED03))
        ctr = np.arange(1, count + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15) + base
        z = _mix(ctr)
    return ((z >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def normal(seed: int, field: int, count: int) -> np.ndarray:
    """Box-Muller normals (double) from two uniform streams."""
    u1 = uniform(seed, 2 * field + 1, count)
    u2 = uniform(seed, 2 * field + 2, count)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def _centres(n):
    return np.arange(n, dtype=np.float64) + 0.5


def _open_faces(solid, periodic=0, outlet=True):
    """Masks of open faces (both adjacent cells non-solid, or an outlet face)."""
    nz, ny, nx = solid.shape
    fluid = solid == 0
    fx = np.zeros((nz, ny, nx + 1), bool)
    fx[:, :, 1:nx] = fluid[:, :, :-1] & fluid[:, :, 1:]
    if periodic & 1:
        fx[:, :, 0] = fx[:, :, nx] = fluid[:, :, -1] & fluid[:, :, 0]
    fy = np.zeros((nz, ny + 1, nx), bool)
    fy[:, 1:ny, :] = fluid[:, :-1, :] & fluid[:, 1:, :]
    if periodic & 2:
        fy[:, 0, :] = fy[:, ny, :] = fluid[:, -1, :] & fluid[:, 0, :]
    fz = np.zeros((nz + 1, ny, nx), bool)
    fz[1:nz] = fluid[:-1] & fluid[1:]
    if periodic & 4:
        fz[0] = fz[nz] = fluid[-1] & fluid[0]
    elif outlet:
        fz[nz] = fluid[-1]
    return fx, fy, fz


def _face_alpha(alpha):
    nz, ny, nx = alpha.shape
    ax = np.zeros((nz, ny, nx + 1))
    ax[:, :, 1:nx] = 0.5 * (alpha[:, :, :-1] + alpha[:, :, 1:])
    ax[:, :, 0] = alpha[:, :, 0]
    ax[:, :, nx] = alpha[:, :, -1]
    ay = np.zeros((nz, ny + 1, nx))
    ay[:, 1:ny] = 0.5 * (alpha[:, :-1] + alpha[:, 1:])
    ay[:, 0] = alpha[:, 0]
    ay[:, ny] = alpha[:, -1]
    az = np.zeros((nz + 1, ny, nx))
    az[1:nz] = 0.5 * (alpha[:-1] + alpha[1:])
    az[0] = alpha[0]
    az[nz] = alpha[-1]
    return ax, ay, az


def _smooth(d, width):
    return 0.5 * (1.0 - np.tanh(d / width))


def _velocities(seed, alpha, solid, sd_liquid, sd_air, periodic=0, outlet=True, field0=10):
    out = []
    opens = _open_faces(solid, periodic, outlet)
    for a, (fa, op) in enumerate(zip(_face_alpha(alpha), opens)):
        z = normal(seed, field0 + a, fa.size).reshape(fa.shape)
        sd = np.where(fa >= 0.5, sd_liquid, sd_air)
        v = (z * sd).astype(np.float32)
        v[~op] = 0.0
        out.append(np.ascontiguousarray(v))
    return out


def _jet(n, scale, seed, h):
    """Two-phase jet + drop with a tapered annular nozzle (jet128 geometry at scale 1)."""
    c = _centres(n)
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    off = uniform(seed, 1, 5)
    mid = n / 2.0
    cx = mid + (off[0] * 8.0 - 4.0) * scale
    cy = mid + (off[1] * 8.0 - 4.0) * scale
    sx = mid + (off[2] * 16.0 - 8.0) * scale
    sy = mid + (off[3] * 16.0 - 8.0) * scale
    sz = n * 0.625 + (off[4] * 16.0 - 8.0) * scale
    w = 1.5 * scale
    d_cyl = np.sqrt((x - cx) ** 2 + (y - cy) ** 2) - 10.0 * scale
    d_sph = np.sqrt((x - sx) ** 2 + (y - sy) ** 2 + (z - sz) ** 2) - 16.0 * scale
    alpha = np.maximum(_smooth(d_cyl, w), _smooth(d_sph, w))
    r = np.sqrt((x - mid) ** 2 + (y - mid) ** 2)
    layers = 32.0 * scale
    inner = 24.0 * scale - 12.0 * scale * np.clip(z / layers, 0.0, 1.0)
    outer = inner + 8.0 * scale
    solid = ((z < layers) & (r >= inner) & (r <= outer)).astype(np.uint8)
    return alpha.astype(np.float32), solid


def make_case(name: str, seed: int = 1, scale: float = 1.0) -> dict:
    """Return a workload dict: dims (nx, ny, nz), h, rho_liquid, rho_air, alpha,
    solid, u, v, w (face arrays shaped (nz, ny, nx+1) etc.), dt, periodic,
    outlet, tol and (adjoint128) force fu, fv, fw."""
    if name == "jet64":
        n = int(round(64 * scale))
        h = 1e-4 / scale
        c = _centres(n)
        _, y, x = np.meshgrid(c, c, c, indexing="ij")
        solid = (np.sqrt((x - n / 2.0) ** 2 + (y - n / 2.0) ** 2) > 28.0 * scale).astype(np.uint8)
        alpha = np.ones((n, n, n), np.float32)
        u, v, w = _velocities(seed, alpha, solid, 0.05, 0.05)
        return dict(name=name, dims=(n, n, n), h=h, rho_liquid=6440.0, rho_air=6440.0, alpha=alpha, solid=solid,
                    u=u, v=v, w=w, dt=1e-5, periodic=0, outlet=True, tol=1e-6)
    if name in ("jet128", "jet256", "adjoint128"):
        base = 256 if name == "jet256" else 128
        n = int(round(base * scale))
        s = n / 128.0
        h = 5e-5 * 128.0 / n
        alpha, solid = _jet(n, s, seed, h)
        u, v, w = _velocities(seed, alpha, solid, 0.2, 0.02)
        case = dict(name=name, dims=(n, n, n), h=h, rho_liquid=6440.0, rho_air=1.2, alpha=alpha, solid=solid,
                    u=u, v=v, w=w, dt=1e-5, periodic=0, outlet=True, tol=1e-6)
        if name == "adjoint128":
            case["dt"] = 1e-6
            fa = _face_alpha(alpha.astype(np.float64))
            opens = _open_faces(solid)
            forces = []
            for a, (f, op) in enumerate(zip(fa, opens)):
                z = normal(seed, 40 + a, f.size).reshape(f.shape) * 1e5
                z[(f < 0.5) | ~op] = 0.0
                forces.append(np.ascontiguousarray(z.astype(np.float32)))
            case["fu"], case["fv"], case["fw"] = forces
            case["steps"] = 8
            case["checkpoint_every"] = 4
        return case
    if name == "column512":
        nx, ny, nz = int(round(512 * scale)), int(round(256 * scale)), int(round(256 * scale))
        h = 2.5e-5 / scale
        cx, cy, cz = _centres(nx), _centres(ny), _centres(nz)
        z, y, x = np.meshgrid(cz, cy, cx, indexing="ij")
        w = 3.0 * scale
        alpha = _smooth(np.sqrt((y - ny / 2.0) ** 2 + (z - nz / 2.0) ** 2) - 20.0 * scale, w)
        p = uniform(seed, 3, 16)
        for k in range(4):
            px, py, pz = p[4 * k] * nx, (0.2 + 0.6 * p[4 * k + 1]) * ny, (0.2 + 0.6 * p[4 * k + 2]) * nz
            rad = (8.0 + 6.0 * p[4 * k + 3]) * scale
            d = np.sqrt((x - px) ** 2 + (y - py) ** 2 + (z - pz) ** 2) - rad
            alpha = np.maximum(alpha, _smooth(d, w))
        alpha = alpha.astype(np.float32)
        solid = np.zeros(alpha.shape, np.uint8)
        u, v, wv = _velocities(seed, alpha, solid, 0.2, 0.02)
        return dict(name=name, dims=(nx, ny, nz), h=h, rho_liquid=6440.0, rho_air=1.2, alpha=alpha, solid=solid,
                    u=u, v=v, w=wv, dt=1e-5, periodic=0, outlet=True, tol=1e-6)
    raise ValueError(f"unknown workload {name!r}")


SIGMA_316 = np.float32(1.0 / 0.75e-6)  # S/m, 316 stainless


def em_edge_dims(dims, axis):
    d = [int(v) + 1 for v in dims]
    d[axis] -= 1
    return tuple(d)


def em_uniform_potential(dims, h, origin, b, scale=1.0):
    """A_s = scale/2 * B x r at every edge midpoint, edges ordered x-, y-, then
    z-edges, each block x-fastest (float32, one value per edge)."""
    blocks = []
    for axis in range(3):
        d = em_edge_dims(dims, axis)
        z, y, x = np.meshgrid(np.arange(d[2]), np.arange(d[1]), np.arange(d[0]), indexing="ij")
        pos = [x.astype(np.float32), y.astype(np.float32), z.astype(np.float32)]
        pos[axis] = pos[axis] + np.float32(0.5)
        r = [np.float32(origin[k]) + pos[k] * np.float32(h) for k in range(3)]
        bb = [np.float32(v) for v in b]
        cr = [bb[1] * r[2] - bb[2] * r[1], bb[2] * r[0] - bb[0] * r[2], bb[0] * r[1] - bb[1] * r[0]]
        blocks.append((np.float32(0.5 * scale) * cr[axis]).reshape(-1))
    return np.concatenate(blocks).astype(np.float32)


def em_ring(n: int) -> dict:
    """The driven-ring EM workload on an n^3 grid (see the module docstring)."""
    h = 1e-3
    origin = (-0.5 * n * h,) * 3
    m = np.zeros((n, n, n), np.uint32)
    c = (n - 1) / 2.0
    y, x = np.mgrid[0:n, 0:n]
    r = np.hypot(x - c, y - c)
    ring = (r >= 0.19 * n) & (r <= 0.38 * n)
    m[n // 3:n - n // 3][:, ring] = 1
    props = np.array([[0.0, 1.0], [SIGMA_316 * 40, 1.0]], np.float32)
    b = (0.0, 0.0, 0.02)
    base = em_uniform_potential((n, n, n), h, origin, b)
    applied = lambda t: (base * np.float32(np.sin(2 * np.pi * 1e3 * t))).astype(np.float32)
    return dict(dims=(n, n, n), h=h, origin=origin, materials=m.reshape(-1), properties=props, dt=1e-5,
                applied=applied)


def em_loop_elements(radius, current, segments, centre=(0.0, 0.0, 0.0), core=0.0):
    """A closed polygonal wire loop in the plane z = centre[2]: `segments`
    straight elements (EmConfig::elements records, 12 float32 each)."""
    ang = 2.0 * np.pi * np.arange(segments + 1) / segments
    pts = np.stack([centre[0] + radius * np.cos(ang), centre[1] + radius * np.sin(ang),
                    np.full(segments + 1, centre[2])], 1)
    el = np.zeros((segments, 12), np.float32)
    el[:, 0:3] = pts[:-1]
    el[:, 4:7] = pts[1:]
    el[:, 8] = core
    el[:, 9] = 0.0
    el[:, 10] = current
    return el


def em_magnet_block_elements(half_x, half_y, half_z, magnetization, divisions, smoothing=0.0):
    """Surface-current elements of a uniformly magnetised block centred at the
    origin (M along z): each side face is split into divisions^2 squares of
    two triangles; element = (centroid, M x outward area vector, smoothing),
    as EmConfig::elements builds magnet bodies."""
    m = np.array([0.0, 0.0, magnetization])
    out = []
    faces = []
    for sx in (-1.0, 1.0):   # x = +-half_x, outward normal along x
        faces.append((np.array([sx * half_x, 0, 0]), np.array([0, 1.0, 0]) * half_y, np.array([0, 0, 1.0]) * half_z,
                      np.array([sx, 0, 0])))
    for sy in (-1.0, 1.0):
        faces.append((np.array([0, sy * half_y, 0]), np.array([1.0, 0, 0]) * half_x, np.array([0, 0, 1.0]) * half_z,
                      np.array([0, sy, 0])))
    for c, du, dv, n in faces:
        for i in range(divisions):
            for j in range(divisions):
                u0, u1 = -1 + 2 * i / divisions, -1 + 2 * (i + 1) / divisions
                v0, v1 = -1 + 2 * j / divisions, -1 + 2 * (j + 1) / divisions
                q = [c + du * u0 + dv * v0, c + du * u1 + dv * v0, c + du * u1 + dv * v1, c + du * u0 + dv * v1]
                for tri in ((q[0], q[1], q[2]), (q[0], q[2], q[3])):
                    a, b, cc = tri
                    area = np.cross(b - a, cc - a) * 0.5
                    if np.dot(area, n) < 0:
                        area = -area
                    e = np.zeros(12)
                    e[0:3] = (a + b + cc) / 3.0
                    e[4:7] = np.cross(m, area)
                    e[8], e[9], e[10] = smoothing, 1.0, 1.0
                    out.append(e)
    return np.array(out, np.float32)


def em_uniform_element(b, scale=1.0):
    e = np.zeros((1, 12), np.float32)
    e[0, 4:7] = b
    e[0, 9] = 2.0
    e[0, 10] = scale
    return e


def em_sphere_materials(cells, h, origin, radius, material=2, sub=4):
    """Material ids of a sphere of `radius` centred at the origin on a cells^3
    grid whose low corner is at `origin` (all axes): cells fully inside carry
    `material`; cut cells carry the partial-cell encoding (bit 31, fraction
    in bits 8..30 from sub^3 point samples, material in bits 0..7)."""
    g = (np.arange(sub) + 0.5) / sub
    c = np.arange(cells)
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    frac = np.zeros((cells,) * 3)
    for a in g:
        for b in g:
            for d in g:
                px, py, pz = origin + (x + a) * h, origin + (y + b) * h, origin + (z + d) * h
                frac += (px * px + py * py + pz * pz) <= radius * radius
    frac /= sub ** 3
    m = np.zeros(frac.shape, np.uint32)
    m[frac >= 1.0] = material
    cut = (frac > 0.0) & (frac < 1.0)
    q = np.round(frac[cut] * 8388607).astype(np.uint32)
    m[cut] = np.uint32(0x80000000) | (q << np.uint32(8)) | np.uint32(material)
    return m.reshape(-1)
