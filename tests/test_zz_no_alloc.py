"""The allocation-free divergence entry point (mhdproj_divergence_noalloc).

Some callers cannot allocate device memory while they run: a simulation loop
that reserved its whole memory budget at start-up, or a diagnostics hook that
runs on another library's stream without a projection context.  The entry
point keeps its reduction scratch in a fixed array inside the library, so it
allocates nothing; this test checks it against the divergence statistics the
projection entry point reports for the same field, on two calls in a row.
"""
import ctypes as C
import math

import numpy as np
import pytest

from mhdproj import synth

TOL = 1e-9  # relative; both sides take the same double-FP32 per-cell divergence


@pytest.mark.gpu
def test_noalloc_divergence_matches_projection_stats(gpu):
    import mhdproj

    torch = gpu
    c = synth.make_case("jet128", scale=0.375)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    alpha, solid = t(c["alpha"]), t(c["solid"])
    us = (t(c["u"]), t(c["v"]), t(c["w"]))
    pr = mhdproj.PressureProjection(c["dims"], c["h"], outlet=True, rel_tol=1e-6, compute_divergence=True)
    pr.set_coefficients(alpha, solid, c["rho_liquid"], c["rho_air"])
    (u, v, w), _, st = pr.project(us, c["dt"])
    m, comps = pr.topology()
    assert not (m == 2).any()  # no pinned cells: both sides cover the same cells
    for _ in range(2):
        mx, rms = mhdproj.divergence_noalloc(c["dims"], c["h"], solid, u, v, w)
        assert math.isclose(mx, st.max_divergence, rel_tol=TOL, abs_tol=0.0)
        assert math.isclose(rms, st.rms_divergence, rel_tol=TOL, abs_tol=0.0)
    # the unprojected field too, against a host evaluation of the same sum
    mx0, rms0 = mhdproj.divergence_noalloc(c["dims"], c["h"], solid, *us)
    nx, ny, nz = c["dims"]
    d = (np.diff(c["u"].astype(np.float64), axis=2) + np.diff(c["v"].astype(np.float64), axis=1)
         + np.diff(c["w"].astype(np.float64), axis=0)) / np.float32(c["h"])
    f = c["solid"] == 0
    assert math.isclose(mx0, np.abs(d[f]).max(), rel_tol=1e-6)
    assert math.isclose(rms0, math.sqrt((d[f] ** 2).mean()), rel_tol=1e-6)


@pytest.mark.gpu
def test_noalloc_periodic_axes_read_face_zero(gpu):
    """On a periodic axis the duplicate high face is ignored: the last cell's
    high face is face 0.  The duplicates are set to garbage to show it."""
    import mhdproj

    torch = gpu
    nx, ny, nz = 40, 19, 11
    rng = np.random.default_rng(11)
    solid = (rng.random((nz, ny, nx)) < 0.1).astype(np.uint8)
    u = rng.standard_normal((nz, ny, nx + 1)).astype(np.float32)
    v = rng.standard_normal((nz, ny + 1, nx)).astype(np.float32)
    w = rng.standard_normal((nz + 1, ny, nx)).astype(np.float32)
    u[:, :, nx] = 1e3
    v[:, ny, :] = -1e3
    w[nz, :, :] = 5e2
    h = 1e-3
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    for periodic in (1, 2, 4, 7):
        uu, vv, ww = (a.astype(np.float64) for a in (u, v, w))
        if periodic & 1:
            uu[:, :, nx] = uu[:, :, 0]
        if periodic & 2:
            vv[:, ny, :] = vv[:, 0, :]
        if periodic & 4:
            ww[nz, :, :] = ww[0, :, :]
        d = (np.diff(uu, axis=2) + np.diff(vv, axis=1) + np.diff(ww, axis=0)) / np.float32(h)
        f = solid == 0
        for _ in range(2):
            mx, rms = mhdproj.divergence_noalloc((nx, ny, nz), h, t(solid), t(u), t(v), t(w), periodic=periodic)
            assert math.isclose(mx, np.abs(d[f]).max(), rel_tol=1e-6)
            assert math.isclose(rms, math.sqrt((d[f] ** 2).mean()), rel_tol=1e-6)


def test_noalloc_rejects_face_arrays_beyond_int32():
    """Host-side guard, checked before any device work (no GPU needed): the
    v array of a 4096 x 1 x 300000 grid has 2.46e9 elements although u has
    1.23e9; extents above INT_MAX are refused too.  The pointers are never
    dereferenced because the call returns before any CUDA call."""
    import mhdproj

    L = mhdproj.load()
    buf = (C.c_float * 4)()
    p = C.cast(buf, C.c_void_p)
    out = (C.c_double * 2)()
    for dims in ((4096, 1, 300000), (1 << 31, 1, 1), (1, 1, 0xFFFFFFFF)):
        g = mhdproj.Grid(dims[0], dims[1], dims[2], 1e-3, 0, 0)
        rc = L.mhdproj_divergence_noalloc(C.byref(g), p, p, p, p, out, None)
        assert rc == 1
        assert b"2^31" in L.mhdproj_last_error(None)


@pytest.mark.gpu
def test_noalloc_rejects_planes_beyond_its_scratch(gpu):
    import mhdproj

    torch = gpu
    nx, ny, nz = 4096, 264, 1  # 128 x 33 = 4224 tiles of 32x8 cells
    solid = torch.zeros((nz, ny, nx), dtype=torch.uint8, device="cuda")
    u = torch.zeros((nz, ny, nx + 1), device="cuda")
    v = torch.zeros((nz, ny + 1, nx), device="cuda")
    w = torch.zeros((nz + 1, ny, nx), device="cuda")
    with pytest.raises(mhdproj.ProjectionError, match="4096 tiles"):
        mhdproj.divergence_noalloc((nx, ny, nz), 1e-3, solid, u, v, w)
