"""The allocation-free divergence entry point (mhdproj_divergence_noalloc).

Some callers cannot allocate device memory while they run: a simulation loop
that reserved its whole memory budget at start-up, or a diagnostics hook that
runs on another library's stream without a projection context.  The entry
point keeps its reduction scratch in a fixed array inside the library, so it
allocates nothing; this test checks it against the divergence statistics the
projection entry point reports for the same field, on two calls in a row.
"""
import math

import numpy as np
import pytest

from mhdproj import synth

pytestmark = pytest.mark.gpu

TOL = 1e-9  # relative; both sides take the same double-FP32 per-cell divergence


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
