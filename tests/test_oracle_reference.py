"""The FP32 restatement of the reference projection (oracle/oracle_ref.c),
checked against the reference's own known answers and acceptance tests.

Each test names the reference test it ports; tolerances are the reference's.
"""
import json
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")


def known():
    with open(GOLDEN) as f:
        return json.load(f)


# ---------------------------------------------------------------- fixtures
def mg_fixture(oracle, d, periodic, walls, reverse, meanfree=False):
    """multigrid/tests.rs:8-63: 1 m cells, rho 7000:1 split at x = d0/2,
    walls at x = d0/2 plus the cell (1,1)."""
    n = d[0] * d[1] * d[2]
    i = np.arange(n)
    x, y = i % d[0], (i // d[0]) % d[1]
    if walls:
        mask01 = ((x != d[0] // 2) & ~((x == 1) & (y == 1))).astype(np.uint32)
    else:
        mask01 = np.ones(n, np.uint32)
    bits = sum(1 << a for a in range(3) if periodic[a])
    comps, mask = oracle.anchors(mask01, d, bits)
    fluid = int((mask != 0).sum())
    occ = ((x < d[0] // 2) ^ reverse).astype(np.float32)
    p = oracle.make_params(d, 1.0, 1e-5, 7000.0, 1.0, True, bits, 1e-5, 1e-5, fluid)
    return p, mask, comps, occ, bits


def set_gauge(oracle, p, mask, comps, meanfree):
    p.initial[3] = 1.0 / float(max(int((mask != 0).sum()), 1)) if (meanfree and comps == 1) else 0.0
    p.solve[2] = 1.0 if (meanfree and comps == 1) else float(int((mask != 0).sum()))


def manufactured(p, mask, cache, binary=False):
    """manufactured_gradient (multigrid/tests.rs:282-329)."""
    d = [p.dims[0], p.dims[1], p.dims[2]]
    f = [p.faces[0], p.faces[1], p.faces[2]]
    per = [bool(p.flags[0] & (1 << a)) for a in range(3)]
    cache = cache.reshape(-1, 4)

    def potential(q):
        if binary:
            return float(min(q[0], d[0] - q[0]))
        tau = 2 * math.pi
        return np.float32(math.cos(tau * (q[0] + 0.5) / d[0]) + 0.3 * math.sin(tau * (q[1] + 0.5) / d[1])
                          + 0.2 * math.cos(tau * (q[2] + 0.5) / d[2]))

    def canon(q):
        return [q[a] % d[a] if per[a] else q[a] for a in range(3)]

    def fluid(q):
        return all(0 <= q[a] < d[a] for a in range(3)) and mask[q[0] + d[0] * (q[1] + d[1] * q[2])] != 0

    nf = f[0] * f[1] * f[2]
    out = np.zeros((nf, 4), np.float32)
    for i in range(nf):
        q = canon([i % f[0], (i // f[0]) % f[1], i // (f[0] * f[1])])
        for a in range(3):
            l = list(q)
            l[a] -= 1
            l = canon(l)
            if fluid(l) and fluid(q):
                fi = q[0] + f[0] * (q[1] + f[1] * q[2])
                out[i, a] = np.float32(cache[fi, a]) * (np.float32(potential(q)) - np.float32(potential(l))) / np.float32(p.physical[0])
    return out


# ------------------------------------------------------------ known answers
def test_hierarchy_known_answers(oracle_lib):
    """hierarchy_uses_exact_ceil_half_workspace_and_checked_indices (multigrid/tests.rs:603-618)."""
    k = known()
    for case in k["hierarchy"]:
        levels, cells = oracle_lib.hierarchy(case["dims"])
        assert cells == case["coarse_cells"]
        assert all(v <= 4 for v in levels[-1][:3])
        assert sum(l[3] for l in levels[1:]) == cells
    for dims in k["hierarchy_rejected"]:
        assert oracle_lib.hierarchy(dims) is None


def test_anchor_known_answers(oracle_lib):
    """pressure_failure_rolls_back_and_disconnected_components_get_gauges (fluid/tests.rs:186-195)."""
    k = known()
    first = k["anchors"][0]
    comps, mask = oracle_lib.anchors(first["mask"], first["dims"], 0)
    assert comps == first["components"]
    assert list(mask & 3) == k["anchors_first_case_classes"]
    assert [int(mask[0] >> 2), int(mask[2] >> 2)] == k["anchors_first_case_roots"]
    per = k["anchors"][1]
    comps, _ = oracle_lib.anchors(per["mask"], per["dims"], 1)
    assert comps == per["components"]


# ------------------------------------------------------- analytic accept.
@pytest.mark.parametrize("floating,multigrid", [(False, False), (True, False), (True, True)])
def test_meanfree_periodic_gradient_recovers_analytic_pressure(oracle_lib, floating, multigrid):
    """pressure_tests.rs:4-71: 16^3 periodic, phi = 0.001 cos(2 pi x/n + pi/n)."""
    n, h, rho, dt = 16, 1e-3, 1000.0, 1e-5
    d = (n, n, n)
    mask01 = np.ones(n ** 3, np.uint32)
    comps, mask = oracle_lib.anchors(mask01, d, 7)
    p = oracle_lib.make_params(d, h, dt, rho, rho, False, 7, 1e-5, 1e-7, n ** 3)
    phi = lambda x: 0.001 * math.cos(2 * math.pi * (x % n) / n + math.pi / n)
    fd = n + 1
    faces = np.zeros((fd ** 3, 4), np.float32)
    for z in range(fd):
        for y in range(fd):
            for x in range(fd):
                faces[x + fd * (y + fd * z), 0] = np.float32((phi(x) - phi((x + n - 1) % n)) / h)
    res, vel, work, _ = oracle_lib.ref_project(p, mask, comps, np.ones(n ** 3, np.float32), faces, max_iterations=4000,
                                               force_mg=int(multigrid), force_meanfree=int(floating))
    assert res.status == 0
    assert res.meanfree == int(floating)
    x = np.arange(n ** 3) % n
    expected = (np.array([phi(v) for v in x]) - phi(0)) * rho / dt
    pot = work[:, 0].astype(np.float64)
    if floating:
        pot = pot - pot[0]
    pressure = pot * rho / dt
    rel = np.sqrt(((pressure - expected) ** 2).sum() / (expected ** 2).sum())
    assert rel < 1e-4
    speed = np.abs(vel[:, :3]).max()
    assert speed < 2e-6


CASES = [((17, 13, 9), (True,) * 3, False), ((16, 12, 8), (False,) * 3, True), ((13, 1, 3), (True,) * 3, True)]


@pytest.mark.parametrize("dims,periodic,walls", CASES)
@pytest.mark.parametrize("reverse", [False, True])
def test_manufactured_pressure_projection_keeps_physical_acceptance(oracle_lib, dims, periodic, walls, reverse):
    """manufactured_pressure_projection_keeps_physical_acceptance (multigrid/tests.rs:330-404)."""
    p, mask, comps, occ, bits = mg_fixture(oracle_lib, dims, periodic, walls, reverse)
    cache = np.zeros((p.faces[3], 4), np.float32)
    set_gauge(oracle_lib, p, mask, comps, False)
    oracle_lib.lib().oref_coefficients(p, mask, occ, None, cache.reshape(-1))
    cand = manufactured(p, mask, cache)
    norm = np.sqrt((cand[:, :3].astype(np.float64) ** 2).sum())
    for mg in (0, 1):
        res, vel, _, _ = oracle_lib.ref_project(p, mask, comps, occ, cand, max_iterations=20000, force_mg=mg,
                                                force_meanfree=0)
        assert res.status == 0, res.status
        err = np.sqrt((vel[:, :3].astype(np.float64) ** 2).sum()) / norm
        assert err < 2e-4


@pytest.mark.parametrize("dims,periodic,walls", CASES + [((16, 12, 8), (False,) * 3, False)])
@pytest.mark.parametrize("multigrid", [False, True])
def test_meanfree_pressure_contrast_and_disconnected_controls(oracle_lib, dims, periodic, walls, multigrid):
    """meanfree_pressure_contrast_and_disconnected_controls (multigrid/tests.rs:406-465)."""
    for reverse in (False, True):
        p, mask, comps, occ, bits = mg_fixture(oracle_lib, dims, periodic, walls, reverse)
        if comps != 1:
            continue
        set_gauge(oracle_lib, p, mask, comps, True)
        cache = np.zeros((p.faces[3], 4), np.float32)
        oracle_lib.lib().oref_coefficients(p, mask, occ, None, cache.reshape(-1))
        cand = manufactured(p, mask, cache)
        res, vel, work, _ = oracle_lib.ref_project(p, mask, comps, occ, cand, max_iterations=20000,
                                                   force_mg=int(multigrid), force_meanfree=1)
        assert res.status == 0 and res.meanfree == 1
        for i in np.nonzero((mask & 3) == 2)[0]:
            assert work[i, 0] == 0.0, "reference pressure drifted"
        norm = np.sqrt((cand[:, :3].astype(np.float64) ** 2).sum())
        assert np.sqrt((vel[:, :3].astype(np.float64) ** 2).sum()) / norm < 2e-4


def _mg(oracle_lib, p, mask, occ, meanfree):
    cache = np.zeros((p.faces[3], 4), np.float32)
    oracle_lib.lib().oref_coefficients(p, mask, occ, None, cache.reshape(-1))
    mg = oracle_lib.lib().oref_mg_create(p, mask, cache.reshape(-1), int(meanfree))
    oracle_lib.lib().oref_mg_build(mg)
    return mg, cache


@pytest.mark.parametrize("dims,periodic,walls", CASES + [((3, 2, 1), (False,) * 3, False)])
@pytest.mark.parametrize("reverse", [False, True])
def test_v_cycle_is_positive_symmetric(oracle_lib, dims, periodic, walls, reverse):
    """v_cycle_is_positive_symmetric_and_preserves_live_lanes (multigrid/tests.rs:202-280)."""
    L = oracle_lib.lib()
    p, mask, comps, occ, bits = mg_fixture(oracle_lib, dims, periodic, walls, reverse)
    set_gauge(oracle_lib, p, mask, comps, False)
    mg, _ = _mg(oracle_lib, p, mask, occ, False)
    n = p.dims[3]
    i = np.arange(n)
    act = (mask & 3) == 1
    r = np.where(act, np.cos(i * 0.17), 0.0).astype(np.float32)
    s = np.where(act, np.sin(i * 0.37), 0.0).astype(np.float32)

    def apply(rhs):
        work = np.zeros((n, 4), np.float32)
        work[:, 0], work[:, 1], work[:, 2] = 0.125, rhs, -0.25
        L.oref_mg_apply(mg, work.reshape(-1))
        assert np.all(work[:, 0] == 0.125) and np.all(work[:, 1] == rhs) and np.all(work[:, 2] == -0.25)
        return work[:, 3].astype(np.float64)

    mr, ms = apply(r), apply(s)
    rr, ss = float(r @ mr), float(s @ ms)
    sym = abs(float(r @ ms) - float(s @ mr)) / math.sqrt(rr * ss)
    L.oref_mg_destroy(mg)
    assert rr > 0 and ss > 0 and sym < 3e-6


@pytest.mark.parametrize("dims,periodic,walls", CASES + [((1, 1, 1), (False,) * 3, False)])
@pytest.mark.parametrize("floating", [False, True])
def test_aggregation_is_galerkin(oracle_lib, dims, periodic, walls, floating):
    """aggregation_is_gpu_galerkin_on_odd_periodic_and_disconnected_domains (multigrid/tests.rs:71-200)."""
    import ctypes as C

    L = oracle_lib.lib()
    for reverse in (False, True):
        p, mask, comps, occ, bits = mg_fixture(oracle_lib, dims, periodic, walls, reverse)
        if floating and comps != 1:
            continue
        set_gauge(oracle_lib, p, mask, comps, floating)
        mg, cache = _mg(oracle_lib, p, mask, occ, floating)
        nl = L.oref_mg_levels(mg, None, None)
        ld = (C.c_uint32 * (4 * nl))()
        offs = (C.c_uint32 * nl)()
        L.oref_mg_levels(mg, C.cast(ld, C.c_void_p), C.cast(offs, C.c_void_p))
        total = sum(ld[4 * l + 3] for l in range(1, nl))
        if total == 0:
            L.oref_mg_destroy(mg)
            continue
        coeff = np.ctypeslib.as_array(L.oref_mg_coeff(mg), shape=(4 * total,)).reshape(total, 4)
        value = np.ctypeslib.as_array(L.oref_mg_value(mg), shape=(4 * total,)).reshape(total, 4)
        assert np.all(np.isfinite(coeff)) and np.all(coeff >= 0)
        active = (mask != 0) if floating else ((mask & 3) == 1)
        n = p.dims[3]
        for level in range(1, nl):
            pd = ld[4 * level:4 * level + 4]
            cd = ld[4 * (level - 1):4 * (level - 1) + 4]
            vec = np.sin(np.arange(pd[3]) * 0.71).astype(np.float32)
            value[offs[level]:offs[level] + pd[3], 1] = vec
            ci = np.arange(cd[3])
            par = (ci % cd[0]) // 2 + pd[0] * (((ci // cd[0]) % cd[1]) // 2 + pd[1] * ((ci // (cd[0] * cd[1])) // 2))
            work = np.zeros((n, 4), np.float32)
            if level == 1:
                work[active, 3] = vec[par][active]
                work[active, 2] = vec[par][active]
            else:
                value[offs[level - 1]:offs[level - 1] + cd[3], 1] = vec[par]
            fine_action = np.zeros(n, np.float32)
            L.oref_mg_probe_action(mg, level - 1, work.reshape(-1), fine_action)
            L.oref_mg_probe_action(mg, level, work.reshape(-1), fine_action if level == 1 else np.zeros(n, np.float32))
            if level == 1:
                child_action = np.where(active, fine_action, 0.0)
            else:
                child_action = value[offs[level - 1]:offs[level - 1] + cd[3], 2].astype(np.float64)
            restricted = np.zeros(pd[3])
            np.add.at(restricted, par, child_action)
            coarse = value[offs[level]:offs[level] + pd[3], 2].astype(np.float64)
            rel = math.sqrt(((coarse - restricted) ** 2).sum() / max((restricted ** 2).sum(), 1e-30))
            assert rel < 2e-6
            if level == 1:
                applied = np.zeros(n, np.float32)
                L.oref_apply_cached(p, mask, cache.reshape(-1), work.reshape(-1), 1, applied)
                assert np.all(np.abs(applied - fine_action)[active] < 1e-6 * (1 + np.abs(applied[active])))
        L.oref_mg_destroy(mg)


@pytest.mark.parametrize("dims", [(17, 13, 9), (3, 2, 1)])
def test_fused_coarse_solve_matches_fixed_jacobi_sequence(oracle_lib, dims):
    """fused_coarse_solve_matches_fixed_jacobi_sequence (multigrid/tests.rs:542-600)."""
    import ctypes as C

    L = oracle_lib.lib()
    p, mask, comps, occ, bits = mg_fixture(oracle_lib, dims, (True,) * 3, False, False)
    set_gauge(oracle_lib, p, mask, comps, False)
    mg, _ = _mg(oracle_lib, p, mask, occ, False)
    nl = L.oref_mg_levels(mg, None, None)
    ld = (C.c_uint32 * (4 * nl))()
    offs = (C.c_uint32 * nl)()
    L.oref_mg_levels(mg, C.cast(ld, C.c_void_p), C.cast(offs, C.c_void_p))
    c = nl - 1
    m = ld[4 * c + 3]
    n = p.dims[3]
    total = sum(ld[4 * l + 3] for l in range(1, nl))
    rhs = np.sin(np.arange(m) * np.float32(0.17)).astype(np.float32)
    work = np.zeros((n, 4), np.float32)
    if c == 0:
        work[:, 1] = np.where((mask & 3) == 1, rhs, 0.0)
        read = lambda: work[:, 3].copy()
    else:
        value = np.ctypeslib.as_array(L.oref_mg_value(mg), shape=(4 * total,)).reshape(total, 4)
        value[offs[c]:offs[c] + m, 0] = rhs
        read = lambda: value[offs[c]:offs[c] + m, 1].copy()
    L.oref_mg_coarse_jacobi_sequence(mg, work.reshape(-1))
    legacy = read().astype(np.float64)
    L.oref_mg_coarse_solve(mg, work.reshape(-1))
    fused = read().astype(np.float64)
    L.oref_mg_destroy(mg)
    rel = math.sqrt(((legacy - fused) ** 2).sum() / (legacy ** 2).sum())
    assert rel < 2e-6


@pytest.mark.parametrize("periodic", [0, 5, 7])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_cached_coefficients_match_original_operator(oracle_lib, periodic, mode):
    """cached_pressure_coefficients_match_original_operator_with_walls_phase_and_periodicity
    (fluid/tests.rs:501-635): channel(8) = 4 x 8 x 4 cells, a wall plane at y = 3."""
    L = oracle_lib.lib()
    d = (4, 8, 4)
    n = 128
    i = np.arange(n)
    mask01 = ((i // 4) % 8 != 3).astype(np.uint32)
    comps, mask = oracle_lib.anchors(mask01, d, periodic)
    fluid = int((mask != 0).sum())
    p = oracle_lib.make_params(d, 0.001, 1e-5, 1000.0, 1.2, mode > 0, periodic, 1e-5, 1e-5, fluid,
                               thermal_drag=(mode == 2), drag_rate=1e6)
    set_gauge(oracle_lib, p, mask, comps, True)
    occ = ((i % 11) / 10.0).astype(np.float32)
    phase = (0.2 + 0.8 * (i % 7) / 6.0).astype(np.float32)
    cache = np.zeros((p.faces[3], 4), np.float32)
    import ctypes as C

    L.oref_coefficients(p, mask, occ, phase.ctypes.data_as(C.c_void_p), cache.reshape(-1))
    work = np.zeros((n, 4), np.float32)
    work[:, 2] = np.sin(i * np.float32(0.1234)).astype(np.float32)
    fast = np.zeros(n, np.float32)
    L.oref_apply_cached(p, mask, cache.reshape(-1), work.reshape(-1), 1, fast)
    exact = np.zeros(n, np.float32)
    diag = np.zeros(n, np.float32)
    L.oref_apply_uncached(p, mask, occ, phase.ctypes.data_as(C.c_void_p), work.reshape(-1), 1, exact, diag)
    f = mask != 0
    assert np.array_equal(cache[:n, 3][f], diag[f])
    rel = math.sqrt(((fast - exact).astype(np.float64)[f] ** 2).sum() / (exact.astype(np.float64)[f] ** 2).sum())
    assert rel < 2e-7


def test_failure_reports_not_converged(oracle_lib):
    """max_iterations = 1 gives "did not converge" (fluid/tests.rs:164-185)."""
    p, mask, comps, occ, bits = mg_fixture(oracle_lib, (16, 12, 8), (False,) * 3, True, False)
    set_gauge(oracle_lib, p, mask, comps, False)
    cache = np.zeros((p.faces[3], 4), np.float32)
    oracle_lib.lib().oref_coefficients(p, mask, occ, None, cache.reshape(-1))
    cand = manufactured(p, mask, cache)
    res, vel, _, _ = oracle_lib.ref_project(p, mask, comps, occ, cand, max_iterations=1, force_mg=0, force_meanfree=0)
    assert res.status == 1
