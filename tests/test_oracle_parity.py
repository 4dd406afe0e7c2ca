"""The GB300 path's discrete problem against the reference's (CPU, no GPU).

The GB300 solver's FP64 oracle (onat_*) builds its own coefficient cache: the
mobility of each cell's three low faces between two active cells, and a
reaction term that folds the faces towards a pinned gauge cell (and the
outlet) into the diagonal.  The reference's restatement (oref_*) builds the
cache of `pressure_coefficients` (src/fluid/solver.wgsl:93-103): the mobility
of every open face and the diagonal, with pinned anchor rows as the identity
(`apply`, :78-92).  On the reference's own closed boundaries the two must
describe the same operator:
  * the same gauge cells (the first cell of every component),
  * bit-identical face mobilities between active cells,
  * reactions equal to the FP32 sum, in the oracle's face order, of the
    reference's mobilities towards the pinned cell,
  * diagonals equal to within the rounding of a six-term FP32 sum,
  * the same operator action on every active cell, to FP32 rounding.
Cases: the reference's multigrid fixtures, its periodic cosine (one phase),
a closed two-phase jet, and thermal phase drag.
"""
import numpy as np
import pytest

import refcases as R

EPS32 = float(np.finfo(np.float32).eps)


def _reference_cache(oracle, c, phase=None, drag_rate=1e6):
    nx, ny, nz = c["dims"]
    mask01 = (np.asarray(c["solid"]).reshape(-1) == 0).astype(np.uint32)
    comps, mask = oracle.anchors(mask01, c["dims"], c["periodic"])
    fluid = int((mask != 0).sum())
    p = oracle.make_params(c["dims"], c["h"], c["dt"], c["rho_liquid"], c["rho_air"], c["two_phase"], c["periodic"],
                           c["rel_tol"], c["abs_div_tol"], fluid, phase is not None, drag_rate)
    rec = np.zeros(((nx + 1) * (ny + 1) * (nz + 1), 4), np.float32)
    ph = None if phase is None else np.ascontiguousarray(phase, np.float32).reshape(-1)
    oracle.lib().oref_coefficients(p, mask, np.asarray(c["alpha"], np.float32).reshape(-1),
                                   None if ph is None else ph.ctypes.data, rec.reshape(-1))
    return p, mask, rec


def _native(oracle, c, phase=None, drag_rate=1e6):
    nx, ny, nz = c["dims"]
    g = oracle.grid(nx, ny, nz, c["h"], c["rho_liquid"], c["rho_air"], c["periodic"], outlet=False,
                    single=not c["two_phase"], phase=phase, drag_rate=drag_rate if phase is not None else 0.0,
                    dt=c["dt"] if phase is not None else 0.0)
    _, cls = oracle.classify(g, c["solid"])
    coef, _ = oracle.coefficients(g, c["alpha"], cls)
    return g, cls, coef


def _neighbour(dims, periodic, x, y, z, axis, d):
    q = [x, y, z]
    q[axis] = q[axis] + d
    if periodic & (1 << axis):
        q[axis] %= dims[axis]
    if not 0 <= q[axis] < dims[axis]:
        return None
    return q


CASES = [
    ("walls17x13x9", lambda: R.wall_case((17, 13, 9), (0, 0, 0), True, False)),
    ("walls16x12x8_periodic_xy", lambda: R.wall_case((16, 12, 8), (1, 1, 0), True, True)),
    ("walls16x12x8_periodic_z", lambda: R.wall_case((16, 12, 8), (0, 0, 1), True, False)),
    ("cosine16_one_phase", lambda: R.cosine_case()),
    ("jet32_closed", lambda: R.jet_case("jet128", 0.25)),
]


def _phase_field(c, seed=4):
    rng = np.random.default_rng(seed)
    f = rng.random(np.asarray(c["alpha"]).shape).astype(np.float32)
    f[f > 0.7] = 1.0  # fully molten cells: no drag on their shared faces
    return f


@pytest.mark.parametrize("drag", [False, True], ids=["no_drag", "phase_drag"])
@pytest.mark.parametrize("name,factory", CASES, ids=[n for n, _ in CASES])
def test_native_operator_is_the_references(oracle_lib, name, factory, drag):
    c = factory()
    phase = _phase_field(c) if drag else None
    p, mask, rec = _reference_cache(oracle_lib, c, phase)
    g, cls, coef = _native(oracle_lib, c, phase)
    nx, ny, nz = c["dims"]
    dims = (nx, ny, nz)
    per = c["periodic"]
    n = nx * ny * nz
    # the same gauge cells: the root of every component
    assert np.array_equal(np.nonzero(cls == 2)[0], np.nonzero((mask & 3) == 2)[0])
    assert np.array_equal(cls != 0, mask != 0)
    frec = rec.reshape(nz + 1, ny + 1, nx + 1, 4)

    def face(q, axis):  # the reference's canonical face at the low side of cell q
        return frec[q[2], q[1], q[0], axis]

    checked = 0
    for i in np.nonzero(cls == 1)[0]:
        x, y, z = i % nx, (i // nx) % ny, i // (nx * ny)
        reaction = np.float32(0.0)
        diag_terms = []
        for axis in range(3):
            for d in (-1, 1):
                q = _neighbour(dims, per, x, y, z, axis, d)
                if q is None:
                    continue
                j = q[0] + nx * (q[1] + ny * q[2])
                if cls[j] == 0:
                    continue
                beta = face((x, y, z) if d < 0 else q, axis)
                diag_terms.append(float(beta))
                if cls[j] == 2:
                    reaction = np.float32(reaction + beta)
                elif d < 0:
                    assert coef[i, axis].view(np.uint32) == np.float32(beta).view(np.uint32), (i, axis)
                    checked += 1
        assert coef[i, 3].view(np.uint32) == reaction.view(np.uint32), i
        # diagonal: the reference's cached value against the native row sum
        nd = float(coef[i, 3])
        for axis in range(3):
            nd += float(coef[i, axis])
            q = _neighbour(dims, per, x, y, z, axis, 1)
            if q is not None:
                j = q[0] + nx * (q[1] + ny * q[2])
                if cls[j] == 1:
                    nd += float(coef[j, axis])
        rd = float(rec[i, 3])
        assert abs(nd - rd) <= 8 * EPS32 * max(sum(diag_terms), 1e-30), (i, nd, rd)
    assert checked > 0

    # operator action on active cells, with the gauge cells at zero
    rng = np.random.default_rng(17)
    x = rng.standard_normal(n).astype(np.float32)
    x[cls != 1] = 0.0
    work = np.zeros((n, 4), np.float32)
    work[:, 2] = x
    want = np.zeros(n, np.float32)
    oracle_lib.lib().oref_apply_cached(p, mask, rec.reshape(-1), work.reshape(-1), 1, want)
    got = oracle_lib.apply(g, coef, x.astype(np.float64))
    act = cls == 1
    scale = rec[:n, 3].astype(np.float64)  # the row's sum of mobilities (the reference's diagonal)
    err = np.abs(got[act] - want[act].astype(np.float64))
    assert np.all(err <= 16 * EPS32 * (scale[act] * np.abs(x).max() + 1e-30)), float(err.max())


def test_phase_drag_reduces_mobility(oracle_lib):
    """f = 1 on both sides leaves a face's mobility unchanged; f < 1 lowers it."""
    c = R.wall_case((17, 13, 9), (0, 0, 0), True, False)
    _, cls, base = _native(oracle_lib, c)
    f = np.ones(np.asarray(c["alpha"]).shape, np.float32)
    f.reshape(-1)[::3] = 0.25
    _, _, dragged = _native(oracle_lib, c, f)
    assert np.all(dragged[:, :3] <= base[:, :3])
    assert np.any(dragged[:, :3] < base[:, :3])
    flat = f.reshape(-1)
    nx = c["dims"][0]
    for i in np.nonzero((cls == 1) & (flat == 1.0))[0][:50]:
        if i % nx and cls[i - 1] == 1 and flat[i - 1] == 1.0:
            assert dragged[i, 0] == base[i, 0]


PROJECTION_CASES = CASES + [("jet32_closed_rev", lambda: R.jet_case("jet64", 0.5))]


@pytest.mark.parametrize("name,factory", PROJECTION_CASES, ids=[n for n, _ in PROJECTION_CASES])
def test_native_projection_equals_the_references(oracle_lib, name, factory):
    """The FP64 oracle's projection on the reference's closed boundaries
    against the restated reference projection (FluidState::project,
    src/fluid/mod.rs:1015-1115, then `correct`, solver.wgsl:245-250) on the
    same inputs: face velocities within the reference's own acceptance bound
    (L2 difference 2e-4 of the candidate field's norm, the measure of
    src/fluid/multigrid/tests.rs:330-465) and the pressure in the
    reference's gauge (the root of each component at 0) to 2e-4 relative."""
    c = factory()
    c = dict(c, rel_tol=3e-6, abs_div_tol=0.0)  # near the FP32 reference's floor on the jets
    ref = R.run_oracle(oracle_lib, c, max_iterations=4000)
    assert ref["result"].status == 0
    nx, ny, nz = c["dims"]
    g = oracle_lib.grid(nx, ny, nz, c["h"], c["rho_liquid"], c["rho_air"], c["periodic"], outlet=False,
                        single=not c["two_phase"])
    nat = oracle_lib.project(g, c["alpha"], c["solid"], c["u"], c["v"], c["w"], c["dt"], 1e-12)
    assert nat["status"] == 0
    num = den = 0.0
    for k in "uvw":
        a = nat[k].reshape(-1)
        b = ref[k].reshape(-1).astype(np.float64)
        num += float(((a - b) ** 2).sum())
        den += float((np.asarray(c[k], np.float64) ** 2).sum())
    assert np.sqrt(num / den) < 2e-4
    fluid = ref["mask"] != 0
    pr, pn = ref["p"].astype(np.float64)[fluid], nat["p"][fluid]
    assert np.linalg.norm(pn - pr) <= 2e-4 * np.linalg.norm(pr)
