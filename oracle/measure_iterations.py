"""Run the oracle's restatement of the reference projection to convergence on
a synthetic workload and record how many CG iterations it needs.

TEST AND MEASUREMENT INFRASTRUCTURE ONLY.  The reference arm of bench.py
times a bounded sample of the same CPU code (set-up plus a few CG
iterations) and scales it to the iteration count recorded here, so that a
bench run stays within minutes.  The file this writes,
reference_iterations.json, sits next to this script:

    python oracle/measure_iterations.py jet256 1e-6

The workload is the named synthetic case with the reference's closed
boundaries (the reference has no outlet) and FluidConfig defaults otherwise
(absolute divergence floor 0, automatic gauge and preconditioner).
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [HERE, os.path.join(ROOT, "mhd-simulator_gb300")]

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from mhdproj import synth  # noqa: E402

OUT = os.path.join(HERE, "reference_iterations.json")


def face_records(case):
    nx, ny, nz = case["dims"]
    rec = np.zeros((nz + 1, ny + 1, nx + 1, 4), np.float32)
    rec[:nz, :ny, :, 0] = case["u"]
    rec[:nz, :, :nx, 1] = case["v"]
    rec[:, :ny, :nx, 2] = case["w"]
    return rec.reshape(-1, 4)


def measure(name, tol, max_iterations=20000, seed=1):
    case = synth.make_case(name, seed=seed)
    nx, ny, nz = case["dims"]
    mask01 = (case["solid"].reshape(-1) == 0).astype(np.uint32)
    comps, mask = oracle.anchors(mask01, (nx, ny, nz), 0)
    fluid = int((mask != 0).sum())
    p = oracle.make_params((nx, ny, nz), case["h"], case["dt"], case["rho_liquid"], case["rho_air"], True, 0, tol,
                           0.0, fluid)
    t0 = time.perf_counter()
    res, *_ = oracle.ref_project(p, mask, comps, case["alpha"].reshape(-1), face_records(case),
                                 max_iterations=max_iterations)
    return dict(workload=name, seed=seed, dims=[nx, ny, nz], rel_tol=tol, boundary="closed",
                status=int(res.status), iterations=int(res.iterations), residual=float(res.residual),
                multigrid=bool(res.multigrid), meanfree=bool(res.meanfree), components=comps,
                seconds=time.perf_counter() - t0, threads=int(os.environ.get("OMP_NUM_THREADS", os.cpu_count())))


if __name__ == "__main__":
    name = sys.argv[1] if len(sys.argv) > 1 else "jet256"
    tol = float(sys.argv[2]) if len(sys.argv) > 2 else 1e-6
    rec = measure(name, tol)
    table = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            table = json.load(f)
    table[f"{name}@{tol:g}"] = rec
    with open(OUT, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    print(json.dumps(rec))
