"""Benchmark of the GB300 pressure projection.

One step = one projection of the 256^3 two-phase jet workload (seeded
synthetic fields of the jet256 construction): the mobility cache rebuild
(mhdproj_set_coefficients) and the projection to a 1e-6 relative residual
(mhdproj_project), inputs resident in HBM.  The inputs (liquid fraction,
solid mask, three face-velocity arrays: 286 MB) exceed the 129 MB L2, so no
flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs N independent replicas (the projection does not shard: replicas
only), one per rank under torchrun; the time is the max over ranks and the
value is the total projections/s.  --impl reference times the reference's
algorithm (the CPU port of its FP32 aggregation-multigrid CG) on the host
cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "mhd-simulator_gb300"))

METRIC = "256^3 two-phase projections/s to 1e-6 relative residual (mixed precision)"
UNIT = "projections/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="jet256")
    ap.add_argument("--precision", default="fp16", choices=["fp16", "bf16", "fp32"])
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-extras", action="store_true", help="skip the FP32/adjoint/e2e/CPU legs")
    ap.add_argument("--step", action="store_true",
                    help="only the fluid-step leg: a few mhdproj_fluid_step calls on the workload's geometry as one "
                         "liquid, then its kernels launched once each (a small launch list for profilers)")
    ap.add_argument("--em", action="store_true",
                    help="only the EM induction leg (driven ring, 128^3 and 64^3)")
    ap.add_argument("--kernels", action="store_true",
                    help="one projection, then each fine-level kernel of a CG iteration launched once in "
                         "isolation (a small, fixed launch list for profilers); prints the kernel times")
    return ap.parse_args()


# ------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        exe = shutil.which("nvidia-smi")
        if not exe:
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.fh = open(self.path, "w")
        self.proc = subprocess.Popen([exe, "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                      "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------ distributed
def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def max_over_ranks(value, pg, device=None):
    if pg is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg, device=None):
    if pg is not None:
        if device is not None:
            pg.barrier(device_ids=[device.index])
        else:
            pg.barrier()


# --------------------------------------------------------------- CPU legs
class CpuReference:
    """The reference algorithm on the host cores: the oracle's restatement of
    the reference projection (FP32 aggregation-multigrid CG, 256-lane
    reductions, closed boundaries, mean-free gauge, the reference's batched
    convergence reads and 64-iteration check) run with OpenMP on every host
    thread.  One sample is one whole projection to the tolerance: the
    coefficient cache, the multigrid build and every CG iteration."""

    def __init__(self, case, threads, tol):
        os.environ["OMP_NUM_THREADS"] = str(threads)
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import numpy as np
        import oracle

        self.np, self.oracle, self.threads = np, oracle, threads
        nx, ny, nz = case["dims"]
        mask01 = (case["solid"].reshape(-1) == 0).astype(np.uint32)
        t0 = time.perf_counter()
        self.comps, self.mask = oracle.anchors(mask01, (nx, ny, nz), 0)
        # the reference's host breadth-first search (anchors), one thread
        self.anchors_s = time.perf_counter() - t0
        fluid = int((self.mask != 0).sum())
        self.params = oracle.make_params((nx, ny, nz), case["h"], case["dt"], case["rho_liquid"], case["rho_air"],
                                         True, 0, tol, 0.0, fluid)
        rec = np.zeros((nz + 1, ny + 1, nx + 1, 4), np.float32)
        rec[:nz, :ny, :, 0] = case["u"]
        rec[:nz, :, :nx, 1] = case["v"]
        rec[:, :ny, :nx, 2] = case["w"]
        self.faces = rec.reshape(-1, 4)
        self.occ = np.ascontiguousarray(case["alpha"].reshape(-1))

    def run(self, iterations=20000):
        """One projection (to convergence, or `iterations` CG iterations);
        returns (seconds, oref_result, projected face records)."""
        t0 = time.perf_counter()
        res, vel, *_ = self.oracle.ref_project(self.params, self.mask, self.comps, self.occ, self.faces,
                                               max_iterations=iterations)
        return time.perf_counter() - t0, res, vel

    def projections(self, count, warmup=0):
        """`warmup` untimed and `count` timed whole projections: the seconds
        of each timed one and the last result."""
        for _ in range(warmup):
            self.run()
        secs, res = [], None
        for _ in range(count):
            t, res, _ = self.run()
            secs.append(t)
        return secs, res


# ------------------------------------------------------------ our arm
# ------------------------------------------------------------ our arm
def run_ours(args):
    import numpy as np
    import torch

    import mhdproj
    from mhdproj import build, synth

    world, rank, local, pg = dist_setup(args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    build.build()
    case = synth.make_case(args.workload, seed=args.seed + rank)
    nx, ny, nz = case["dims"]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    alpha, solid = t(case["alpha"]), t(case["solid"])
    us = (t(case["u"]), t(case["v"]), t(case["w"]))
    out = tuple(torch.empty_like(x) for x in us)
    p_out = torch.empty((nz, ny, nx), dtype=torch.float32, device=dev)
    def make(precision):
        return mhdproj.PressureProjection(case["dims"], case["h"], outlet=True, precision=precision,
                                          rel_tol=args.tol)

    def step(pr):
        pr.set_coefficients(alpha, solid, case["rho_liquid"], case["rho_air"])
        _, _, st = pr.project(us, case["dt"], out=out)
        return st

    def timed(pr, steps, fn=step):
        sts = []
        torch.cuda.synchronize(dev)
        barrier(pg, dev)
        torch.cuda.synchronize(dev)
        # events on the library's stream: the span of device work of the steps
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(pr.stream)
        for _ in range(steps):
            sts.append(fn(pr))
        e1.record(pr.stream)
        torch.cuda.synchronize(dev)
        barrier(pg, dev)
        ms = e0.elapsed_time(e1)
        return max_over_ranks(ms, pg, dev), sts

    def fluid_step_leg(steps, reps, two_phase=False):
        """FluidState::step on the workload's geometry.  One liquid: SL-RK2
        advection, viscosity, gravity, the warm-started projection, fields and
        diagnostics.  Two phases (the workload's densities): a moving
        interface, so Newtonian stress diffusion (liquid-metal viscosity
        3.7e-7 m^2/s, air 1.8e-5 Pa s), capillary force (sigma 0.5 N/m, zero
        curvature), face densities, the projection, fields."""
        ps = mhdproj.PressureProjection(case["dims"], case["h"], outlet=True, precision=args.precision,
                                        rel_tol=args.tol)
        ps.set_coefficients(alpha, solid, case["rho_liquid"], case["rho_air"] if two_phase else case["rho_liquid"])
        su = [x.clone() for x in us]
        dt_step = 2e-6 if two_phase else 5e-6
        nu_step = 3.7e-7 if two_phase else 1e-6

        def step_fn(prj):
            st, d = prj.fluid_step(su, dt_step, acceleration=(0.0, 0.0, -9.81), viscosity=nu_step, advection=True,
                                   surface_tension=0.5, air_viscosity=1.8e-5)
            st["viscous_substeps"] = d["viscous_substeps"]
            return st

        for _ in range(2):
            step_fn(ps)
        ms_s, sts_s = timed(ps, steps, step_fn)
        prof_s = ps.profile_kernels(reps=reps)
        ps.close()
        return {"ms_per_step": ms_s / steps, "steps_per_s": 1000.0 * steps / ms_s, "iterations": sts_s[-1]["iterations"],
                "viscous_substeps": sts_s[-1]["viscous_substeps"], "dt": dt_step, "kinematic_viscosity": nu_step,
                "densities": [case["rho_liquid"], case["rho_air"] if two_phase else case["rho_liquid"]],
                "kernels": [{"name": k["name"], "us": k["ms"] * 1e3, "GBps": k["bytes"] / (k["ms"] * 1e-3) / 1e9}
                            for k in prof_s if k["name"].startswith("step_")]}

    def chain_leg(name, scale, steps, every, reps):
        """Forward chain u_{k+1} = P(u_k + dt f / rho_face) of `steps` steps
        and its gradient dJ/df (outlet-plane objective, checkpoints every
        `every` steps), each timed on the library stream; plus the device
        memory the context holds (free memory before creation minus the
        lowest free memory after the chain)."""
        c = synth.make_case(name, seed=args.seed + rank, scale=scale)
        ta = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
        torch.cuda.synchronize(dev)
        free0 = torch.cuda.mem_get_info(dev)[0]
        pc = mhdproj.PressureProjection(c["dims"], c["h"], outlet=True, precision=args.precision, rel_tol=args.tol)
        pc.set_coefficients(ta(c["alpha"]), ta(c["solid"]), c["rho_liquid"], c["rho_air"])
        u0 = (ta(c["u"]), ta(c["v"]), ta(c["w"]))
        rng = np.random.default_rng(args.seed + 40)
        if "fu" in c:
            f = tuple(ta(c[k]) for k in ("fu", "fv", "fw"))
        else:
            f = tuple(ta((rng.standard_normal(x.shape) * 1e5 * (x != 0)).astype(np.float32)) for x in
                      (c["u"], c["v"], c["w"]))
        dt_c = 1e-6
        fwd = lambda prj: prj.chain_forward(u0, f, dt_c, steps, every)[2]
        bwd = lambda prj: prj.chain_backward(u0)[1]
        fwd(pc)
        bwd(pc)
        ms_f, st_f = timed(pc, reps, fwd)
        ms_b, _ = timed(pc, reps, bwd)
        # the objective summed over every state of the chain: its backward
        # pass recomputes each checkpoint segment's states from the checkpoint
        pc.chain_set_objective("summed")
        fwd(pc)
        bwd(pc)
        ms_fs, _ = timed(pc, reps, fwd)
        ms_bs, st_bs = timed(pc, reps, bwd)
        pc.chain_set_objective("final")
        summed = {"forward_ms": ms_fs / reps, "backward_ms": ms_bs / reps, "backward_over_forward": ms_bs / ms_fs,
                  "recomputed_steps": steps - (steps + every - 1) // every,
                  "backward_iterations": st_bs[-1].iterations}
        # a single projection of the same workload for projections/s
        us_c = (ta(c["u"]), ta(c["v"]), ta(c["w"]))
        out_c = tuple(torch.empty_like(x) for x in us_c)
        proj = lambda prj: prj.project(us_c, c["dt"], out=out_c)[2]
        proj(pc)
        ms_p, st_p = timed(pc, reps, proj)
        torch.cuda.synchronize(dev)
        used = free0 - torch.cuda.mem_get_info(dev)[0]
        pc.close()
        nx_, ny_, nz_ = c["dims"]
        peak_c, _ = hbm_peak()
        bytes_c = projection_bytes(nx_ * ny_ * nz_, st_p[-1].iterations, st_p[-1].refinements, args.precision)
        return {"projection_model_gb": bytes_c / 1e9,
                "projection_hbm_fraction": bytes_c / (ms_p / reps * 1e-3) / 1e9 / peak_c,
                "workload": f"{name}: {nx_}x{ny_}x{nz_} cells", "steps": steps, "checkpoint_every": every,
                "forward_ms": ms_f / reps, "backward_ms": ms_b / reps, "backward_over_forward": ms_b / ms_f,
                "projections_per_s": 1000.0 * reps / ms_p, "projection_ms": ms_p / reps,
                "iterations": st_p[-1].iterations, "true_relative_residual": st_p[-1].true_relative_residual,
                "device_memory_gb": used / 1e9, "summed_objective": summed}

    def em_leg(n, steps, warm=2):
        """EmState::step on the driven-ring workload (synth.em_ring): the
        bit-exact Jacobi-CG induction solve, fields and commit per step, timed
        on the EM context's stream.  Algorithmic bytes per CG iteration: the
        operator reads p, the edge flags and conductivity and writes A p
        (13 B/edge) plus the face reluctivities (about 4 B/edge); the residual
        update reads r, A p, x, p, the diagonal and conductivity and writes x,
        r and the diagonal (36 B/edge); the search update reads r, the
        diagonal and p and writes p (16 B/edge): 69 B per edge."""
        c = synth.em_ring(n)
        em = mhdproj.EmInduction(c["dims"], c["h"], dt_s=c["dt"], origin_m=c["origin"])
        em.set_materials(torch.from_numpy(c["materials"].view(np.int32)).to(dev), c["properties"])
        dt_e = c["dt"]
        fields_ = [torch.from_numpy(c["applied"](k * dt_e)).to(dev) for k in range(warm + steps + 1)]
        em.advance(0.0, initial=True, applied=fields_[0])
        for k in range(1, warm + 1):
            em.advance(k * dt_e, applied=fields_[k])
        counter = [warm]

        def em_step(e):
            counter[0] += 1
            return e.advance(counter[0] * dt_e, applied=fields_[counter[0]])

        l0 = em.kernel_launches()
        ms_e, ds = timed(em, steps, em_step)
        launches = em.kernel_launches() - l0
        its = sum(d.iterations for d in ds)
        em.close()
        per_it_ms = ms_e / max(its, 1)
        bytes_it = 69 * (3 * n * (n + 1) ** 2)
        peak_e, _ = hbm_peak()
        return {"workload": f"em_ring: {n}^3 cells, {3 * n * (n + 1) ** 2} edges, driven conducting annulus",
                "steps_per_s": 1000.0 * steps / ms_e, "ms_per_step": ms_e / steps, "iterations_per_step": its / steps,
                "ms_per_iteration": per_it_ms, "iteration_bytes": bytes_it,
                "GBps_per_iteration": bytes_it / (per_it_ms * 1e-3) / 1e9,
                "hbm_fraction_per_iteration": bytes_it / (per_it_ms * 1e-3) / 1e9 / peak_e,
                "relative_residual": ds[-1].relative_residual, "max_J": ds[-1].maxima[1],
                "kernel_launches_per_step": launches / steps}

    def em_sources_leg(n, segments, reps=5):
        """The source pass (src/em/source.wgsl): a wire loop of `segments`
        straight elements summed at every edge of an n^3 grid, timed on the
        EM stream.  About 60 flops, two logarithms and three square roots
        per edge-element interaction."""
        c = synth.em_ring(n)
        em = mhdproj.EmInduction(c["dims"], c["h"], dt_s=c["dt"], origin_m=c["origin"])
        el = synth.em_loop_elements(0.3 * n * c["h"], 100.0, segments, core=c["h"])
        em.evaluate_sources(el)
        ms_s, _ = timed(em, reps, lambda e: e.evaluate_sources(el))
        edges = em.edges
        em.close()
        sec = ms_s / reps * 1e-3
        return {"workload": f"{segments} wire segments at the {edges} edges of {n}^3 cells",
                "ms": ms_s / reps, "interactions_per_s": edges * segments / sec,
                "approx_tflops": 60.0 * edges * segments / sec / 1e12}

    def em_cpu_leg(n, warm=1):
        """The oracle's FP32 restatement of the same EM step on the host cores
        (OpenMP over edge groups), one timed step after `warm` steps."""
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as _o

        c = synth.em_ring(n)
        s = _o.EmSolve(c["dims"], c["h"], dt=c["dt"], origin=c["origin"])
        s.set_materials(c["materials"], c["properties"])
        s.advance(0.0, initial=True, applied=c["applied"](0.0))
        for k in range(1, warm + 1):
            s.advance(k * c["dt"], applied=c["applied"](k * c["dt"]))
        a = c["applied"]((warm + 1) * c["dt"])
        t0 = time.perf_counter()
        rc, st, _ = s.advance((warm + 1) * c["dt"], applied=a)
        sec = time.perf_counter() - t0
        el = synth.em_loop_elements(0.3 * n * c["h"], 100.0, 256, core=c["h"])
        t0 = time.perf_counter()
        s.evaluate_sources(el)
        src_sec = time.perf_counter() - t0
        edges = s.edges
        s.close()
        return {"steps_per_s": 1.0 / sec, "seconds_per_step": sec, "iterations": int(st[6]), "ok": rc == 0,
                "source_pass_interactions_per_s": edges * 256 / src_sec,
                "cores": os.cpu_count() or 1, "kind": "port",
                "sample": f"oracle/oracle_em.c on em_ring {n}^3, step {warm + 1} of the driven sequence"}

    pr = make(args.precision)
    if args.em:
        out_e = {"em_step128": em_leg(128, 5), "em_step64": em_leg(64, 5), "em_sources": em_sources_leg(128, 1024)}
        if rank == 0:
            print(json.dumps(out_e))
        pr.close()
        return
    if args.step:
        out_s = fluid_step_leg(2, 1)
        out_t = fluid_step_leg(2, 1, two_phase=True)
        if rank == 0:
            print(json.dumps({"fluid_step": out_s, "fluid_step_two_phase": out_t}))
        pr.close()
        return
    if args.kernels:
        step(pr)
        prof = pr.profile_kernels(reps=1)
        torch.cuda.synchronize(dev)
        if rank == 0:
            print(json.dumps({"kernels": [{"name": k["name"], "us": k["ms"] * 1e3, "bytes": k["bytes"]} for k in prof]}))
        pr.close()
        return
    for _ in range(args.warmup):
        step(pr)
    clocks = ClockSampler(local)
    clocks.start()
    k0 = pr.kernel_launches()
    ms, sts = timed(pr, args.steps)
    launches = pr.kernel_launches() - k0
    clk = clocks.stop()
    ms_per = ms / args.steps
    value = world * 1000.0 / ms_per
    its = [s.iterations for s in sts]
    res = [s.true_relative_residual for s in sts]
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": f"{args.precision} multigrid levels, fp32 CG, fp64 reductions",
        "data": "synthetic (seeded jet256 fields; no public dataset exists for this path)",
        "config": {
            "workload": f"{args.workload}: {nx}x{ny}x{nz} cells, rho 6440:1.2, top outlet, tol {args.tol:g}",
            "solver": "CG + red-black Gauss-Seidel aggregation V-cycle, FP64 refinement",
            "precision": args.precision,
            "parallelism": f"replicas x{world}",
            "l2": "inputs (286 MB) larger than L2 (129 MB); no flush",
            "iterations": its[-1],
            "refinements": sts[-1].refinements,
            "true_relative_residual": max(res),
        },
        "clocks": clk,
        "gpu_launches": launches,
    }
    peak0, _ = hbm_peak()
    pbytes = projection_bytes(nx * ny * nz, its[-1], sts[-1].refinements, args.precision)
    line["projection_hbm"] = {"model_gb": pbytes / 1e9, "achieved_gbs": pbytes / (ms_per * 1e-3) / 1e9,
                              "fraction": pbytes / (ms_per * 1e-3) / 1e9 / peak0,
                              "model": "N (95 + 24 R + 112 k) bytes: compulsory traffic of one projection"}
    if rank == 0 and not args.no_extras:
        # FP32-level comparator (same algorithm, FP32 multigrid fields)
        p32 = make("fp32")
        for _ in range(2):
            step(p32)
        ms32, st32 = timed(p32, max(3, args.steps // 2))
        ms32 /= len(st32)
        line["fp32_levels"] = {"projections_per_s": 1000.0 / ms32, "ms_per_step": ms32,
                               "iterations": st32[-1].iterations, "refinements": st32[-1].refinements,
                               "true_relative_residual": st32[-1].true_relative_residual}
        line["mixed_vs_fp32"] = (1000.0 / ms_per) / (1000.0 / ms32)
        p32.close()
        # BF16 levels, and the FP16 levels at a 1e-8 relative residual
        for key, prec, tol in (("bf16_levels", "bf16", args.tol), ("fp16_tol_1e-8", "fp16", 1e-8)):
            pv = mhdproj.PressureProjection(case["dims"], case["h"], outlet=True, precision=prec, rel_tol=tol)
            for _ in range(2):
                step(pv)
            msv, stv = timed(pv, max(3, args.steps // 2))
            msv /= len(stv)
            line[key] = {"projections_per_s": 1000.0 / msv, "ms_per_step": msv, "iterations": stv[-1].iterations,
                         "refinements": stv[-1].refinements,
                         "true_relative_residual": stv[-1].true_relative_residual}
            pv.close()
        # adjoint / forward cost on the same coefficients
        gu = tuple(torch.randn_like(x) for x in us)

        def vjp_step(prj):
            _, st = prj.vjp(gu, None, case["dt"])
            return st

        def fwd_only(prj):
            _, _, st = prj.project(us, case["dt"], out=out)
            return st

        pr.set_coefficients(alpha, solid, case["rho_liquid"], case["rho_air"])
        msf, _ = timed(pr, 3, fwd_only)
        msa, sta = timed(pr, 3, vjp_step)
        line["adjoint_over_forward"] = msa / msf
        line["adjoint"] = {"iterations": sta[-1].iterations, "refinements": sta[-1].refinements,
                           "ms": msa / 3, "forward_ms": msf / 3}
        # end to end through the C ABI with host buffers (pinned)
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
        h_alpha, h_solid = pin(case["alpha"]), pin(case["solid"])
        h_us = tuple(pin(case[k]) for k in ("u", "v", "w"))
        h_out = tuple(pin(np.empty_like(case[k])) for k in ("u", "v", "w"))
        h_p = pin(np.empty((nz, ny, nx), np.float32))
        pe = make(args.precision)
        for _ in range(2):
            pe.project_host(h_alpha, h_solid, case["rho_liquid"], case["rho_air"], h_us, case["dt"], out=h_out,
                            p_out=h_p)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        ke = max(3, args.steps // 2)
        for _ in range(ke):
            pe.project_host(h_alpha, h_solid, case["rho_liquid"], case["rho_air"], h_us, case["dt"], out=h_out,
                            p_out=h_p)
        torch.cuda.synchronize(dev)
        e2e_s = (time.perf_counter() - t0) / ke
        h2d = h_alpha.nbytes + h_solid.nbytes + sum(a.nbytes for a in h_us)
        d2h = sum(a.nbytes for a in h_out) + h_p.nbytes
        line["e2e"] = {"value": world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                       "d2h_bytes_per_step": int(d2h)}
        pe.close()
        # the GB300 solver on the reference's own closed boundaries (no
        # outlet; each component pinned at its root cell) and the same inputs
        # as the reference arm, device-resident and end to end
        pc = mhdproj.PressureProjection(case["dims"], case["h"], outlet=False, precision=args.precision,
                                        rel_tol=args.tol)
        try:
            for _ in range(2):
                step(pc)
            msc, stc = timed(pc, max(3, args.steps // 2))
            msc /= len(stc)
            for _ in range(2):
                pc.project_host(h_alpha, h_solid, case["rho_liquid"], case["rho_air"], h_us, case["dt"], out=h_out,
                                p_out=h_p)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            for _ in range(ke):
                pc.project_host(h_alpha, h_solid, case["rho_liquid"], case["rho_air"], h_us, case["dt"], out=h_out,
                                p_out=h_p)
            torch.cuda.synchronize(dev)
            e2e_c = (time.perf_counter() - t0) / ke
            line["closed256"] = {"workload": f"{args.workload}: {nx}x{ny}x{nz} cells, closed boundaries (the "
                                             f"reference's), tol {args.tol:g}",
                                 "projections_per_s": 1000.0 / msc, "ms_per_step": msc,
                                 "iterations": stc[-1].iterations, "refinements": stc[-1].refinements,
                                 "true_relative_residual": stc[-1].true_relative_residual,
                                 "e2e": {"value": 1.0 / e2e_c, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                                         "d2h_bytes_per_step": int(d2h)}}
        except mhdproj.ProjectionError as exc:
            line["closed256"] = {"unavailable": str(exc)}
        pc.close()
        # roofline of the dominant kernel (isolated launches, CUDA events on the library stream)
        pr.set_coefficients(alpha, solid, case["rho_liquid"], case["rho_air"])
        step(pr)
        prof = pr.profile_kernels(reps=20)
        peak, peak_src = hbm_peak()
        best = max((k for k in prof if k["per_iteration"] > 0), key=lambda k: k["ms"] * k["per_iteration"])
        achieved = best["bytes"] / (best["ms"] * 1e-3) / 1e9
        line["roofline"] = {"bound": "hbm", "kernel": best["name"], "achieved": achieved, "peak": peak,
                            "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_src,
                            "traffic": measured_traffic(args.workload, args.precision, best["name"]),
                            "algorithmic_bytes_per_launch": best["bytes"]}
        line["kernels"] = [{"name": k["name"], "us": k["ms"] * 1e3,
                            "GBps": k["bytes"] / (k["ms"] * 1e-3) / 1e9 if k["bytes"] > 0 and k["ms"] > 0 else None,
                            "per_iteration": k["per_iteration"]} for k in prof]
        # share of a projection spent below the finest level: one coarse-grid
        # correction per CG iteration plus one per refinement pass start
        crs = next((k for k in prof if k["name"] == "coarse_levels"), None)
        if crs is not None:
            cycles = its[-1] + sts[-1].refinements + 1
            line["coarse_levels"] = {"us_per_vcycle": crs["ms"] * 1e3, "vcycles": cycles,
                                     "share_of_step": crs["ms"] * cycles / ms_per}
        # gauge/topology labelling of the solid mask on the GPU (union-find,
        # four kernels), run when the mask changes
        topo = next((k for k in prof if k["name"] == "topology"), None)
        if topo is not None:
            line["topology"] = {"gpu_us": topo["ms"] * 1e3, "GBps": topo["bytes"] / (topo["ms"] * 1e-3) / 1e9,
                                "bytes_per_cell": topo["bytes"] / (nx * ny * nz)}
        # the reference algorithm on this GPU: the bit-exact CUDA port of its
        # FP32 multigrid CG (closed boundaries), for the algorithmic gap
        try:
            pref = mhdproj.PressureProjection(case["dims"], case["h"], outlet=False, solver="reference",
                                              rel_tol=args.tol, abs_div_tol=0.0, max_iterations=20000)
            pref.set_coefficients(alpha, solid, case["rho_liquid"], case["rho_air"])

            def ref_step(prj):
                _, _, st = prj.project(us, case["dt"], out=out)
                return st

            ref_step(pref)
            msr, str_ = timed(pref, 3, ref_step)
            line["reference_algorithm_gpu"] = {"projections_per_s": 3000.0 / msr, "ms_per_step": msr / 3,
                                               "iterations": str_[-1].iterations,
                                               "relative_residual": str_[-1].relative_residual,
                                               "boundary": "closed (the reference has no outlet)"}
            pref.close()
        except mhdproj.ProjectionError as exc:
            line["reference_algorithm_gpu"] = {"unavailable": str(exc)}
        # the 128^3 adjoint chain (K = 8 steps, checkpoints every 4) and the
        # 512x256x256 liquid column (K = 4): forward, gradient, projection
        # throughput and device memory
        line["adjoint128_chain"] = chain_leg("adjoint128", 1.0, 8, 4, 3)
        line["column512"] = chain_leg("column512", 1.0, 4, 4, 3)
        for key, tp in (("fluid_step", False), ("fluid_step_two_phase", True)):
            try:
                line[key] = fluid_step_leg(5, 10, two_phase=tp)
            except mhdproj.ProjectionError as exc:
                line[key] = {"unavailable": str(exc)}
        # the EM induction step (src/em): 128^3 on the GPU, and 64^3 on the GPU
        # beside the oracle's CPU restatement of the same step
        try:
            line["em_step"] = em_leg(128, 5)
            e64 = em_leg(64, 5)
            if rank == 0 and world == 1:
                e64["cpu_baseline"] = em_cpu_leg(64)
            line["em_step64"] = e64
            line["em_sources"] = em_sources_leg(128, 1024)
        except mhdproj.ProjectionError as exc:
            line["em_step"] = {"unavailable": str(exc)}
        # CPU leg: whole projections of the reference algorithm on the host
        # cores, then the FP64 oracle as the checker of the 256^3 results
        cpu_leg(args, case, line, outputs_for_accuracy(args, case, mhdproj, torch, dev, alpha, solid, us))
    pr.close()
    if rank == 0:
        print(json.dumps(line))
    if pg is not None:
        pg.destroy_process_group()


def outputs_for_accuracy(args, case, mhdproj, torch, dev, alpha, solid, us):
    """The workload projected with FP16 and BF16 multigrid levels at 1e-6 and
    1e-8 (untimed), copied to the host for the FP64 check."""
    import numpy as np

    runs = {}
    for prec in ("fp16", "bf16"):
        for tol in (1e-6, 1e-8):
            pa = mhdproj.PressureProjection(case["dims"], case["h"], outlet=True, precision=prec, rel_tol=tol)
            pa.set_coefficients(alpha, solid, case["rho_liquid"], case["rho_air"])
            (u, v, w), p, st = pa.project(us, case["dt"])
            torch.cuda.synchronize(dev)
            runs[(prec, tol)] = dict(u=u.cpu().numpy(), v=v.cpu().numpy(), w=w.cpu().numpy(), p=p.cpu().numpy(),
                                     iterations=st.iterations, true_relative_residual=st.true_relative_residual)
            pa.close()
    return runs


def cpu_leg(args, case, line, runs):
    """The CPU leg of the bench (rank 0, N = 1).

    cpu_baseline: the oracle's restatement of the reference projection (the
    reference's FP32 aggregation-multigrid CG, closed boundaries: the
    reference has no outlet) timed as whole projections of the workload on
    every host thread, one untimed then two timed.  `vs_cpu_reference` sets
    the GPU legs against it: the outlet headline, and the GB300 solver on the
    same closed problem.

    accuracy: the FP64 oracle (onat_project, 1e-12) solves the workload and
    checks the GPU outputs of `runs`: max and relative-L2 errors of the
    pressure and of the face velocities (all three arrays together)."""
    import numpy as np

    nx, ny, nz = case["dims"]
    threads = os.cpu_count() or 1
    cref = CpuReference(case, threads, args.tol)
    secs, res = cref.projections(2, warmup=1)
    cpu_s = statistics.median(secs)
    line["cpu_baseline"] = {
        "value": 1.0 / cpu_s, "unit": UNIT, "cores": threads, "kind": "port",
        "sample": f"2 whole projections (after 1 untimed) of the oracle's restatement of the reference FP32 "
                  f"multigrid CG on {args.workload} {nx}x{ny}x{nz}, closed boundaries (the reference has no outlet), "
                  f"to {args.tol:g}: {res.iterations} CG iterations each; {threads} OpenMP threads",
        "seconds_per_projection": cpu_s, "iterations": int(res.iterations), "status": int(res.status)}
    if "topology" in line:
        line["topology"]["host_search_ms"] = cref.anchors_s * 1e3
        line["topology"]["host_search"] = "the reference's anchors() breadth-first search (oracle), 1 thread"
    cpu_rate = 1.0 / cpu_s
    ratios = {"outlet_over_closed_cpu": line["value"] / cpu_rate}
    if "e2e" in line:
        ratios["outlet_e2e_over_closed_cpu"] = line["e2e"]["value"] / cpu_rate
    if "projections_per_s" in line.get("closed256", {}):
        ratios["closed_over_closed_cpu"] = line["closed256"]["projections_per_s"] / cpu_rate
        ratios["closed_e2e_over_closed_cpu"] = line["closed256"]["e2e"]["value"] / cpu_rate
    line["vs_cpu_reference"] = ratios
    # accuracy against the FP64 oracle
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    g = oracle.grid(nx, ny, nz, case["h"], case["rho_liquid"], case["rho_air"], case["periodic"], case["outlet"])
    t0 = time.perf_counter()
    ref = oracle.project(g, case["alpha"], case["solid"], case["u"], case["v"], case["w"], case["dt"], 1e-12)
    t_ref = time.perf_counter() - t0
    ref_u = np.concatenate([ref[k] for k in "uvw"])
    ref_p = ref["p"]
    acc = {"oracle": f"FP64 onat_project to 1e-12 ({ref['iterations']} iterations, {t_ref:.1f} s on {threads} threads)",
           "pressure_max": float(np.abs(ref_p).max()), "velocity_max": float(np.abs(ref_u).max())}
    for (prec, tol), r in runs.items():
        gu = np.concatenate([r[k].reshape(-1).astype(np.float64) for k in "uvw"])
        gp = r["p"].reshape(-1).astype(np.float64)
        acc[f"{prec}@{tol:g}"] = {
            "iterations": r["iterations"], "true_relative_residual": r["true_relative_residual"],
            "p_max_abs_error": float(np.abs(gp - ref_p).max()),
            "p_rel_l2_error": float(np.linalg.norm(gp - ref_p) / np.linalg.norm(ref_p)),
            "u_max_abs_error": float(np.abs(gu - ref_u).max()),
            "u_rel_l2_error": float(np.linalg.norm(gu - ref_u) / np.linalg.norm(ref_u))}
    line["accuracy"] = acc


def projection_bytes(n, iterations, refinements, precision):
    """Compulsory HBM bytes of one projection: N (95 + 24 R + k (52 + 60))
    with FP16/BF16 levels, N (95 + 24 R + 148 k) with FP32 levels (k CG
    iterations, R refinement residuals after the first pass)."""
    per_it = 112.0 if precision != "fp32" else 148.0
    return n * (95.0 + 24.0 * refinements + per_it * iterations)


def measured_traffic(workload, precision, kernel):
    """DRAM bytes (read + write) of one launch of `kernel` from the committed
    ncu summary (profiles/traffic.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            rec = json.load(f)
        return rec[f"{workload}/{precision}"][kernel]
    except (OSError, KeyError, ValueError):
        return None


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s"


# ------------------------------------------------------- reference arm
def run_reference(args):
    world, rank, local, pg = dist_setup(args)
    if rank != 0:
        if pg is not None:
            pg.destroy_process_group()
        return
    from mhdproj import synth

    case = synth.make_case(args.workload, seed=args.seed)
    nx, ny, nz = case["dims"]
    threads = os.cpu_count() or 1
    cref = CpuReference(case, threads, args.tol)
    # Each step: one whole projection of the reference algorithm (coefficient
    # cache, multigrid build, every CG iteration to the tolerance).
    secs, res = cref.projections(args.steps, warmup=args.warmup)
    total = sum(secs)
    value = args.steps / total
    sample = (f"per step: one whole projection by the oracle's restatement of the reference FP32 multigrid CG on "
              f"{nx}x{ny}x{nz} (closed boundaries), {res.iterations} CG iterations to {args.tol:g} "
              f"(status {res.status}); {threads} OpenMP threads")
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32",
        "data": "synthetic (seeded jet256 fields)",
        "config": {"workload": f"{args.workload}: {nx}x{ny}x{nz} cells, closed boundaries (the reference has no outlet), "
                               f"tol {args.tol:g}",
                   "iterations": int(res.iterations), "relative_residual": float(res.residual),
                   "seconds_per_projection": [round(x, 3) for x in secs]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
