#!/usr/bin/env python
"""Benchmark of the element assembly on GB300.

Workload (one "step"): one Newton 'NRP' bulk assembly -- setEquationsBulk with
the FP64 residual and the FP64 forward-difference Jacobian (56 residual
evaluations per element, the reference algorithm, bit-exact) -- on the
cylinder-in-channel mesh with 40,000 Q2 quads, Giesekus alpha = 0.1,
beta = 0.59, Wi = 0.5, square-root conformation (SQRT) form, arclength
unknown (Nex = 1).  Synthetic seeded state (no dataset exists for this path).

* value: elements/s with the state resident in HBM (vefem_assemble with
  device pointers), CUDA events on the library's stream over the timed steps;
* e2e: the same metric through the C ABI with pinned host buffers: the host
  TL/EU go in and the residual and all AIJ values come back every step;
* roofline: the FD kernel is bound by the FP64 pipe; achieved = algorithmic
  FP64 operations per launch (counted from the kernel source, see
  vefem_algorithmic_ops) / its event-timed duration, peak = the FP64
  instruction rate measured live on this GPU by a probe kernel;
* cpu_baseline: the CPU oracle (a C restatement of the reference algorithm)
  on all host cores, on a bounded sample of the same workload;
* continuation: the metric's continuation comparison, Wi 0.1 -> 1.0 by
  pseudo-arclength on the 20,000-quad mesh (``--cont-nel``): the plain FP64
  path (FD64 Jacobian, tangent predictor, the reference's factorisation reuse)
  against the learned + mixed path (FP32 Jacobian, learned predictor,
  contraction-monitored reuse), both with the GPU frontal LU; wall time,
  steps/s, Newton iterations, factorisations and the wall-time ratio.
  ``--ablations`` and ``--secant`` add arms; ``--continuation-only`` runs
  only this comparison;
* newton_precision: the precision form's Newton solves on 40,000 quads
  (Giesekus, SQRT; ``--newton-nel``): FP64 forward-difference Jacobian
  against FP32 exact Jacobian + FP64 residual, iterations, factorisations and
  the converged solution's error against the FP64 one, every run;
* batched: the batched form, 64 instances of 2,000-20,000 quads at Wi in
  [0.1, 1.0], one persistent launch per kernel replayed as a CUDA graph,
  against one call per instance;
* stability: the linear-stability A/B assembly for 16 spanwise wavenumbers
  on 20,000 quads (``--stab-nel``), with the CPU oracle on a sample.

``--impl reference`` times that CPU implementation as the reference arm.
Multi-GPU: the assembly of one mesh does not shard across GPUs in this
library (replicas only): under torchrun every rank runs its own instance and
``value`` is the total over ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import dataclasses
import faulthandler
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from ve_flow_around_cylinder_fortran_gb300 import build as B  # noqa: E402
from ve_flow_around_cylinder_fortran_gb300 import mesh as M  # noqa: E402
from ve_flow_around_cylinder_fortran_gb300 import pattern as P  # noqa: E402
from ve_flow_around_cylinder_fortran_gb300 import state as S  # noqa: E402
from ve_flow_around_cylinder_fortran_gb300 import vefem as V  # noqa: E402

METRIC = "Continuation steps/s learned+mixed vs plain FP64 GPU at ||R||<1e-10; elem/s"
UNIT = "elem/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["vefem", "reference"], default="vefem")
    ap.add_argument("--nel", type=int, default=40000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cont-nel", type=int, default=20000,
                    help="mesh of the continuation comparison (0 = skip it)")
    ap.add_argument("--cont-wi", type=float, default=1.0, help="Wi the continuation ends at")
    ap.add_argument("--cont-log", action="store_true",
                    help="with --continuation-only: every Newton iteration and step on stderr")
    ap.add_argument("--secant", action="store_true",
                    help="add the secant-predictor arm to the continuation comparison")
    ap.add_argument("--ablations", action="store_true",
                    help="add the ablation arms to the continuation comparison (the learned arm "
                         "with the reference's reuse rules; POD extrapolation without the network)")
    ap.add_argument("--cont-arms", default="",
                    help="comma-separated arm names of the continuation comparison to run "
                         "(default: all)")
    ap.add_argument("--krylov", type=int, default=0,
                    help="GMRES iterations allowed per Newton-Krylov correction of the learned + "
                         "mixed arm, in place of a new factorisation (0: chord steps only)")
    ap.add_argument("--newton-nel", type=int, default=40000,
                    help="mesh of the precision-form Newton comparison in the default line "
                         "(0 = skip it)")
    ap.add_argument("--newton-only", type=int, default=0, metavar="NEL",
                    help="only the precision-form Newton comparison (FP64 vs FP32 Jacobian, "
                         "natural continuation Wi 0.1, 0.2, 0.3, 0.4, 0.5) on a mesh of NEL quads")
    ap.add_argument("--linear-solver", choices=["auto", "frontal", "superlu"], default="auto",
                    help="linear solver of the Newton and continuation legs (auto: the GPU "
                         "frontal LU from 1,000 elements on, host SuperLU below)")
    ap.add_argument("--continuation-only", action="store_true",
                    help="run only the continuation comparison and print its JSON line")
    ap.add_argument("--batch-inst", type=int, default=64,
                    help="instances of the batched-form measurement (0 = skip it)")
    ap.add_argument("--stab-nel", type=int, default=20000,
                    help="mesh of the linear-stability measurement (0 = skip it)")
    ap.add_argument("--only", choices=["fd64", "residual", "exact64", "exact32", "stability",
                                       "frontal"],
                    default=None,
                    help="time one assembly form alone on the --nel workload (profiling case)")
    return ap.parse_args()


def workload(nel: int):
    mesh = M.build_cylinder_mesh(nel)
    phys = S.giesekus(alpha=0.1, Wi=0.5, beta=0.59, form="SQRT", nex=1)
    TL, EU = S.seeded_state(mesh.xyz, phys, seed=0)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, phys.nex)
    cfg = {
        "workload": f"cylinder-in-channel (R=1, y in [-2,2], x in [-15,25]), {mesh.nel} Q2 quads, "
                    "Giesekus alpha=0.1, beta=0.59, Wi=0.5, SQRT form, Nex=1; one Newton 'NRP' "
                    "bulk assembly: FP64 residual + FP64 forward-difference Jacobian into AIJ",
        "nel": mesh.nel, "nnodes": mesh.nnodes, "dofs": int(len(rowptr) - 1),
        "nnz": int(len(colind)), "seed": 0,
        "l2": "no flush: every step streams > 1 GB (element scratch + AIJ values), "
              "well above the 129 MB L2",
    }
    return mesh, phys, TL, EU, rowptr, colind, cfg


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,utilization.gpu,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-i", str(self.device), "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 10:
                continue
            try:
                rows.append(dict(sm=float(f[1]), smax=float(f[2]), power=float(f[3]),
                                 util=float(f[4]), hw=f[6], hwt=f[7], swt=f[8], swp=f[9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        load = [r for r in rows if r["util"] >= 50] or rows
        reasons = set()
        for r in load:
            for k, name in (("hw", "hw_slowdown"), ("hwt", "hw_thermal_slowdown"),
                            ("swt", "sw_thermal_slowdown"), ("swp", "sw_power_cap")):
                if r[k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r["sm"] for r in load),
                "sm_max_mhz": max(r["smax"] for r in load), "samples": len(load),
                "reasons": sorted(reasons)}


def dist_setup(backend: str = "nccl"):
    """torchrun environment: one process per GPU (replicas: each rank assembles
    its own instance; the only collectives are the barrier and the max of the
    timings).  backend "gloo" serves the CPU tests of this path."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local, dist


def max_over_ranks(x: float, dist, device=None) -> float:
    """The largest x over all ranks (the job's time is its slowest rank's)."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world: int, units_per_rank: float, steps: int, seconds: float) -> float:
    """Whole-job throughput of replicas: every rank processes units_per_rank per
    step, the job time is the slowest rank's."""
    return world * units_per_rank * steps / seconds


def fp64_peak(device: int):
    lib = ctypes.CDLL(B.PROBE)
    lib.vefem_probe_fp64.argtypes = [ctypes.c_int, ctypes.c_void_p]
    out = np.zeros(3)
    rc = lib.vefem_probe_fp64(device, out.ctypes.data)
    if rc:
        raise RuntimeError(f"FP64 probe failed: {rc}")
    return {"dfma_inst_per_s": out[0], "dadd_inst_per_s": out[1], "dmul_inst_per_s": out[2]}


def measured_hbm_gbs():
    """The machine's measured copy bandwidth (GB/s), if the file is present."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


def fp32_peak(device: int) -> float:
    """FFMA instructions/s of a probe kernel on this GPU."""
    lib = ctypes.CDLL(B.PROBE)
    lib.vefem_probe_fp32.argtypes = [ctypes.c_int, ctypes.c_void_p]
    out = np.zeros(1)
    rc = lib.vefem_probe_fp32(device, out.ctypes.data)
    if rc:
        raise RuntimeError(f"FP32 probe failed: {rc}")
    return float(out[0])


def algorithmic_ops(phys, flags):
    L = V.load()
    L.vefem_algorithmic_ops.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    out = np.zeros(6)
    p = V.make_params(phys)
    if L.vefem_algorithmic_ops(ctypes.byref(p), flags, out.ctypes.data):
        raise RuntimeError("vefem_algorithmic_ops failed")
    return out


def cpu_oracle_rate(phys, mesh, TL, EU, rowptr, colind, target_s: float, reps: int,
                    threads: int = 0):
    """Elements/s of the oracle assembly on ``threads`` host cores (0: all),
    on the first n elements of the mesh, n sized for about target_s seconds
    per repetition."""
    from oracle import oracle as O
    cores = threads or os.cpu_count() or 1
    conn = mesh.conn
    n0 = min(mesh.nel, 512)
    t = time.perf_counter()
    O.assemble(phys, np.ascontiguousarray(conn[:, :n0]), mesh.xyz, TL, EU, rowptr, colind,
               nthreads=cores)
    rate0 = n0 / (time.perf_counter() - t)
    n = int(min(mesh.nel, max(n0, rate0 * target_s)))
    sub = np.ascontiguousarray(conn[:, :n])
    times = []
    for _ in range(reps):
        t = time.perf_counter()
        O.assemble(phys, sub, mesh.xyz, TL, EU, rowptr, colind, nthreads=cores)
        times.append(time.perf_counter() - t)
    return n / statistics.median(times), n, cores, times


def traffic_per_element():
    path = os.path.join(ROOT, "profiles", "k_fd64_dram.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("dram_bytes_per_element")
    return None


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    mesh, phys, TL, EU, rowptr, colind, cfg = workload(args.nel)
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    # size each step as a bounded sample of the workload (about 3 s of CPU work)
    _, n, _, _ = cpu_oracle_rate(phys, mesh, TL, EU, rowptr, colind, 3.0, 1)
    sub = np.ascontiguousarray(mesh.conn[:, :n])
    for _ in range(args.warmup):
        O.assemble(phys, sub, mesh.xyz, TL, EU, rowptr, colind, nthreads=cores)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        O.assemble(phys, sub, mesh.xyz, TL, EU, rowptr, colind, nthreads=cores)
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = n * args.steps / total
    sample = f"first {n} of {mesh.nel} elements per step (full residual + FD Jacobian into AIJ)"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": cfg,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample, "flags": O.build_flags(), "cpu_model": O.cpu_model()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference (Fortran + PETSc + MPI) cannot be built on this machine or the "
                "GPU box (no Fortran compiler); its algorithm runs as the C oracle port, "
                "OpenMP over elements, sequential element-ordered AIJ adds",
    }
    print(json.dumps(line))
    return 0


def continuation_compare(nel: int, wi_end: float = 1.0, device: int = 0, log=None,
                         secant: bool = True, step_log=None, ablations: bool = True,
                         only=None, linear_solver: str = "auto", krylov: int = 0):
    """Arclength continuation Wi 0.1 -> wi_end (Oldroyd-B, beta = 0.59, SQRT
    form) on the GPU assembly, arms from the same start: the plain FP64 path
    (FD64 Jacobian, the reference's tangent predictor), the same with a
    secant predictor, the learned + mixed path (FP32 exact Jacobian with FP64
    residual, learned POD/MLP predictor: cubic extrapolation in the POD space
    of the converged points from the 4th point on, corrected by the network
    trained online after the first 20 points; factorisations reused across
    steps while chord iterations contract), and two ablations: the learned
    arm with the reference's factorisation-reuse rules, and the contraction
    policy without the network (the reduced-space extrapolation alone).
    Every point is converged to ||R|| < 1e-10 and ||dx|| < 1e-10; host wall
    time per arm.  All arms share one linear solver (``linear_solver``: the
    GPU frontal LU, or the host SuperLU on small meshes), whose one-time
    symbolic phase is timed apart."""
    from ve_flow_around_cylinder_fortran_gb300 import continuation as C
    from ve_flow_around_cylinder_fortran_gb300 import learned as LP
    from ve_flow_around_cylinder_fortran_gb300 import linsolve as LS
    from ve_flow_around_cylinder_fortran_gb300 import newton as NW
    mesh = M.build_cylinder_mesh(nel)
    phys = S.oldroyd_b(0.1, 0.59, "SQRT", nex=1)
    TL, EU = NW.initial_state(mesh, phys)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, phys.nex)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind, outlet_edges=True, device=device)
    t_sym = time.perf_counter()
    solver = LS.make_solver(linear_solver, rowptr, colind, mesh)
    t_sym = time.perf_counter() - t_sym
    solver_name = type(solver).__name__
    cfg = C.ArclengthSettings(dArN=0.01, lam_max=wi_end / phys.Wi0, max_steps=2000)
    # the learned + mixed arm reuses factorisations across steps while chord
    # iterations contract (theta < 0.6), cuts a failed step back (dS halved,
    # predicted again) before relaxing, and checks its solves to 1e-8 relative
    # residual (an inexact Newton by design); the plain arm keeps the
    # reference's rules and the solver's 1e-10 check
    chord = dataclasses.replace(cfg, reuse="contraction", theta_max=0.6, cutbacks=4,
                                krylov=krylov, solve_check_tol=1.0e-8)
    arms, states = {}, {}
    runs = [("plain_fp64", "fd64", None, cfg), ("learned_fp32", "exact32", "learned", chord),
            ("learned_fp32_reference_reuse", "exact32", "learned", cfg),
            ("pod_cubic_fp32", "exact32", "ablate", chord)]
    if secant:
        runs.insert(1, ("secant_fp64", "fd64", "secant", cfg))
    if not ablations:
        runs = [r for r in runs if r[0] not in ("learned_fp32_reference_reuse", "pod_cubic_fp32")]
    if only:
        runs = [r for r in runs if r[0] in only]
    for name, jac, kind, arm_cfg in runs:
        cont = C.ArclengthContinuation(asm, mesh, phys, jac, arm_cfg, log=step_log,
                                       linear_solver=solver)
        if step_log:
            step_log(f"arm {name}")
        pred = None
        if kind in ("learned", "ablate"):
            pred = LP.LearnedPredictor(n_modes=32, start=20, device=f"cuda:{device}",
                                       use_net=kind == "learned")
            pred.warm_up(len(rowptr) - 1)      # one-time framework start-up, not timed
        elif kind == "secant":
            pred = C.SecantPredictor()
        t0 = time.perf_counter()
        recs, xs = cont.run(TL, EU, predictor=pred)
        wall = time.perf_counter() - t0
        if kind in ("learned", "ablate"):
            pred.net.close()
        states[name] = xs
        arms[name] = {
            "jacobian": jac,
            "predictor": {"learned": "learned POD/MLP", "secant": "secant", None: "tangent",
                          "ablate": "POD cubic extrapolation, network off"}[kind],
            "solve_check_rel_residual": arm_cfg.solve_check_tol
            if arm_cfg.solve_check_tol is not None else getattr(solver, "check_tol", None),
            "factorisation_reuse": arm_cfg.reuse if arm_cfg.reuse == "reference"
            else f"contraction (theta_max {arm_cfg.theta_max}), {arm_cfg.cutbacks} step cutbacks"
            + (f", Newton-Krylov corrections (GMRES <= {arm_cfg.krylov} iterations, rtol "
               f"{arm_cfg.krylov_rtol:g}) before a new factorisation" if arm_cfg.krylov else ""),
            "gmres_iterations": cont.krylov_iterations, "gmres_misses": cont.krylov_failures,
            "wall_s": wall, "steps": len(recs), "steps_per_s": len(recs) / wall,
            "newton_iterations": sum(r.newton_iterations for r in recs),
            "factorisations": sum(r.factorisations for r in recs),
            "learned_taken": sum(r.predictor == "learned" for r in recs),
            "extrapolation_taken": sum(r.predictor == "extrapolation" for r in recs),
            "mean_err_pr_after_20": float(np.mean([r.pred_error for r in recs[20:]]))
            if len(recs) > 20 else None,
            "emergency_restarts": sum(r.emergencies for r in recs),
            "step_cutbacks": sum(r.cutbacks for r in recs),
            "singular_factorisations": cont.failed_factorisations,
            "final_wi": recs[-1].wi, "max_final_res_norm": max(r.res_norm for r in recs),
            "time_split_s": {"assembly": sum(r.assembly_s for r in recs),
                             "lu_factor": sum(r.factor_s for r in recs),
                             "lu_solve": sum(r.solve_s for r in recs),
                             "predictor": sum(r.predictor_s for r in recs)},
            "mean_dS_after_20": float(np.mean([r.dS for r in recs[20:]])) if len(recs) > 20 else None,
        }
        if kind in ("learned", "ablate"):
            arms[name]["predictor_split_s"] = dict(pred.timers, judge=cont.judge_s)
        if log:
            log(f"{name}: {arms[name]}")
    asm.close()
    out = {
        "workload": f"arclength continuation Wi 0.1 -> {wi_end}, Oldroyd-B beta=0.59, SQRT form, "
                    f"{mesh.nel} Q2 quads ({len(rowptr) - 1} unknowns), LN0=1, dArN=0.01, "
                    f"Eps_Pr=1e-3, dS0=1, dS_max=50; linear solver: {_solver_desc(solver)}",
        "linear_solver": solver_name, "solver_setup_s": t_sym,
        "arms": arms,
    }
    if "plain_fp64" not in states or "learned_fp32" not in states:
        return out
    # the learned arm's points against the plain arm's branch (linear interpolation in lambda)
    xp = states["plain_fp64"]
    lp = np.array([x[-1] for x in xp])
    dev = 0.0
    for x in states["learned_fp32"][1:-1]:
        k = int(np.searchsorted(lp, x[-1]))
        if 0 < k < len(lp):
            w = (x[-1] - lp[k - 1]) / (lp[k] - lp[k - 1])
            ref = (1 - w) * xp[k - 1] + w * xp[k]
            dev = max(dev, float(np.linalg.norm(x - ref) / np.linalg.norm(ref)))
    out.update({
        "speedup_wall": arms["plain_fp64"]["wall_s"] / arms["learned_fp32"]["wall_s"],
        "speedup_factorisations": arms["plain_fp64"]["factorisations"]
        / max(1, arms["learned_fp32"]["factorisations"]),
        "branch_max_rel_dev": dev,
    })
    return out


def _solver_desc(solver) -> str:
    if type(solver).__name__ == "FrontalLU":
        return (f"GPU panel-frontal LU, FP64 ({solver.npan} panels of {solver.G} elements, "
                f"{solver.flops / 1e12:.2f} TFLOP per factorisation)")
    return "host SuperLU (nested dissection)"


def newton_precision_compare(nel: int, device: int = 0, wis=(0.1, 0.2, 0.3, 0.4, 0.5),
                             linear_solver: str = "auto"):
    """Precision form on one Newton solve per Weissenberg number: Giesekus
    alpha = 0.1, beta = 0.59, SQRT form, natural continuation through ``wis``
    from the fully developed start, each point to ||R|| < 1e-10 and
    ||dx|| < 1e-10, once with the FP64 forward-difference Jacobian (the
    reference algorithm; its iterates equal the oracle-driven Newton's bit for
    bit) and once with the FP32 exact Jacobian beside the FP64 residual.
    Reports iterations, factorisations and host time per solve, and the FP32
    run's converged state against the FP64 one."""
    from ve_flow_around_cylinder_fortran_gb300 import linsolve as LS
    from ve_flow_around_cylinder_fortran_gb300 import newton as NW
    mesh = M.build_cylinder_mesh(nel)
    phys = S.giesekus(0.1, wis[0], 0.59, "SQRT", nex=0)
    rowptr, colind = P.build_pattern(mesh.element_nodes(), mesh.nnodes, phys.nex)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind, outlet_edges=True, device=device)
    t_sym = time.perf_counter()
    solver = LS.make_solver(linear_solver, rowptr, colind, mesh)
    t_sym = time.perf_counter() - t_sym
    runs, final = {}, {}
    # the FP32 arm first: a refused pivot of the other arm would leave the
    # shared solver with delayed pressures (larger fronts) for the rest
    for jac in ("exact32", "fd64"):
        t0 = time.perf_counter()
        # a point whose Newton iteration diverges, or has not converged after
        # 20 iterations, ends the run (no emergency restarts: relaxed Newton
        # at this size takes minutes per attempt); the points before it are
        # reported
        res = NW.natural_continuation(asm, mesh, phys, list(wis), jacobian=jac, tol=1e-10,
                                      linear_solver=solver, max_restarts=0,
                                      stop_on_failure=True, max_iter=20)
        wall = time.perf_counter() - t0
        runs[jac] = {
            "wall_s": wall,
            "reached_wi": wis[len(res) - 1] if res else None,
            "stopped_at_wi": wis[len(res)] if len(res) < len(wis) else None,
            "solves": [{"wi": wi, "iterations": r.iterations,
                        "factorisations": sum(h["flag"] == "NRP" for h in r.history),
                        "final_res_norm": r.history[-1]["res_norm"],
                        "assembly_s": r.assembly_s, "factor_and_solve_s": r.solve_s}
                       for wi, r in zip(wis, res)],
        }
        final[jac] = [r.TL for r in res]
    asm.close()
    common = min(len(final["fd64"]), len(final["exact32"]))
    err = {"solution_error_at_wi": None, "solution_rel_err_2norm": None,
           "solution_rel_err_maxnorm": None}
    if common:
        ref = final["fd64"][common - 1]
        d = final["exact32"][common - 1] - ref
        err = {"solution_error_at_wi": wis[common - 1],
               "solution_rel_err_2norm": float(np.linalg.norm(d) / np.linalg.norm(ref)),
               "solution_rel_err_maxnorm": float(np.max(np.abs(d)) / np.max(np.abs(ref)))}
    return {
        "workload": f"Newton solves by natural continuation Wi = {', '.join(str(w) for w in wis)}, "
                    f"Giesekus alpha=0.1, beta=0.59, SQRT form, {mesh.nel} Q2 quads "
                    f"({len(rowptr) - 1} unknowns), outlet edges, Dirichlet rows on the device; "
                    f"linear solver: {_solver_desc(solver)}",
        "linear_solver": type(solver).__name__, "solver_setup_s": t_sym,
        "fd64": runs["fd64"], "fp32_jacobian": runs["exact32"], **err,
    }


def batched_compare(ninst: int, steps: int, warmup: int, device: int = 0, seed: int = 0):
    """Batched form: ninst Oldroyd-B instances (beta = 0.59, SQRT form), Wi
    uniform in [0.1, 1.0], meshes of 2,000-20,000 quads drawn log-uniformly
    (nearest block layout), seeded states; FP64 residual + FP32 Jacobian per
    step, all instances in one persistent launch per kernel replayed as a
    CUDA graph, tiles from the autotuner -- against one vefem_assemble per
    instance on the same device buffers."""
    import torch
    rng = np.random.default_rng(seed)
    sizes = np.round(np.exp(rng.uniform(np.log(2000), np.log(20000), ninst))).astype(int)
    wis = rng.uniform(0.1, 1.0, ninst)
    meshes, physs, pats, TLs, EUs = [], [], [], [], []
    d = torch.device(f"cuda:{device}")
    for k in range(ninst):
        m = M.build_cylinder_mesh(int(sizes[k]), exact=False)
        p = S.oldroyd_b(float(wis[k]), 0.59, "SQRT", nex=0)
        TL, _ = S.seeded_state(m.xyz, p, seed=k)
        meshes.append(m)
        physs.append(p)
        pats.append(V.build_pattern(m.conn, m.nnodes, 0))
        TLs.append(torch.from_numpy(TL).to(d))
        EUs.append(torch.zeros(1, dtype=torch.float64, device=d))
    bs = [torch.zeros(len(rp) - 1, dtype=torch.float64, device=d) for rp, _ in pats]
    vs = [torch.zeros(len(ci), dtype=torch.float32, device=d) for _, ci in pats]
    nel = int(sum(m.nel for m in meshes))
    flags = V.VEFEM_RESIDUAL | V.VEFEM_JAC_EXACT32 | V.VEFEM_ZERO_FIRST
    bt = V.BatchAssembler(meshes, physs, pats, device=device)
    t0 = time.perf_counter()
    tiles = bt.autotune(flags, reps=2)
    tune_s = time.perf_counter() - t0
    for _ in range(warmup):
        bt.assemble(TLs, EUs, flags, bs, vs, on_device=True)
    bt.assemble(TLs, EUs, flags | V.VEFEM_TIMING, bs, vs, on_device=True)
    tm = bt.last_timing()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        bt.assemble(TLs, EUs, flags, bs, vs, on_device=True)
    torch.cuda.synchronize()
    bat_s = time.perf_counter() - t0
    info = bt.info()
    bt.close()
    singles = [V.BulkAssembler(m, p, rp, ci, device=device) for m, p, (rp, ci) in zip(meshes, physs, pats)]
    for _ in range(warmup):
        for a, TL, b, v in zip(singles, TLs, bs, vs):
            a.assemble(TL, None, flags, b, v, on_device=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        for a, TL, b, v in zip(singles, TLs, bs, vs):
            a.assemble(TL, None, flags, b, v, on_device=True)
    torch.cuda.synchronize()
    seq_s = time.perf_counter() - t0
    for a in singles:
        a.close()
    return {
        "workload": f"{ninst} Oldroyd-B instances (beta=0.59, SQRT form, Nex=0), Wi ~ U[0.1,1.0], "
                    f"{int(sizes.min())}-{int(sizes.max())} quads drawn log-uniformly in "
                    "[2000, 20000] (nearest block layout), seeded states; FP64 residual + FP32 "
                    "exact Jacobian into AIJ",
        "elements": nel, "value": nel * steps / bat_s, "unit": UNIT,
        "ms_per_step": 1e3 * bat_s / steps,
        "sequential_value": nel * steps / seq_s, "speedup_vs_sequential": seq_s / bat_s,
        "element_kernels_ms": tm[0], "scatter_ms": tm[1], "zeroing_ms": tm[2],
        "tiles_by_size_class": tiles, "autotune_s": tune_s, "work_items": info["work_items"],
        "grid": info["grid"], "launches_per_step": info["launches"],
        "timing": "host clock around graph replays, each call synchronised",
    }


def run_only(args, asm, mesh, TL, EU, cfg, dev):
    """One assembly form alone, device-resident (the profiling case)."""
    import torch
    d = torch.device(f"cuda:{dev}")
    jflag = {"fd64": V.VEFEM_JAC_FD64, "residual": 0, "exact64": V.VEFEM_JAC_EXACT64,
             "exact32": V.VEFEM_JAC_EXACT32}[args.only]
    flags = V.VEFEM_RESIDUAL | jflag | V.VEFEM_ZERO_FIRST
    tTL = torch.from_numpy(TL).to(d)
    tEU = torch.from_numpy(EU).to(d)
    tb = torch.zeros(asm.N, dtype=torch.float64, device=d)
    tv = None
    if jflag:
        tv = torch.zeros(asm.nnz, dtype=torch.float32 if args.only == "exact32" else torch.float64,
                         device=d)
    for _ in range(args.warmup):
        asm.assemble(tTL, tEU, flags, tb, tv, on_device=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        asm.assemble(tTL, tEU, flags, tb, tv, on_device=True)
    torch.cuda.synchronize()
    s = time.perf_counter() - t0
    print(json.dumps({"only": args.only, "value": mesh.nel * args.steps / s, "unit": UNIT,
                      "steps": args.steps, "config": cfg}))
    asm.close()
    return 0


def frontal_solve_timing(nel: int, steps: int, warmup: int, device: int = 0):
    """The continuation's linear solver alone (the profiling case): the GPU
    panel-frontal LU of the bordered FD64 Jacobian of a perturbed fully
    developed Oldroyd-B state (Wi = 0.5, SQRT form, arclength row), one
    factorisation and ``steps`` solves timed with CUDA events on the
    current stream, the solve checked against the CSR matrix."""
    import torch
    from ve_flow_around_cylinder_fortran_gb300 import continuation as C
    from ve_flow_around_cylinder_fortran_gb300 import frontal as FR
    from ve_flow_around_cylinder_fortran_gb300 import newton as NW
    mesh = M.build_cylinder_mesh(nel)
    phys = S.oldroyd_b(0.5, 0.59, "SQRT", nex=1)
    rp, ci = P.build_pattern(mesh.element_nodes(), mesh.nnodes, 1)
    asm = V.BulkAssembler(mesh, phys, rp, ci, outlet_edges=True, device=device)
    rows, values = NW.boundary_conditions(mesh, phys)
    TL, EU = NW.initial_state(mesh, phys)
    TLs, _ = S.seeded_state(mesh.xyz, phys, 0)
    TL = TL + 0.01 * (TLs - TL)
    dev = NW.DeviceAssembly(asm, rows, values, "fd64", True)
    b, vals = dev(TL, EU, True)
    asm.close()
    lrow = C.LambdaRow(rp, ci)
    x = np.concatenate([TL.T.reshape(-1), EU])
    t = np.random.default_rng(0).standard_normal(len(x))
    lrow.mode, lrow.t, lrow.x_o, lrow.dS = "arclength", t / np.linalg.norm(t), x * 0.99, 0.1
    lrow(x, b, vals)
    lu = FR.FrontalLU(rp, ci, mesh)
    d = torch.device(f"cuda:{device}")
    dv = torch.from_numpy(vals).to(d)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lu.factor(dv)
    torch.cuda.synchronize()
    t_fac = time.perf_counter() - t0
    bt = torch.from_numpy(b).to(d)
    xs = lu._sweep(bt)
    rel = float(torch.linalg.vector_norm(bt - lu.A @ xs) / torch.linalg.vector_norm(bt))
    for _ in range(warmup):
        lu._sweep(bt)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    for _ in range(steps):
        xr = lu._sweep(bt)
    ev1.record()
    torch.cuda.synchronize()
    out = {"workload": f"bordered FD64 Jacobian, {mesh.nel} Q2 quads ({len(rp) - 1} unknowns), "
                       f"Oldroyd-B Wi=0.5 SQRT, perturbed fully developed state; "
                       f"{_solver_desc(lu)}",
           "factor_s": t_fac, "factor_mode": lu.mode, "min_relative_pivot": lu.min_pivot,
           "solve_ms": ev0.elapsed_time(ev1) / steps, "launches_per_solve": 2 * lu.npan + 2,
           "solve_path": {1: "programmatic dependent launch", 2: "plain stream order"}.get(
               lu.solve_path, None),
           "solve_rel_residual": rel, "reproducible": bool(torch.equal(xs, xr))}
    lu.close()
    return out


def stability_compare(nel: int, steps: int, warmup: int, device: int = 0, cpu: bool = True):
    """Linear stability (Oldroyd-B, beta = 0.59, Wi = 0.7, T form): A(k) for
    16 spanwise wavenumbers uniform in [0, 4] and B, 10 unknowns per node, on
    a seeded base state; one element launch and one scatter for all k."""
    import torch
    mesh = M.build_cylinder_mesh(nel)
    phys = S.oldroyd_b(0.7, 0.59, "T", nex=0)
    TL, _ = S.seeded_state(mesh.xyz, phys, seed=0)
    TLb = np.zeros((10, mesh.nnodes))
    TLb[0:2] = TL[0:2]
    TLb[3:7] = TL[2:6]
    rowptr, colind = V.build_pattern(mesh.conn, mesh.nnodes, 0)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind, device=device)
    rp10, ci10 = asm.stability_pattern()
    d = torch.device(f"cuda:{device}")
    kws = np.linspace(0.0, 4.0, 16)
    tA = [torch.zeros(len(ci10), dtype=torch.float64, device=d) for _ in kws]
    tB = torch.zeros(len(ci10), dtype=torch.float64, device=d)
    tTLb = torch.from_numpy(TLb).to(d)
    for _ in range(warmup):
        asm.stability_assemble(tTLb, kws, V.VEFEM_ZERO_FIRST, tA, tB, on_device=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        asm.stability_assemble(tTLb, kws, V.VEFEM_ZERO_FIRST, tA, tB, on_device=True)
    torch.cuda.synchronize()
    sec = (time.perf_counter() - t0) / steps
    out = {
        "workload": f"{mesh.nel} Q2 quads, Oldroyd-B beta=0.59 Wi=0.7, T form, seeded base state; "
                    "A(k) for 16 wavenumbers k in [0, 4] and B, 10 unknowns per node "
                    f"({len(rp10) - 1} rows, nnz {len(ci10)} per matrix)",
        "ms_per_assembly": 1e3 * sec, "element_wavenumbers_per_s": mesh.nel * len(kws) / sec,
        "unit": "element-wavenumber/s", "hbm_bytes_written": 17 * len(ci10) * 8,
    }
    asm.close()
    del tA, tB
    if cpu:
        from oracle import oracle as O
        n = min(mesh.nel, 200)
        t0 = time.perf_counter()
        O.stability_elements(phys, mesh.conn, mesh.xyz, TLb, np.zeros_like(TLb), 1.0, e0=0, e1=n,
                             nthreads=os.cpu_count() or 1)
        c = time.perf_counter() - t0
        out["cpu_oracle"] = {"value": n / c, "unit": "element-wavenumber/s",
                             "cores": os.cpu_count(), "kind": "port",
                             "sample": f"forward-difference A and B of the first {n} elements "
                                       "at one wavenumber (element blocks, no scatter)"}
    return out


def run_vefem(args):
    import torch
    world, rank, local, dist = dist_setup()
    dev = local
    torch.cuda.set_device(dev)
    B.build()
    if args.only == "frontal":
        if rank == 0:
            print(json.dumps({"only": "frontal", "frontal": frontal_solve_timing(
                args.nel, args.steps, args.warmup, dev)}))
        return 0
    if args.only == "stability":
        if rank == 0:
            print(json.dumps({"only": "stability",
                              "stability": stability_compare(args.nel, args.steps, args.warmup, dev,
                                                             cpu=False)}))
        return 0
    if args.newton_only > 0:
        if rank == 0:
            print(json.dumps({"newton_precision": newton_precision_compare(
                args.newton_only, dev, linear_solver=args.linear_solver)}))
        return 0
    if args.continuation_only:
        if rank == 0:
            out = continuation_compare(
                args.cont_nel, args.cont_wi, dev, secant=args.secant,
                ablations=args.ablations,
                only=[a for a in args.cont_arms.split(",") if a] or None,
                linear_solver=args.linear_solver, krylov=args.krylov,
                step_log=(lambda m: print(m, file=sys.stderr, flush=True)) if args.cont_log else None)
            print(json.dumps({"continuation": out}))
        if dist:
            dist.destroy_process_group()
        return 0
    mesh, phys, TL, EU, rowptr, colind, cfg = workload(args.nel)
    asm = V.BulkAssembler(mesh, phys, rowptr, colind, device=dev)
    if args.only:
        return run_only(args, asm, mesh, TL, EU, cfg, dev)
    nel = mesh.nel
    d = torch.device(f"cuda:{dev}")
    tTL = torch.from_numpy(TL).to(d)
    tEU = torch.from_numpy(EU).to(d)
    tb = torch.zeros(asm.N, dtype=torch.float64, device=d)
    tv = torch.zeros(asm.nnz, dtype=torch.float64, device=d)
    flags = V.VEFEM_RESIDUAL | V.VEFEM_JAC_FD64 | V.VEFEM_ZERO_FIRST | V.VEFEM_TIMING
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(asm.stream(), device=d)

    # ---- device-resident timed region
    for _ in range(args.warmup):
        asm.assemble(tTL, tEU, flags, tb, tv, on_device=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    k_times = []
    launches = 0
    for _ in range(args.steps):
        asm.assemble(tTL, tEU, flags, tb, tv, on_device=True)
        t = asm.last_timing()
        k_times.append(t[0])
        launches += asm.last_launch_count()
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, d)
    value = replica_rate(world, nel, args.steps, ms * 1e-3)

    # ---- residual-only ('MNR') on the same state
    rflags = V.VEFEM_RESIDUAL | V.VEFEM_ZERO_FIRST | V.VEFEM_TIMING
    for _ in range(args.warmup):
        asm.assemble(tTL, tEU, rflags, tb, None, on_device=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    r_k = []
    for _ in range(args.steps):
        asm.assemble(tTL, tEU, rflags, tb, None, on_device=True)
        r_k.append(asm.last_timing()[0])
    ev1.record(stream)
    torch.cuda.synchronize()
    r_ms = ev0.elapsed_time(ev1)

    # ---- exact-Jacobian forms on the same state: FP64, and the FP32 precision form
    #      (FP64 residual + FP32 Jacobian into a float AIJ array)
    tv32 = torch.zeros(asm.nnz, dtype=torch.float32, device=d)
    forms = {}
    for name, jflag, vbuf in (("exact64_jacobian", V.VEFEM_JAC_EXACT64, tv),
                              ("fp32_jacobian", V.VEFEM_JAC_EXACT32, tv32)):
        xflags = V.VEFEM_RESIDUAL | jflag | V.VEFEM_ZERO_FIRST | V.VEFEM_TIMING
        for _ in range(args.warmup):
            asm.assemble(tTL, tEU, xflags, tb, vbuf, on_device=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        tk = []
        for _ in range(args.steps):
            asm.assemble(tTL, tEU, xflags, tb, vbuf, on_device=True)
            tk.append(asm.last_timing())
        ev1.record(stream)
        torch.cuda.synchronize()
        xms = ev0.elapsed_time(ev1)
        forms[name] = {"value": nel * args.steps / (xms * 1e-3), "unit": UNIT,
                       "ms_per_step": xms / args.steps,
                       "element_kernels_ms": statistics.mean(x[0] for x in tk),
                       "scatter_ms": statistics.mean(x[1] + x[2] for x in tk),
                       "residual": "FP64 (bit-exact)",
                       "jacobian": "exact derivative, " + ("FP32" if "32" in name else "FP64")}
    # ---- roofline of the precision form's Jacobian kernel alone (no residual
    #      beside it): FP32 operations counted from its source / its event time,
    #      against the FFMA rate of a probe kernel (an FMA = two operations)
    jflags = V.VEFEM_JAC_EXACT32 | V.VEFEM_ZERO_FIRST | V.VEFEM_TIMING
    for _ in range(args.warmup):
        asm.assemble(tTL, tEU, jflags, None, tv32, on_device=True)
    torch.cuda.synchronize()
    jk = []
    for _ in range(args.steps):
        asm.assemble(tTL, tEU, jflags, None, tv32, on_device=True)
        jk.append(asm.last_timing()[0])
    ops32 = algorithmic_ops(phys, V.VEFEM_JAC_EXACT32)
    jk_ms = statistics.mean(jk)
    ffma = fp32_peak(dev)
    ach32 = ops32[0] * nel / (jk_ms * 1e-3)
    step32 = forms["fp32_jacobian"]["ms_per_step"]
    # algorithmic bytes of one precision-form step: state, coordinates and
    # connectivity read, residual (FP64) and AIJ values (FP32) written
    alg_bytes = (TL.nbytes + EU.nbytes + mesh.xyz[:2].nbytes + mesh.conn.nbytes
                 + asm.N * 8 + asm.nnz * 4)
    hbm = measured_hbm_gbs()
    forms["fp32_jacobian"]["roofline"] = {
        "kernel": "k_exact_batched<float>", "bound": "fp32", "achieved": ach32 / 1e12,
        "peak": 2.0 * ffma / 1e12, "unit": "TOP/s", "frac": ach32 / (2.0 * ffma),
        "traffic": None, "ops_per_element": ops32[0],
        "ops_split": {"add": ops32[1], "mul": ops32[2], "div": ops32[3], "sqrt": ops32[4]},
        "kernel_ms_avg": jk_ms,
        "peak_source": "measured live: FFMA instruction rate of a probe kernel x 2",
        "step_hbm": {"algorithmic_bytes": alg_bytes,
                     "achieved_gbs": alg_bytes / (step32 * 1e-3) / 1e9,
                     "peak_gbs": hbm, "frac": (alg_bytes / (step32 * 1e-3) / 1e9 / hbm) if hbm else None,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if hbm else None}}
    del tv32

    # ---- end to end through the C ABI with pinned host buffers
    hTL = torch.from_numpy(TL).pin_memory().numpy()
    hEU = torch.from_numpy(EU).pin_memory().numpy()
    hb = torch.zeros(asm.N, dtype=torch.float64).pin_memory().numpy()
    hv = torch.zeros(asm.nnz, dtype=torch.float64).pin_memory().numpy()
    eflags = V.VEFEM_RESIDUAL | V.VEFEM_JAC_FD64 | V.VEFEM_ZERO_FIRST
    for _ in range(args.warmup):
        asm.assemble(hTL, hEU, eflags, hb, hv, on_device=False)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        asm.assemble(hTL, hEU, eflags, hb, hv, on_device=False)
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, d)
    e2e = {"value": replica_rate(world, nel, args.steps, e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": int(hTL.nbytes + hEU.nbytes),
           "d2h_bytes_per_step": int(hb.nbytes + hv.nbytes)}

    if rank != 0:
        asm.close()
        dist.destroy_process_group()
        return 0

    # ---- roofline of the dominant kernel (FD Jacobian kernel, FP64 pipe bound)
    peaks = fp64_peak(dev)
    ops = algorithmic_ops(phys, flags)
    k_avg_ms = statistics.mean(k_times)
    achieved = ops[0] * nel / (k_avg_ms * 1e-3)
    peak = peaks["dfma_inst_per_s"]
    tpe = traffic_per_element()
    roof = {"kernel": "k_fd64<SQRT>", "bound": "fp64", "achieved": achieved / 1e12,
            "peak": peak / 1e12, "unit": "TOP/s", "frac": achieved / peak,
            "traffic": (tpe * nel if tpe else None),
            "ops_per_element": ops[0], "ops_split": {"add": ops[1], "mul": ops[2], "div": ops[3],
                                                     "sqrt": ops[4], "exp": ops[5]},
            "kernel_ms_avg": k_avg_ms, "kernel_share_of_step": k_avg_ms / (ms / args.steps),
            "peak_source": "measured live: FP64 DFMA instruction rate of a probe kernel "
                           "(one instruction = one operation; this path cannot use FMA)",
            "dadd_peak": peaks["dadd_inst_per_s"] / 1e12, "dmul_peak": peaks["dmul_inst_per_s"] / 1e12}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": cfg, "e2e": e2e, "gpu_launches": launches, "roofline": roof,
        "cpu_baseline": None, "clocks": clk,
        "residual_only": {"value": nel * args.steps / (r_ms * 1e-3), "unit": UNIT,
                          "kernel_ms_avg": statistics.mean(r_k)},
    }
    line.update(forms)
    asm.close()
    def leg(name, fn):
        # a secondary measurement that fails is reported in the line, not fatal
        try:
            line[name] = fn()
        except Exception as exc:      # noqa: BLE001
            import traceback
            traceback.print_exc()
            line[name] = {"error": f"{type(exc).__name__}: {exc}"}

    if world == 1 and args.batch_inst > 0:
        leg("batched", lambda: batched_compare(args.batch_inst, max(3, args.steps // 2),
                                               args.warmup, dev))
    if world == 1 and args.newton_nel > 0:
        leg("newton_precision", lambda: newton_precision_compare(
            args.newton_nel, dev, linear_solver=args.linear_solver))
        npr = line["newton_precision"]
        if "fp32_jacobian" in npr:
            line["fp32_jacobian"]["newton"] = {
                "workload": npr["workload"],
                "reached_wi": npr["fp32_jacobian"]["reached_wi"],
                "iterations": [x["iterations"] for x in npr["fp32_jacobian"]["solves"]],
                "factorisations": [x["factorisations"] for x in npr["fp32_jacobian"]["solves"]],
                "fp64_iterations": [x["iterations"] for x in npr["fd64"]["solves"]],
                "solution_error_at_wi": npr["solution_error_at_wi"],
                "solution_rel_err_2norm": npr["solution_rel_err_2norm"],
                "solution_rel_err_maxnorm": npr["solution_rel_err_maxnorm"]}
    if world == 1 and args.cont_nel > 0:
        leg("continuation", lambda: continuation_compare(
            args.cont_nel, args.cont_wi, dev, secant=args.secant, ablations=args.ablations,
            linear_solver=args.linear_solver, krylov=args.krylov))
    if world == 1 and args.stab_nel > 0:
        leg("stability", lambda: stability_compare(args.stab_nel, max(3, args.steps // 4),
                                                   args.warmup, dev, cpu=not args.no_cpu_baseline))
    # the CPU baseline runs last: its OpenMP worker threads stay on the host
    # cores afterwards and would slow the host side of the parts above
    if world == 1 and not args.no_cpu_baseline:
        rate, n, cores, times = cpu_oracle_rate(phys, mesh, TL, EU, rowptr, colind, 6.0, 3)
        rate1, n1, _, times1 = cpu_oracle_rate(phys, mesh, TL, EU, rowptr, colind, 3.0, 3,
                                               threads=1)
        from oracle import oracle as O
        line["cpu_baseline"] = {
            "value": rate, "unit": UNIT, "cores": cores, "kind": "port",
            "flags": O.build_flags(), "cpu_model": O.cpu_model(),
            "sample": f"first {n} of {nel} elements, residual + FD Jacobian into AIJ, "
                      f"median of 3 ({', '.join(f'{x:.2f}' for x in times)} s)",
            "one_core": {"value": rate1, "unit": UNIT,
                         "sample": f"first {n1} of {nel} elements, median of 3 "
                                   f"({', '.join(f'{x:.2f}' for x in times1)} s)"}}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    faulthandler.enable()   # a crash in native code still prints the Python stack
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_vefem(args)


if __name__ == "__main__":
    sys.exit(main())
