#!/usr/bin/env python
"""Time-steps/s of the wPFAW3D time step on GB300.

Workload: one 256^3 synthetic wormholing domain (K = exp(sigma g), log-K
variance 2, correlation length 8 cells, seeded), Darcy solve to a 1e-8
relative residual with the FP32 MG-PCG inside FP64 iterative refinement,
then the fused phase / concentration update.  A "step" is one pass of the
main-loop body (wPFAW3D.f90:2226-2280).  Inputs (all FP64 fields, ~2 GB)
are far larger than the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

With N > 1 (torchrun) every rank advances its own replica (different seed);
the path has no exchange step on one domain, so there is no collective in
the timed region -- only the barrier and the max-over-ranks timing.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "time-steps/s at 256^3, 1e-8 Darcy residual: warm-started FP32-refined vs plain FP64"
KC_NAMES = ["permeability", "resid64", "coefficients", "smooth_l0", "mg_other", "apply",
            "pcg_vec", "fused_update", "other", "bottom"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256, help="cells per axis")
    ap.add_argument("--solver", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--rtol", type=float, default=1e-8)
    ap.add_argument("--log-var", type=float, default=2.0)
    ap.add_argument("--corr", type=float, default=8.0)
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--w-from", type=int, default=3,
                    help="first multigrid level cycled twice (0 = library default, 2); 3 is the "
                         "fastest at 256^3 of 2, 3, 4 and a V-cycle (same PCG iterations as 2)")
    ap.add_argument("--breakdown", action="store_true",
                    help="time every kernel class (diagnostic run; adds event overhead)")
    ap.add_argument("--plain-w-from", type=int, default=2,
                    help="W-cycle level of the plain FP64 comparison run (2: its fewest PCG "
                         "iterations; from level 3 it takes 7 instead of 5 at 256^3)")
    ap.add_argument("--nu", type=int, default=2, help="smoothing sweeps per side of a cycle")
    ap.add_argument("--sweep-min", type=int, default=0,
                    help="cells from which a level uses the pipelined sweep (0 = library default)")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch the preconditioner cycle kernel by kernel")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain FP64 MG-PCG comparison run")
    ap.add_argument("--no-tma", action="store_true",
                    help="stage the finest-level sweep with cp.async instead of bulk-tensor copies")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the run with the learned correction of the start")
    ap.add_argument("--spinup", type=int, default=40,
                    help="untimed steps before the warm-up: the timed window starts past "
                         "the start-up transient of the run (dt jump at step 3, first front "
                         "motion), as in the 500-2000-step runs the metric stands for")
    ap.add_argument("--no-step-graph", action="store_true",
                    help="host-driven steps (a read-back per PCG iteration) instead of one "
                         "graph launch per step with the solver loops on the device")
    ap.add_argument("--warm-start", default="extrap", choices=["none", "extrap"],
                    help="start of each solve: previous pressure, or extrapolated in time")
    return ap.parse_args()


def solver_kwargs(args, solver=None):
    """Solver options of the timed arm; solver="fp64" gives the plain method
    (FP64 MG-PCG started from the previous pressure, as the reference)."""
    plain = solver == "fp64"
    return dict(solver=solver or args.solver, rtol=args.rtol,
                w_from_level=args.plain_w_from if plain else args.w_from,
                smooth_sweeps=args.nu, sweep_min_cells=args.sweep_min,
                graphs=not args.no_graphs, tma=not args.no_tma,
                step_graph=not args.no_step_graph,
                extrapolate=(not plain) and args.warm_start == "extrap")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(ms: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's time: every rank's replica finishes within it."""
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(world: int, steps: int, ms: float) -> float:
    """Whole-job time-steps/s: every rank advances its own replica `steps`
    steps in the (max-over-ranks) time `ms` (weak scaling, replicas only)."""
    return world * steps / (ms / 1000.0)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-i", str(self.gpu), "-lms", "200"], stdout=open(self.path, "w"),
                stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return d["hbm_gbs"], "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def sweep_traffic_per_cell():
    """DRAM bytes per cell per launch of the finest-level sweep, averaged over
    a cycle, as measured by ncu (profiles/k_sweep_async_224.md)."""
    try:
        with open(os.path.join(HERE, "profiles", "k_sweep_async_224.md")) as fh:
            for line in fh:
                if line.startswith("traffic_bytes_per_cell_avg"):
                    return float(line.split("=")[1])
    except (OSError, ValueError):
        pass
    return None


def make_workload(args, rank):
    from mizuho_edit_gb300.cases import make_case
    n = args.n
    return make_case((n, n, n), log_var=args.log_var, corr_len=args.corr, seed=args.seed + rank)


def config_of(args, world):
    n = args.n
    return {"workload": f"wPFAW3D step, {n}^3 cells, synthetic GRF log-K var {args.log_var} "
                        f"corr {args.corr}, Pe 100, Da 10, Dirichlet p 1->0",
            "grid": [n, n, n], "solver": "fp32-mg-pcg-in-fp64-refinement" if args.solver == "mixed"
            else "fp64-mg-pcg", "darcy_rtol": args.rtol, "dtype_state": "f64",
            "warm_start": ("time-extrapolated pressure with fallback to the previous pressure"
                           if args.warm_start == "extrap" and args.solver == "mixed"
                           else "previous pressure"),
            "compared_with": f"plain FP64 MG-PCG from the previous pressure (plain_fp64; W-cycle "
                             f"from level {args.plain_w_from})",
            "timed_steps": f"{args.spinup + args.warmup + 1}..{args.spinup + args.warmup + args.steps}"
                           f" of the run (spin-up {args.spinup} + warm-up {args.warmup} untimed)",
            "multigrid": {"w_cycle_from_level": args.w_from, "sweeps_per_side": args.nu,
                          "pipelined_sweep_min_cells": args.sweep_min or (1 << 23)},
            "step": "one CUDA graph launch per step" if not args.no_step_graph else "host-driven",
            "l2_policy": "inputs larger than L2 (~2 GB of fields per step)",
            "parallelism": f"replicas{world}" if world > 1 else "single-domain"}


def cpu_sample(sim, args):
    """One reference time step (BiCGStab + SOR(10, 1.7), rtol 1e-10, the
    reference's PETSc settings) on the host cores from the GPU run's state."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    p = sim.params
    f = sim.download("phase", "concent", "pressure")
    ref = O.OracleSim(p, sim._kr_cache, f["phase"][1:-1, 1:-1, 1:-1],
                      f["concent"][1:-1, 1:-1, 1:-1])
    ref.pressure[...] = f["pressure"]
    ref.itime, ref.dtime, ref.taumin = sim.itime, sim.dtime, sim.taumin
    t0 = time.perf_counter()
    info = ref.step(O.SOLVE_BCGS_SOR, 1e-10, 1000, threads)
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": "time-steps/s", "cores": threads, "kind": "port",
            "sample": f"1 reference time step at {p.nx}^3 from the benchmark's warm state "
                      f"(BiCGStab+SOR(10,1.7) rtol 1e-10, {info.iterations} its, "
                      f"{threads} OpenMP threads as {threads} SOR blocks), {dt:.1f} s"}


def run_ours(args):
    import torch
    from mizuho_edit_gb300 import capi
    from mizuho_edit_gb300.sim import Simulation
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    case = make_workload(args, rank)
    sim = Simulation(case.params, case.permeab_rock, case.phase, case.concent,
                     **solver_kwargs(args))
    L = sim.L
    KC_SMOOTH0 = 3
    NK = len(KC_NAMES)
    # Kernel-class timers bracket every launch with events, and a step with
    # timers on is host-driven (the device-resident step graph is off while
    # they are): the timed steps run without them, except in a --breakdown run;
    # the per-launch time of the roofline kernel comes from a second window of
    # the same length right after, with its class timed.  The timing mask is
    # part of the captured preconditioner graphs: it is set before the warm-up
    # so that the capture happens there.
    mask = (1 << NK) - 1 if args.breakdown else 0
    capi.check(L.wpf_set_kernel_timing(sim.h, mask), "timing")
    for _ in range(args.spinup + args.warmup):
        sim.step()
    sp = C.c_void_p()
    capi.check(L.wpf_get_stream(sim.h, C.byref(sp)), "wpf_get_stream")
    stream = torch.cuda.ExternalStream(sp.value)
    capi.check(L.wpf_set_kernel_timing(sim.h, mask), "timing")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    n0 = C.c_int64()
    L.wpf_launch_count(sim.h, C.byref(n0))
    e0.record(stream)
    stats = [sim.step() for _ in range(args.steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    n1 = C.c_int64()
    L.wpf_launch_count(sim.h, C.byref(n1))
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    kms = (C.c_double * NK)()
    kcnt = (C.c_int64 * NK)()
    if not args.breakdown:   # the roofline window: the finest-level smoother timed
        capi.check(L.wpf_set_kernel_timing(sim.h, 1 << KC_SMOOTH0), "timing")
        sim.step()   # recaptures the cycle graphs with the timer nodes
        capi.check(L.wpf_set_kernel_timing(sim.h, 1 << KC_SMOOTH0), "timing")
        for _ in range(args.steps):
            sim.step()
    L.wpf_kernel_times(sim.h, kms, kcnt, NK)
    capi.check(L.wpf_set_kernel_timing(sim.h, 0), "timing")
    ms_max = max_over_ranks(ms, world)
    n = args.n
    ncell = n ** 3
    value = job_rate(world, args.steps, ms_max)

    # roofline of the finest-level red-black Gauss-Seidel smoother (the
    # largest share of the step in the launch list).  A finest level of at
    # least 2^23 cells runs the one-pass pipelined sweep, whose algorithmic
    # bytes per cell (FP32) are: couplings cx,cy,cz (12 B) + 1/diag (4 B) +
    # b (4 B) + the input x (4 B) + the output x (4 B) = 28 B; the zero-guess
    # first sweep of a cycle reads no input x (24 B); the coarse correction is
    # a separate prolongation pass before the post-sweeps.  Four sweeps per cycle
    # (nu = 2 on each side).  Smaller finest levels run two half-sweep
    # kernels: 20 B/cell each (12 B couplings + 2 B other colour + 6 B b,
    # 1/diag, new x of this colour), 12 B for the zero-guess one.
    nu = 2
    cnt = int(kcnt[KC_SMOOTH0])
    smooth_ms = float(kms[KC_SMOOTH0])
    if ncell >= (1 << 23):
        cycles = cnt // (2 * nu)
        smooth_bytes = (cycles * 24.0 + (cnt - cycles) * 28.0) * ncell
        kname, per_cell = "k_sweep_async<float> (finest level)", 28
    else:
        n_first = cnt // (4 * nu)
        smooth_bytes = (n_first * 12.0 + (cnt - n_first) * 20.0) * ncell
        kname, per_cell = "k_rbgs<float> (finest level)", 20
    peak, peak_kind = measured_peaks()
    achieved = smooth_bytes / (smooth_ms / 1000.0) / 1e9 if smooth_ms > 0 else None
    traffic = None   # DRAM bytes per launch, from the ncu capture summarised in profiles/
    if ncell >= (1 << 23):
        tpc = sweep_traffic_per_cell()
        traffic = tpc * ncell if tpc else None
    roof = {"kernel": kname, "bound": "hbm",
            "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "traffic": traffic,
            "traffic_source": "profiles/k_sweep_async_224.md (ncu, 224^3, scaled by cells)",
            "peak_source": peak_kind, "bytes_per_cell_per_launch": per_cell,
            "launches": cnt, "avg_launch_us": smooth_ms * 1000.0 / max(cnt, 1)}

    upd_ms = statistics.mean(s.update_ms for s in stats)
    out = {
        "metric": METRIC, "value": value, "unit": "time-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Gaussian random field permeability; no data set)",
        "config": config_of(args, world),
        "cell_updates_per_s": value * ncell,
        "darcy_solve_ms": statistics.mean(s.solve_ms for s in stats),
        "pcg_iterations_per_step": statistics.mean(s.inner_iterations for s in stats),
        "outer_passes_per_step": statistics.mean(s.outer_iterations for s in stats),
        "relres_max": max(s.relres for s in stats),
        "fused_update_ms": upd_ms,
        # (quiescent bricks move no bytes: a cell rate, not an algorithmic GB/s)
        "fused_update_cell_updates_per_s": ncell / (upd_ms / 1000.0) if upd_ms > 0 else None,
        "gpu_launches": int(n1.value - n0.value),
        "launches_before_timed": int(n0.value),   # skip count for a launch list of the timed steps
        "roofline": roof,
        "clocks": clk,
        "kernel_class_ms": ({KC_NAMES[c]: float(kms[c]) / args.steps for c in range(NK)}
                            if args.breakdown else {KC_NAMES[3]: smooth_ms / args.steps}),
        "kernel_class_launches": ({KC_NAMES[c]: int(kcnt[c]) // args.steps for c in range(NK)}
                                  if args.breakdown else None),
        "relres0_mean": statistics.mean(s.relres0 for s in stats),
        "warm_start_used": sum(1 for s in stats if s.warm_start == 1),
        "warm_start_fallbacks": sum(1 for s in stats if s.warm_start == -1),
    }
    if args.solver == "mixed" and not args.no_plain:
        out["plain_fp64"] = plain_fp64_pass(args, case, world)
        out["speedup_vs_plain_fp64"] = value / out["plain_fp64"]["value"]
    if args.solver == "mixed" and not args.no_learned:
        out["learned"] = learned_pass(args, case, world)
    if not args.no_e2e:
        out["e2e"] = e2e_pass(args, sim, stream, world)
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            out["cpu_baseline"] = cpu_sample(sim, args)
        except Exception as e:  # the baseline must not sink the GPU line
            out["cpu_baseline"] = {"value": None, "error": str(e)[:200]}
    sim.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)


def learned_pass(args, case, world):
    """The same run with the learned correction on top of the extrapolated
    start (weights trained on 128^3 runs, mizuho_edit_gb300/weights), timed
    the same way; reports what it changes against the headline run."""
    import torch
    from mizuho_edit_gb300 import capi, learned
    from mizuho_edit_gb300.sim import Simulation
    path = learned.DEFAULT_WEIGHTS
    if not os.path.exists(path):
        return {"unavailable": "no trained weights at mizuho_edit_gb300/weights"}
    n = args.n
    net = learned.WarmStartNet(n // 2, n // 2, n // 2)
    net.set_params(learned.WarmStartNet.load_params(path))
    kw = solver_kwargs(args)
    kw["extrapolate"] = True
    with Simulation(case.params, case.permeab_rock, case.phase, case.concent, **kw) as sim:
        learned.attach(sim, net)
        for _ in range(args.spinup + args.warmup):
            sim.step()
        sp = C.c_void_p()
        capi.check(sim.L.wpf_get_stream(sim.h, C.byref(sp)), "wpf_get_stream")
        stream = torch.cuda.ExternalStream(sp.value)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        stats = [sim.step() for _ in range(args.steps)]
        e1.record(stream)
        torch.cuda.synchronize()
        ms = max_over_ranks(e0.elapsed_time(e1), world)
        learned.attach(sim, None)
    net.close()
    return {"value": job_rate(world, args.steps, ms), "unit": "time-steps/s",
            "ms_per_step": ms / args.steps,
            "darcy_solve_ms": statistics.mean(s.solve_ms for s in stats),
            "pcg_iterations_per_step": statistics.mean(s.inner_iterations for s in stats),
            "relres0_mean": statistics.mean(s.relres0 for s in stats),
            "net_start_kept": sum(1 for s in stats if s.warm_start == 2),
            "extrapolation_only": sum(1 for s in stats if s.warm_start == 1),
            "fallbacks_to_previous_pressure": sum(1 for s in stats if s.warm_start == -1),
            "relres_max": max(s.relres for s in stats)}


def plain_fp64_pass(args, case, world):
    """The plain method on the same input: FP64 MG-PCG to the same 1e-8
    residual, same warm-up and step count, timed the same way."""
    import torch
    from mizuho_edit_gb300 import capi
    from mizuho_edit_gb300.sim import Simulation
    with Simulation(case.params, case.permeab_rock, case.phase, case.concent,
                    **solver_kwargs(args, "fp64")) as sim:
        for _ in range(args.spinup + args.warmup):
            sim.step()
        sp = C.c_void_p()
        capi.check(sim.L.wpf_get_stream(sim.h, C.byref(sp)), "wpf_get_stream")
        stream = torch.cuda.ExternalStream(sp.value)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        stats = [sim.step() for _ in range(args.steps)]
        e1.record(stream)
        torch.cuda.synchronize()
        ms = max_over_ranks(e0.elapsed_time(e1), world)
    return {"value": job_rate(world, args.steps, ms), "unit": "time-steps/s",
            "ms_per_step": ms / args.steps,
            "darcy_solve_ms": statistics.mean(s.solve_ms for s in stats),
            "pcg_iterations_per_step": statistics.mean(s.inner_iterations for s in stats),
            "relres_max": max(s.relres for s in stats)}


def e2e_pass(args, sim, stream, world):
    """Same metric through the C ABI with host-owned fields: every step uploads
    the state the time loop changes -- phase, concent, pressure -- from pinned
    host buffers, runs wpf_step and downloads the same three (the reference
    keeps its module arrays on the host).  permeab_rock, which the reference
    reads once at load time and never changes (wPFAW3D.f90:494), is uploaded
    once before the timed steps."""
    import torch
    from mizuho_edit_gb300 import capi
    L = sim.L
    sh = sim.halo_shape
    G = sh[0] * sh[1] * sh[2]
    bufs = {}
    for name in ("permeab_rock", "phase", "concent", "pressure"):
        ptr = C.c_void_p()
        capi.check(L.wpf_host_alloc(G * 8, C.byref(ptr)), "wpf_host_alloc")
        arr = np.ctypeslib.as_array((C.c_double * G).from_address(ptr.value))
        bufs[name] = (ptr, arr.reshape(sh, order="F"))
    f = sim.download("phase", "concent", "pressure")
    for k in ("phase", "concent", "pressure"):
        bufs[k][1][...] = f[k]
    kr = np.zeros(sh, order="F")
    kr[1:-1, 1:-1, 1:-1] = sim._kr_cache
    bufs["permeab_rock"][1][...] = kr
    dp = {k: v[1].ctypes.data_as(capi.DP) for k, v in bufs.items()}
    capi.check(L.wpf_upload(sim.h, dp["permeab_rock"], None, None, None), "wpf_upload")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    st = capi.StepStats()
    for _ in range(args.steps):
        capi.check(L.wpf_upload(sim.h, None, dp["phase"], dp["concent"], dp["pressure"]),
                   "wpf_upload")
        sim.itime += 1
        dt = C.c_double(sim.dtime)
        capi.check(L.wpf_step(sim.h, sim.itime, C.byref(dt), C.byref(st)), "wpf_step")
        sim.dtime = dt.value
        capi.check(L.wpf_download(sim.h, dp["phase"], dp["concent"], dp["pressure"], None, None,
                                  None, None), "wpf_download")
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ms = max_over_ranks(ms, world)
    for ptr, _ in bufs.values():
        L.wpf_host_free(ptr)
    return {"value": job_rate(world, args.steps, ms), "unit": "time-steps/s",
            "h2d_bytes_per_step": 3 * G * 8, "d2h_bytes_per_step": 3 * G * 8,
            "path": "wpf_upload + wpf_step + wpf_download per step, pinned host buffers"}


def run_reference(args):
    """The reference's own CPU algorithm for this path: the reference
    (Fortran + Intel MPI + PETSc 3.22) does not build here, so its C
    restatement (oracle/) runs in reference-mirroring mode -- BiCGStab +
    SOR(10, 1.7) at rtol 1e-10, warm-started, OpenMP threads as SOR blocks."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    case = make_workload(args, 0)
    s = O.OracleSim(case.params, case.permeab_rock, case.phase, case.concent)
    budget_w, budget_t = 60.0, 100.0   # seconds: the whole arm ends in about four minutes
    t0 = time.perf_counter()
    wdone = 0
    for _ in range(max(args.warmup, 1)):
        s.step(O.SOLVE_BCGS_SOR, 1e-10, 1000, threads)
        wdone += 1
        if time.perf_counter() - t0 > budget_w:
            break
    times = []
    for _ in range(args.steps):
        t1 = time.perf_counter()
        s.step(O.SOLVE_BCGS_SOR, 1e-10, 1000, threads)
        times.append(time.perf_counter() - t1)
        if sum(times) > budget_t:
            break
    tot = sum(times)
    v = len(times) / tot
    n = args.n
    sample = (f"{len(times)} of {args.steps} requested reference time steps at {n}^3 after "
              f"{wdone} warm-up steps (BiCGStab+SOR(10,1.7), rtol 1e-10, {threads} OpenMP "
              f"threads as SOR blocks), {tot:.1f} s")
    out = {"metric": METRIC, "value": v, "unit": "time-steps/s", "n_gpus": world,
           "steps": len(times), "warmup": wdone, "ms_per_step": 1000.0 * tot / len(times),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded Gaussian random field permeability; no data set)",
           "config": config_of(args, world), "impl": "reference",
           "cell_updates_per_s": v * n ** 3,
           "cpu_baseline": {"value": v, "unit": "time-steps/s", "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": v, "unit": "time-steps/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
