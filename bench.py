#!/usr/bin/env python
"""Time-steps/s of the wPFAW3D time step on GB300.

Workload: one 256^3 synthetic wormholing domain (K = exp(sigma g), log-K
variance 2, correlation length 8 cells, seeded; dissolved-rock permeability
kwh = 1e3 x the geometric-mean rock K), Darcy solve to a 1e-8 relative
residual.  A "step" is one pass of the main-loop body (wPFAW3D.f90:2226-2280).

One run is advanced with the FP32-refined, extrapolated form; at each window
(by default after 40 and after 2000 steps) every arm is timed on the run's
state: the learned start (the headline, `value`), the extrapolated start
without the network, and the plain FP64 MG-PCG from the previous pressure.
The headline is the last window, where the acid has reached almost every
cell and the fused update works on the whole grid.  A second run at kwh = 20
is reported beside it.  Inputs (the FP64 fields a step reads are over 1 GB
at 256^3; 5.8 GB of fields and solver levels in all) are far larger than the
129 MB L2, so no flush is needed between steps.

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

METRIC = "time-steps/s at 256^3, 1e-8 Darcy residual: learned+FP32-refined vs plain FP64"
KC_NAMES = ["permeability", "resid64", "coefficients", "smooth_l0", "mg_other", "apply",
            "pcg_vec", "fused_update", "other", "bottom"]
# the timed forms ("arms") of the Darcy solve, all on the same run's state
ARMS = ("learned", "extrapolated", "plain_fp64")
# Untimed steps before each arm's W warm-up steps: a step graph bakes in its
# buffers, the step's ping-pong buffers cycle with period 6 and the first
# steps after a solver switch or an upload run with transient state, so the
# first ~8 steps of an arm capture graphs (tens of ms each at 512^3) that the
# rest of a long run replays.
GRAPH_WARMUP = 8


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256, help="cells per axis")
    ap.add_argument("--rtol", type=float, default=1e-8)
    ap.add_argument("--log-var", type=float, default=2.0)
    ap.add_argument("--corr", type=float, default=8.0)
    ap.add_argument("--kwh", type=float, default=1000.0,
                    help="permeability of dissolved rock (1e3 x the geometric-mean rock K)")
    ap.add_argument("--kwh-alt", type=float, default=20.0,
                    help="a second run at this kwh, reported beside the headline (0: none)")
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--windows", default="40,2000",
                    help="steps run before each timed window; the headline is the last window")
    ap.add_argument("--headline", default="learned", choices=["learned", "extrapolated"],
                    help="the FP32-refined form whose time-steps/s is `value`")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 arm")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned arm (the headline becomes the extrapolated form)")
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--w-from", type=int, default=3,
                    help="first multigrid level cycled twice in the FP32-refined forms (3: the "
                         "fastest at 256^3 of 2, 3, 4 and a V-cycle)")
    ap.add_argument("--plain-w-from", type=int, default=2,
                    help="W-cycle level of the plain FP64 arm (2: its fewest PCG iterations)")
    ap.add_argument("--breakdown", action="store_true",
                    help="time every kernel class in an extra host-driven window (diagnostic)")
    ap.add_argument("--nu", type=int, default=2, help="smoothing sweeps per side of a cycle")
    ap.add_argument("--sweep-min", type=int, default=0,
                    help="cells from which a level uses the pipelined sweep (0 = library default)")
    ap.add_argument("--sweep-zchunk", type=int, default=0,
                    help="z planes per block of the pipelined sweep (0 = the wave-filling chunk)")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch the preconditioner cycle kernel by kernel")
    ap.add_argument("--no-tma", action="store_true",
                    help="stage the finest-level sweep with cp.async instead of bulk-tensor copies")
    ap.add_argument("--no-step-graph", action="store_true",
                    help="host-driven steps instead of one graph launch per step")
    ap.add_argument("--no-ensemble", action="store_true",
                    help="skip the ensemble line (48 members: 16 each at 64^3, 96^3, 128^3)")
    ap.add_argument("--ensemble-steps", type=int, default=20)
    return ap.parse_args()


def arm_kwargs(args, arm):
    """Solver options of an arm.  plain_fp64: the plain method, FP64 MG-PCG
    from the previous pressure (the reference's start, wPFAW3D.f90:980);
    extrapolated: FP32 MG-PCG inside FP64 refinement from the pressure
    extrapolated in time; learned: the same plus the network's correction of
    the extrapolation.  All finish at the same FP64 relative residual."""
    plain = arm == "plain_fp64"
    return dict(mode="fp64" if plain else "mixed", rtol=args.rtol,
                w_from_level=args.plain_w_from if plain else args.w_from,
                smooth_sweeps=args.nu, sweep_min_cells=args.sweep_min, sweep_zchunk=args.sweep_zchunk,
                graphs=not args.no_graphs, tma=not args.no_tma,
                step_graph=not args.no_step_graph, extrapolate=not plain)


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


def make_workload(args, rank, kwh=None):
    from mizuho_edit_gb300.cases import make_case
    n = args.n
    return make_case((n, n, n), log_var=args.log_var, corr_len=args.corr, seed=args.seed + rank,
                     kwh=args.kwh if kwh is None else kwh)


def windows_of(args):
    return [int(w) for w in args.windows.split(",") if w.strip()]


def headline_arm(args):
    return "extrapolated" if args.no_learned else args.headline


def workload_name(args, kwh=None):
    n = args.n
    return (f"wPFAW3D step, {n}^3 cells, synthetic GRF log-K var {args.log_var} corr {args.corr}, "
            f"kwh {args.kwh if kwh is None else kwh}, Pe 100, Da 10, Dirichlet p 1->0")


def config_of(args, world):
    n = args.n
    w = windows_of(args)
    arm = headline_arm(args)
    ext = ("previous pressure plus the least-squares combination of the last two increments "
           "(the quadratic-in-time extrapolation where the previous pressure is above 100 rtol)")
    start = {"learned": ext + " plus the learned network's correction where its gate opens "
                        "(fallback to the previous pressure when the start does not lower the FP64 residual)",
             "extrapolated": ext + " (fallback to the previous pressure)"}[arm]
    return {"workload": workload_name(args), "grid": [n, n, n],
            "solver": "fp32-mg-pcg-in-fp64-refinement", "darcy_rtol": args.rtol, "dtype_state": "f64",
            "warm_start": start, "form": arm,
            "compared_with": f"plain FP64 MG-PCG from the previous pressure on the same state "
                             f"(plain_fp64; W-cycle from level {args.plain_w_from})",
            "timed_steps": f"{w[-1] + GRAPH_WARMUP + args.warmup + 1}.."
                           f"{w[-1] + GRAPH_WARMUP + args.warmup + args.steps} of the run (spin-up "
                           f"{w[-1]} steps, then per arm {GRAPH_WARMUP} steps that capture its step "
                           f"graphs and {args.warmup} warm-up steps, untimed); every arm is timed on "
                           f"these steps from the same saved state",
            "spinup_form": "extrapolated FP32-refined start, one graph launch per step",
            "multigrid": {"w_cycle_from_level": args.w_from, "sweeps_per_side": args.nu,
                          "pipelined_sweep_min_cells": args.sweep_min or (1 << 23)},
            "step": "one CUDA graph launch per step" if not args.no_step_graph else "host-driven",
            "learned_correction": "evaluated in the step graph (an IF node) when the extrapolated "
                                  "start misses the 1e-8 tolerance by at most 1.02x (the net's measured reach)",
            "l2_policy": "inputs larger than L2 (over 1 GB of FP64 fields read per step at 256^3; "
                         "5.8 GB of fields and solver levels in all)",
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


class Arms:
    """One simulation whose Darcy-solve form can be switched between the
    arms; every arm is timed on the same state of the same run."""

    def __init__(self, args, case, want_net):
        from mizuho_edit_gb300.sim import Simulation
        self.args = args
        kw = arm_kwargs(args, "extrapolated")
        self.sim = Simulation(case.params, case.permeab_rock, case.phase, case.concent,
                              solver=kw.pop("mode"), **kw)
        self.net = None
        self.arm = "extrapolated"
        if want_net:
            from mizuho_edit_gb300 import learned
            if os.path.exists(learned.DEFAULT_WEIGHTS):
                n = args.n
                self.net = learned.WarmStartNet(n // 2, n // 2, n // 2)
                self.net.set_params(learned.WarmStartNet.load_params(learned.DEFAULT_WEIGHTS))

    def set(self, arm):
        from mizuho_edit_gb300 import learned
        if arm == self.arm:
            return
        self.sim.set_solver(**arm_kwargs(self.args, arm))
        learned.attach(self.sim, self.net if arm == "learned" else None)
        self.arm = arm

    def stream(self):
        import torch
        from mizuho_edit_gb300 import capi
        sp = C.c_void_p()
        capi.check(self.sim.L.wpf_get_stream(self.sim.h, C.byref(sp)), "wpf_get_stream")
        return torch.cuda.ExternalStream(sp.value)

    def advance_to(self, step):
        self.set("extrapolated")
        while self.sim.itime < step:
            self.sim.step()

    def snapshot(self):
        """The run's state at a window: fields, step number, dt, time, taumin."""
        sim = self.sim
        f = sim.download("phase", "concent", "pressure")
        return (f, sim.itime, sim.dtime, sim.time, sim.taumin)

    def restore(self, snap):
        """Back to a snapshot, so that every arm is timed on the same steps of
        the same state (the increment history of the extrapolation is rebuilt
        by the warm-up steps)."""
        from mizuho_edit_gb300 import capi
        f, itime, dtime, tm, taumin = snap
        sim = self.sim
        sim.upload(None, f["phase"], f["concent"], f["pressure"])
        sim.itime, sim.dtime, sim.time, sim.taumin = itime, dtime, tm, taumin
        capi.check(sim.L.wpf_set_taumin(sim.h, taumin), "wpf_set_taumin")

    def time(self, arm, world, clocks=None):
        """GRAPH_WARMUP steps that capture the arm's step graphs, W warm-up
        steps, then exactly K timed steps between a barrier + synchronize and
        a synchronize, CUDA events on the library's stream; max over ranks.
        clocks: a running ClockSampler, stopped after the timed steps."""
        import torch
        args, sim = self.args, self.sim
        self.set(arm)
        for _ in range(GRAPH_WARMUP + args.warmup):
            sim.step()
        stream = self.stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0, n1 = C.c_int64(), C.c_int64()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        if clocks:   # the headline region: a profiler run with --profile-from-start off sees it alone
            torch.cuda.profiler.start()
        sim.L.wpf_launch_count(sim.h, C.byref(n0))
        first = sim.itime + 1
        e0.record(stream)
        stats = [sim.step() for _ in range(args.steps)]
        e1.record(stream)
        torch.cuda.synchronize()
        if clocks:
            torch.cuda.profiler.stop()
        sim.L.wpf_launch_count(sim.h, C.byref(n1))
        clk = clocks.stop() if clocks else None
        ms = max_over_ranks(e0.elapsed_time(e1), world)
        ncell = args.n ** 3
        out = {"value": job_rate(world, args.steps, ms), "unit": "time-steps/s",
               "window": [first, first + args.steps - 1], "ms_per_step": ms / args.steps,
               "darcy_solve_ms": statistics.mean(s.solve_ms for s in stats),
               "pcg_iterations_per_step": statistics.mean(s.inner_iterations for s in stats),
               "outer_passes_per_step": statistics.mean(s.outer_iterations for s in stats),
               "relres0_mean": statistics.mean(s.relres0 for s in stats),
               "relres_max": max(s.relres for s in stats),
               "fused_update_ms": statistics.mean(s.update_ms for s in stats),
               "update_active_fraction": statistics.mean(s.active_cells for s in stats) / ncell,
               "update_interface_fraction": statistics.mean(s.interface_cells for s in stats) / ncell,
               "max_courant": max(s.max_courant for s in stats),
               "gpu_launches": int(n1.value - n0.value)}
        if arm != "plain_fp64":
            codes = [s.warm_start for s in stats]
            out["starts"] = {"net": codes.count(2), "extrapolation": codes.count(1),
                             "previous_pressure": codes.count(-1)}
        if clk is not None:
            out["clocks"] = clk
        return out

    def close(self):
        from mizuho_edit_gb300 import learned
        if self.sim is not None:
            learned.attach(self.sim, None)
            self.sim.close()
            self.sim = None
        if self.net is not None:
            self.net.close()
            self.net = None


def device_memory(arms):
    """The library's device allocations for this domain (wpf_device_bytes:
    fields, solver hierarchies of both precisions, the net's buffers) and the
    device memory in use in the process now, against the HBM size."""
    import torch
    from mizuho_edit_gb300 import capi
    nb = C.c_int64()
    capi.check(arms.sim.L.wpf_device_bytes(arms.sim.h, C.byref(nb)), "wpf_device_bytes")
    free, total = torch.cuda.mem_get_info()
    return {"library_bytes": int(nb.value), "in_use_bytes": int(total - free), "hbm_bytes": int(total)}


def update_roofline(head_line, ncell):
    """The fused update (classification + listed cells), the largest share of
    a late-window step once the least-squares start has taken the PCG out of
    most steps.  Algorithmic bytes per step: the classification reads phase
    and concentration of every cell (16 B) and writes both for the copied
    cells (16 B); a listed cell also reads pressure (8 B), the three face
    factors Tv (24 B), its flags (1 B) and its work-list index (4 B) and
    writes both fields (16 B).  Timed per step by the step's own events."""
    peak, peak_kind = measured_peaks()
    listed = head_line["update_active_fraction"] * ncell
    nbytes = 16.0 * ncell + 16.0 * (ncell - listed) + 53.0 * listed
    ms = head_line["fused_update_ms"]
    achieved = nbytes / (ms / 1000.0) / 1e9 if ms > 0 else None
    return {"kernel": "fused update (k_update_split + k_update_active over its two lists)", "bound": "hbm",
            "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None, "bytes_per_step": nbytes,
            "ms_per_step": ms, "peak_source": peak_kind,
            "note": "latency- and FP64-pipe-bound, not HBM-bound (ncu at a late 160^3 state: "
                    "DRAM 10 % and 23 % of peak, FP64 pipe 64 % in both lists, "
                    "profiles/k_update_active_160_late.md)"}


def fp64_peak(arms):
    """The device's FP64 FMA throughput (wpf_measure_fp64_rate): the ceiling of
    the kernels bound by the FP64 pipe, which the measured copy and BF16 GEMM
    peaks do not give."""
    from mizuho_edit_gb300 import capi
    t = C.c_double()
    rc = arms.sim.L.wpf_measure_fp64_rate(C.byref(t))
    return {"tflops": t.value if rc == capi.WPF_OK else None, "unit": "TFLOP/s",
            "source": "wpf_measure_fp64_rate: 8 independent FP64 FMA chains per thread, 2048 threads per SM"}


def roofline_window(args, arms):
    """The finest-level red-black sweep timed per launch (the step's largest
    HBM-bound share): its kernel class is timed with events around every
    launch, which makes the steps host-driven, so this is a separate window
    right after the timed ones (extrapolated arm)."""
    from mizuho_edit_gb300 import capi
    sim = arms.sim
    L = sim.L
    KC_SMOOTH0 = 3
    NK = len(KC_NAMES)
    arms.set("extrapolated")
    mask = (1 << NK) - 1 if args.breakdown else (1 << KC_SMOOTH0)
    capi.check(L.wpf_set_kernel_timing(sim.h, mask), "timing")
    sim.step()   # recaptures the cycle graphs with the timer nodes
    capi.check(L.wpf_set_kernel_timing(sim.h, mask), "timing")
    for _ in range(args.steps):
        sim.step()
    kms = (C.c_double * NK)()
    kcnt = (C.c_int64 * NK)()
    L.wpf_kernel_times(sim.h, kms, kcnt, NK)
    capi.check(L.wpf_set_kernel_timing(sim.h, 0), "timing")
    ncell = args.n ** 3
    # algorithmic bytes per cell of the finest-level sweep (FP32): on levels of
    # at least 2^23 cells the one-pass pipelined sweep reads the couplings
    # cx, cy, cz (12 B), 1/diag (4 B), b (4 B) and the input x (4 B) and
    # writes the output x (4 B): 28 B; the zero-guess first sweep of a cycle
    # reads no x: 24 B; nu = 2 sweeps per side, four per cycle.  Smaller finest
    # levels run two half-sweep kernels: 20 B per cell each, 12 B zero-guess.
    nu = args.nu
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
    roof = {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "traffic": traffic,
            "traffic_source": "profiles/k_sweep_async_224.md (ncu, 224^3, scaled by cells)",
            "peak_source": peak_kind, "bytes_per_cell_per_launch": per_cell,
            "launches": cnt, "avg_launch_us": smooth_ms * 1000.0 / max(cnt, 1)}
    breakdown = None
    if args.breakdown:
        breakdown = {KC_NAMES[c]: {"ms_per_step": float(kms[c]) / args.steps,
                                   "launches_per_step": int(kcnt[c]) / args.steps} for c in range(NK)}
        # the stencil classes whose algorithmic bytes per launch are fixed: the
        # finest-level sweep (above) and k_apply_p (z, p_old, cx, cy, cz, diag
        # read, p and q written: 32 B per cell in FP32)
        apply_ms = float(kms[5])
        if apply_ms > 0:
            breakdown["apply"]["achieved_gbs"] = 32.0 * ncell * int(kcnt[5]) / (apply_ms / 1000.0) / 1e9
        if achieved:
            breakdown["smooth_l0"]["achieved_gbs"] = achieved
    return roof, breakdown


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    head = headline_arm(args)
    arms_list = [a for a in ARMS if not (a == "learned" and args.no_learned)
                 and not (a == "plain_fp64" and args.no_plain)]
    # the headline arm is timed last in the last window, under the clock sampler
    arms_list.sort(key=lambda a: a == head)
    wins = windows_of(args)
    case = make_workload(args, rank)
    arms = Arms(args, case, want_net="learned" in arms_list)
    if arms.net is None and "learned" in arms_list:
        arms_list.remove("learned")
        head = "extrapolated"
    windows = []
    head_line = None
    for wi, w in enumerate(wins):
        arms.advance_to(w)
        snap = arms.snapshot()
        row = {}
        clocks = None
        if wi == len(wins) - 1:   # sampled over the last window's arms, the headline last
            clocks = ClockSampler(dev)
            clocks.start()
        for arm in arms_list:
            last = wi == len(wins) - 1 and arm == head
            arms.restore(snap)
            r = arms.time(arm, world, clocks if last else None)
            row[arm] = r
            if last:
                head_line = r
        if "plain_fp64" in row:
            for arm in row:
                if arm != "plain_fp64":
                    row[arm]["speedup_vs_plain_fp64"] = row[arm]["value"] / row["plain_fp64"]["value"]
        windows.append(row)
    ncell = args.n ** 3
    value = head_line["value"]
    roof, breakdown = roofline_window(args, arms)
    memory = device_memory(arms)
    fp64 = fp64_peak(arms)
    out = {
        "metric": METRIC, "value": value, "unit": "time-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head_line["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Gaussian random field permeability; no data set)",
        "config": config_of(args, world),
        "cell_updates_per_s": value * ncell,
        "darcy_solve_ms": head_line["darcy_solve_ms"],
        "pcg_iterations_per_step": head_line["pcg_iterations_per_step"],
        "outer_passes_per_step": head_line["outer_passes_per_step"],
        "relres_max": head_line["relres_max"],
        "relres0_mean": head_line["relres0_mean"],
        "fused_update_ms": head_line["fused_update_ms"],
        "update_active_fraction": head_line["update_active_fraction"],
        "update_interface_fraction": head_line["update_interface_fraction"],
        "gpu_launches": head_line["gpu_launches"],
        "roofline": roof,
        "roofline_update": update_roofline(head_line, ncell),
        "clocks": head_line.get("clocks"),
        "windows": windows,
        "device_memory": memory,
        "fp64_peak": fp64,
    }
    last = windows[-1]
    if "plain_fp64" in last:
        out["plain_fp64"] = last["plain_fp64"]
        out["speedup_vs_plain_fp64"] = value / last["plain_fp64"]["value"]
    for arm in ("learned", "extrapolated"):
        if arm in last and arm != head:
            out[arm] = last[arm]
    if breakdown:
        out["kernel_class_ms"] = breakdown
    if not args.no_e2e:
        arms.set(head)
        out["e2e"] = e2e_pass(args, arms.sim, arms.stream(), world)
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            out["cpu_baseline"] = cpu_sample(arms.sim, args)
        except Exception as e:  # the baseline must not sink the GPU line
            out["cpu_baseline"] = {"value": None, "error": str(e)[:200]}
    arms.close()
    if args.kwh_alt > 0:
        out["kwh_alt"] = alt_kwh_pass(args, rank, world, [a for a in arms_list if a != "learned"])
    if not args.no_ensemble and world == 1:
        out["ensemble"] = ensemble_pass(args)
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)


def ensemble_pass(args):
    """48 permeability realisations with uneven grids (16 each at 64^3, 96^3,
    128^3; log-K variance U(0.5, 3), correlation length U(3, 12), Damkohler
    log-uniform on [1, 100]), FP32-refined solve to 1e-8: launch shapes and
    solver settings autotuned per grid shape, then every ensemble step one
    launch of one CUDA graph holding all members (wpf_ensemble_run); timed
    with a synchronize on both sides."""
    from mizuho_edit_gb300 import ensemble
    members = ensemble.make_members((16, 16, 16))
    tuned = ensemble.autotune(members, spinup=10, steps=4, log=lambda *a: None)
    res = ensemble.run(members, tuned, args.ensemble_steps, 20, 16, log=lambda *a: None)
    # the same steps in the two other launch forms, for comparison
    turn = ensemble.run(members, tuned, args.ensemble_steps, 20, 16, log=lambda *a: None, in_turn=True)
    pool = ensemble.run(members, tuned, args.ensemble_steps, 20, 16, log=lambda *a: None, step_graph=False)
    return {"metric": "ensemble cell-updates/s", "value": res["ensemble_cell_updates_per_s"],
            "members": res["members"], "shapes": res["shapes"], "steps": res["steps"],
            "spinup": res["spinup"], "wall_s": res["wall_s"],
            "member_steps_per_s": res["member_steps_per_s"],
            "converged_last_step": res["converged_last_step"],
            "launch": "one CUDA graph launch per ensemble step (all members' steps as branches)",
            "other_launch_forms": {
                "members_in_turn_one_graph_launch_each": turn["ensemble_cell_updates_per_s"],
                "host_driven_steps_16_threads": pool["ensemble_cell_updates_per_s"]},
            "tuned": ensemble.tuned_table(tuned)}


def alt_kwh_pass(args, rank, world, arm_names):
    """The same windows at a second dissolved-rock permeability (kwh): how
    the numbers move with the contrast between dissolved and intact rock."""
    case = make_workload(args, rank, kwh=args.kwh_alt)
    arms = Arms(args, case, want_net=False)
    rows = []
    try:
        for w in windows_of(args):
            arms.advance_to(w)
            snap = arms.snapshot()
            row = {}
            for a in arm_names:
                arms.restore(snap)
                row[a] = arms.time(a, world)
            if "plain_fp64" in row and "extrapolated" in row:
                row["extrapolated"]["speedup_vs_plain_fp64"] = (row["extrapolated"]["value"] /
                                                                row["plain_fp64"]["value"])
            rows.append(row)
    finally:
        arms.close()
    return {"workload": workload_name(args, args.kwh_alt), "windows": rows}


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
    cfg = {"workload": workload_name(args), "grid": [n, n, n],
           "solver": "BiCGStab + SOR(10 sweeps, omega 1.7) at rtol 1e-10, maxit 1000, from the "
                     "previous pressure: the reference's PETSc settings (wPFAW3D.f90:616-617, "
                     "980, 994-1000), host-driven on the CPU (C restatement, OpenMP threads as "
                     "the SOR blocks of MPI ranks)",
           "darcy_rtol": 1e-10, "dtype_state": "f64",
           "timed_steps": f"{wdone + 1}..{wdone + len(times)} of a cold run (the GPU arms time "
                         f"steps past {windows_of(args)[-1]}; this solver needs 62-72 BiCGStab "
                         f"iterations per solve at every step observed, early or late, so its "
                         f"cost per step does not depend on the window)",
           "parallelism": "single-domain, host cores"}
    out = {"metric": METRIC, "value": v, "unit": "time-steps/s", "n_gpus": world,
           "steps": len(times), "warmup": wdone, "ms_per_step": 1000.0 * tot / len(times),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded Gaussian random field permeability; no data set)",
           "config": cfg, "impl": "reference",
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
