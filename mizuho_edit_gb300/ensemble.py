"""Ensembles of permeability realisations with uneven grids, advanced together.

The members are independent wPFAW3D domains (no counterpart in the reference,
which runs one).  ``wpf_ensemble_run`` advances them together: once every
member can take the device-resident step, each ensemble step is one launch of
one CUDA graph holding all members' steps as independent branches (their
solver loops are conditional nodes), so that small grids -- whose kernels are
too short to fill 152 SMs -- overlap on the device with no host round trip;
before that (the first steps) a pool of host threads steps the members, each
on its own stream.  Before the timed run, an
autotuner picks, per grid shape, the solver configuration and the launch shapes (multigrid cycle
shape, the level size from which the pipelined sweep kernel is used,
smoothing sweeps, the sweep's z planes per block, the row-patch kernels'
blocks per SM) with the best measured time per step.

Why one graph launch per ensemble step rather than one persistent kernel:
every PCG iteration of every member ends in a reduction that decides the next
launch, so a persistent kernel would need a grid-wide barrier per solver phase
of each member and one block shape for kernels whose best shapes differ
(32x8 sweep tiles, 128-row patches, the one-block bottom cycle); the graph
keeps each kernel's own launch shape, turns the decisions into conditional
nodes evaluated on the device and still costs one launch and one
synchronisation per ensemble step.

    python -m mizuho_edit_gb300.ensemble [--members 16,16,16] [--steps 20]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np

from . import capi
from .cases import make_case
from .sim import Simulation

SHAPES = ((64, 64, 64), (96, 96, 96), (128, 128, 128))
# candidate solver configurations: (W-cycle from level, pipelined-sweep threshold, sweeps per
# side, z planes per block of the pipelined sweep (0: the wave-filling chunk), row-patch blocks
# per SM (0: 8))
CANDIDATES = [(2, 0, 2, 0, 0), (1, 0, 2, 0, 0), (3, 0, 2, 0, 0), (2, 0, 3, 0, 0),
              (2, 1 << 18, 2, 0, 0), (1, 1 << 18, 2, 0, 0), (2, 1 << 18, 2, 16, 0), (2, 1 << 18, 2, 32, 0),
              (2, 0, 2, 0, 4), (2, 0, 2, 0, 16)]


def make_members(counts=(16, 16, 16), seed: int = 48):
    """log-K variance U(0.5, 3), correlation length U(3, 12) cells, Damkohler
    log-uniform on [1, 100]; seeded."""
    rng = np.random.default_rng(seed)
    out = []
    for shape, cnt in zip(SHAPES, counts):
        for _ in range(cnt):
            lv = float(rng.uniform(0.5, 3.0))
            cl = float(rng.uniform(3.0, 12.0))
            da = float(10.0 ** rng.uniform(0.0, 2.0))
            s = int(rng.integers(1 << 30))
            out.append((shape, dict(log_var=lv, corr_len=cl, da=da, seed=s)))
    return out


def _opts(c):
    w, thr, nu, zc, rb = c
    return dict(w_from_level=w, sweep_min_cells=thr, smooth_sweeps=nu, sweep_zchunk=zc,
                row_blocks_per_sm=rb)


def _sim(shape, kw, opts, step_graph=False):
    case = make_case(shape, **kw)
    return Simulation(case.params, case.permeab_rock, case.phase, case.concent, solver="mixed", rtol=1e-8,
                      extrapolate=True, step_graph=step_graph, **opts)


def autotune(members, spinup: int = 20, steps: int = 6, log=print):
    """Per grid shape: time every candidate on the first member of that shape
    (after `spinup` steps and 3 steps that rebuild the start history), keep
    the fastest.  Returns {shape: (candidate, {candidate: ms per step})}."""
    import torch
    best = {}
    for shape in sorted({m[0] for m in members}):
        kw = next(m[1] for m in members if m[0] == shape)
        times = {}
        with _sim(shape, kw, _opts(CANDIDATES[0])) as sim:
            for _ in range(spinup):
                sim.step()
            for c in CANDIDATES:
                sim.set_solver("mixed", 1e-8, extrapolate=True, **_opts(c))
                for _ in range(3):
                    sim.step()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for _ in range(steps):
                    sim.step()
                torch.cuda.synchronize()
                times[c] = 1e3 * (time.perf_counter() - t0) / steps
        c = min(times, key=times.get)
        best[shape] = (c, times)
        log(f"{shape}: best {c} ({times[c]:.2f} ms/step) of " +
            ", ".join(f"{k}: {v:.2f}" for k, v in times.items()))
    return best


def run(members, tuned, steps: int, spinup: int, threads: int, log=print, step_graph: bool = True,
        in_turn: bool = False):
    """Advance every member `spinup` untimed steps, then `steps` timed ones
    through wpf_ensemble_run (step_graph: every step from the third one launch
    of one graph holding all members; else host-driven steps from a thread
    pool); in_turn (with step_graph) times the members' steps one after
    another instead, each wpf_step one launch of that member's own graph.
    Returns the throughput figures."""
    import torch
    sims = [_sim(shape, kw, _opts(tuned[shape][0] if tuned else CANDIDATES[0]), step_graph)
            for shape, kw in members]
    try:
        L = sims[0].L
        n = len(sims)
        hs = (C.c_void_p * n)(*[s.h.value for s in sims])
        dt = (C.c_double * n)(*[s.dtime for s in sims])
        stats = (capi.StepStats * n)()
        status = (C.c_int32 * n)()
        ok = (capi.WPF_OK, capi.WPF_ERR_NOT_CONVERGED)
        warm = 2 if in_turn else 0   # the members' own graphs are captured in these
        capi.check(L.wpf_ensemble_run(hs, n, 1, spinup - warm, threads, dt, stats, status), "ensemble spin-up",
                   ok)

        def in_turn_steps(first, count):
            for it in range(first, first + count):
                for m in range(n):
                    d = C.c_double(dt[m])
                    status[m] = L.wpf_step(hs[m], it, C.byref(d), C.byref(stats[m]))
                    capi.check(status[m], "wpf_step", ok)
                    dt[m] = d.value
        if warm:
            in_turn_steps(1 + spinup - warm, warm)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if in_turn:
            in_turn_steps(1 + spinup, steps)
        else:
            capi.check(L.wpf_ensemble_run(hs, n, 1 + spinup, steps, threads, dt, stats, status), "ensemble", ok)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        cells = sum(int(np.prod(shape)) for shape, _ in members)
        res = {"members": n, "shapes": {str(s): sum(1 for m in members if m[0] == s) for s in SHAPES},
               "steps": steps, "spinup": spinup, "threads": threads, "wall_s": wall,
               "one_graph_per_step": step_graph and not in_turn,
               "ensemble_cell_updates_per_s": cells * steps / wall,
               "member_steps_per_s": n * steps / wall,
               "converged_last_step": int(sum(1 for s in stats if s.converged)),
               "status": sorted(set(int(x) for x in status))}
        return res
    finally:
        for s in sims:
            s.close()


def tuned_table(tuned):
    """The autotuner's choice per shape, JSON-ready."""
    if not tuned:
        return None
    return {str(k): {"w_from_level": v[0][0], "sweep_min_cells": v[0][1], "smooth_sweeps": v[0][2],
                     "sweep_zchunk": v[0][3], "row_blocks_per_sm": v[0][4],
                     "ms_per_step": {str(c): t for c, t in v[1].items()}}
            for k, v in tuned.items()}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--members", default="16,16,16")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--spinup", type=int, default=20)
    ap.add_argument("--threads", type=int, default=16)
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--host-steps", action="store_true",
                    help="host-driven steps only (no device-resident step graphs)")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    counts = tuple(int(x) for x in a.members.split(","))
    members = make_members(counts)
    tuned = None if a.no_tune else autotune(members)
    res = run(members, tuned, a.steps, a.spinup, a.threads, step_graph=not a.host_steps)
    if not a.host_steps:   # the thread-pool form on the same members, for comparison
        res["host_threaded_cell_updates_per_s"] = run(
            members, tuned, a.steps, a.spinup, a.threads, step_graph=False)["ensemble_cell_updates_per_s"]
    res["tuned"] = tuned_table(tuned)
    # the same members one after the other on one thread, for comparison
    if not a.no_tune:
        seq = run(members, tuned, max(a.steps // 4, 2), a.spinup, 1, step_graph=False)
        res["one_thread_cell_updates_per_s"] = seq["ensemble_cell_updates_per_s"]
    s = json.dumps(res)
    print(s)
    if a.out:
        with open(a.out, "w") as fh:
            fh.write(s + "\n")


if __name__ == "__main__":
    main()
