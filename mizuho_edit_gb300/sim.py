"""Host-side mirror of the wPFAW3D module interface over the C ABI.

``Simulation`` carries the reference's module state (wPFAW3D.f90:78-103) on
the GPU and exposes the reference's subroutines under their own names
(``calcPermeability``, ``solvePressure``, ``calcVelocity``,
``calcPhaseDeriv``, ``calcConcentDeriv``, ``evolvePhase``,
``evolveConcent``), plus the fused ``step`` of the main-loop body
(wPFAW3D.f90:2226-2280), ``showProgress``-style diagnostics and ``.fld``
restart I/O.  Every compute call goes through libwpf_gb300.so.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import capi
from .config import Params, load_config
from .fld import read_fld, write_fld

__all__ = ["Simulation"]


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(capi.DP)


class Simulation:
    """One wPFAW3D domain resident on the current CUDA device."""

    def __init__(self, params: Params, permeab_rock: Optional[np.ndarray] = None,
                 phase: Optional[np.ndarray] = None, concent: Optional[np.ndarray] = None,
                 solver: str = "fp64", rtol: float = 1e-8, inner_rtol: float = 1e-4,
                 max_inner: int = 500, max_outer: int = 20, smooth_sweeps: int = 2,
                 sweep_min_cells: int = 0, w_from_level: int = 0, graphs: bool = True,
                 extrapolate: bool = False, tma: bool = True, step_graph: bool = False,
                 sweep_zchunk: int = 0, row_blocks_per_sm: int = 0, net_always: bool = False,
                 fp64_update: bool = False, net_coarse: bool = False, fixed_start: bool = False):
        self.L = capi.load()
        self.params = p = params
        if p.tfac is None:
            raise ValueError("tfac is required")
        cp = capi.Params(p.nx, p.ny, p.nz, p.ix_ref, p.iy_ref, p.iz_ref, p.dx, p.epsilon,
                         p.lambda_, p.porosity, p.viscosity, p.diffusion, p.ral, p.rat,
                         p.permeab_hole, p.alpha, p.tfac)
        h = C.c_void_p()
        capi.check(self.L.wpf_create(C.byref(cp), C.byref(h)), "wpf_create")
        self.h = h
        ws = (capi.Well * max(1, len(p.wells)))()
        for n, w in enumerate(p.wells):
            ws[n] = capi.Well(w.ix, w.iy, w.iz, 0, w.pressure, w.injection, w.phase, w.concent)
        capi.check(self.L.wpf_set_wells(h, ws, len(p.wells)), "wpf_set_wells")
        self.set_solver(solver, rtol, inner_rtol=inner_rtol, max_inner=max_inner,
                        max_outer=max_outer, smooth_sweeps=smooth_sweeps,
                        sweep_min_cells=sweep_min_cells, w_from_level=w_from_level,
                        graphs=graphs, extrapolate=extrapolate, tma=tma, step_graph=step_graph,
                        sweep_zchunk=sweep_zchunk, row_blocks_per_sm=row_blocks_per_sm,
                        net_always=net_always, fp64_update=fp64_update, net_coarse=net_coarse,
                        fixed_start=fixed_start)
        # initial fields exactly as loadConfig builds them (wPFAW3D.f90:464-496)
        sh = self.halo_shape
        kr = np.full(sh, p.init_permeab, order="F")
        ph = np.full(sh, p.init_phase, order="F")
        cc = np.full(sh, p.init_concent, order="F")
        pr = np.full(sh, p.pini, order="F")
        for w in p.wells:
            if 1 <= w.ix <= p.nx and 1 <= w.iy <= p.ny and 1 <= w.iz <= p.nz:
                ph[w.ix, w.iy, w.iz] = w.phase
                cc[w.ix, w.iy, w.iz] = w.concent
        if permeab_rock is not None:
            kr[1:-1, 1:-1, 1:-1] = permeab_rock
        if phase is not None:
            ph[1:-1, 1:-1, 1:-1] = phase
        if concent is not None:
            cc[1:-1, 1:-1, 1:-1] = concent
        self._kr_cache = np.array(kr[1:-1, 1:-1, 1:-1])
        self.upload(kr, ph, cc, pr)
        self.itime = 0
        self.time = p.time_start
        self.dtime = p.dtime
        self.taumin = 0.0
        self.last = capi.StepStats()

    # -- construction from files ------------------------------------------------
    @classmethod
    def from_config(cls, path: str, **kw) -> "Simulation":
        """``loadConfig`` + ``loadField`` (wPFAW3D.f90:264-557)."""
        p = load_config(path)
        kr = ph = cc = None
        if p.filename_init:
            f = read_fld(p.filename_init, expect_grid=(p.nx, p.ny, p.nz))
            p.time_start = f.time
            kr, ph, cc = f.permeab_rock, f.phase, f.concent
        else:
            p.time_start = 0.0
        p.time_end = p.time_start + p.time_total
        return cls(p, kr, ph, cc, **kw)

    # -- plumbing -----------------------------------------------------------------
    @property
    def halo_shape(self):
        p = self.params
        return (p.nx + 2, p.ny + 2, p.nz + 2)

    def set_solver(self, mode: str = "fp64", rtol: float = 1e-8, inner_rtol: float = 1e-4,
                   max_inner: int = 500, max_outer: int = 20, smooth_sweeps: int = 2,
                   sweep_min_cells: int = 0, w_from_level: int = 0, graphs: bool = True,
                   extrapolate: bool = False, tma: bool = True, step_graph: bool = False,
                   sweep_zchunk: int = 0, row_blocks_per_sm: int = 0, net_always: bool = False,
                   fp64_update: bool = False, net_coarse: bool = False, fixed_start: bool = False):
        """Solver options (wpf_set_solver); graphs=False launches every
        preconditioner cycle kernel by kernel instead of replaying a CUDA graph;
        extrapolate=True starts each solve from the pressure extrapolated in
        time -- in the mixed form the least-squares combination of the last two
        increments unless fixed_start -- with the fallback to the previous
        pressure; tma=False stages the pipelined sweep with cp.async instead of
        bulk-tensor copies;
        step_graph=True runs each step (from the fourth) as one CUDA graph launch
        with the solver's loops on the device; sweep_zchunk and row_blocks_per_sm
        are launch shapes (z planes per block of the pipelined sweep, blocks per
        SM of the row-patch kernels; 0 = the library's choice); net_always
        evaluates an attached net's correction at every solve instead of only
        when the extrapolated start misses rtol by at most 1.02x; fp64_update
        keeps the mixed form's update rates in FP64; net_coarse makes the net's
        output, in the solves where it was evaluated, the one-vector coarse
        space of a deflated PCG; fixed_start keeps the extrapolated start's
        fixed quadratic-in-time coefficients instead of the least-squares
        ones."""
        m = {"fp64": capi.SOLVER_FP64, "mixed": capi.SOLVER_MIXED}[mode]
        flags = (0 if graphs else capi.SOLVER_NO_GRAPHS) | \
            (capi.SOLVER_EXTRAPOLATE if extrapolate else 0) | \
            (0 if tma else capi.SOLVER_NO_TMA) | \
            (capi.SOLVER_STEP_GRAPH if step_graph else 0) | \
            (capi.SOLVER_NET_ALWAYS if net_always else 0) | \
            (capi.SOLVER_FP64_UPDATE if fp64_update else 0) | \
            (capi.SOLVER_NET_COARSE if net_coarse else 0) | \
            (capi.SOLVER_FIXED_START if fixed_start else 0)
        o = capi.SolverOpts(m, max_outer, max_inner, smooth_sweeps, rtol, inner_rtol,
                            sweep_min_cells, w_from_level, flags, sweep_zchunk, row_blocks_per_sm)
        capi.check(self.L.wpf_set_solver(self.h, C.byref(o)), "wpf_set_solver")
        self.solver = mode

    def upload(self, permeab_rock=None, phase=None, concent=None, pressure=None):
        arrs = [None if a is None else np.asfortranarray(a, dtype=np.float64)
                for a in (permeab_rock, phase, concent, pressure)]
        for a in arrs:
            if a is not None and a.shape != self.halo_shape:
                raise ValueError(f"expected a halo array of shape {self.halo_shape}")
        capi.check(self.L.wpf_upload(self.h, *[_p(a) for a in arrs]), "wpf_upload")

    def download(self, *names):
        """Halo arrays by reference name: phase, concent, pressure, permeab,
        velocity, dphasedt, dconcentdt."""
        sh = self.halo_shape
        out = {}
        want = names or ("phase", "concent", "pressure")
        for n in want:
            if n == "permeab":
                out[n] = np.zeros((4,) + sh, order="F")
            elif n == "velocity":
                out[n] = np.zeros((3,) + sh, order="F")
            else:
                out[n] = np.zeros(sh, order="F")
        order = ["phase", "concent", "pressure", "permeab", "velocity", "dphasedt", "dconcentdt"]
        args = [_p(out.get(n)) for n in order]
        capi.check(self.L.wpf_download(self.h, *args), "wpf_download")
        return out if len(want) > 1 or not names else out[want[0]]

    def close(self):
        if getattr(self, "h", None):
            self.L.wpf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- the reference routines -----------------------------------------------------
    def calcPermeability(self):
        capi.check(self.L.wpf_calc_permeability(self.h), "calcPermeability")

    def solvePressure(self) -> capi.StepStats:
        st = capi.StepStats()
        capi.check(self.L.wpf_solve_pressure(self.h, C.byref(st)), "solvePressure")
        return st

    def calcVelocity(self):
        capi.check(self.L.wpf_calc_velocity(self.h), "calcVelocity")

    def calcPhaseDeriv(self) -> float:
        t = C.c_double()
        o = C.c_int32()
        capi.check(self.L.wpf_calc_phase_deriv(self.h, C.byref(t), C.byref(o)), "calcPhaseDeriv")
        self.taumin = t.value
        self.overshoot = o.value
        return t.value

    def calcConcentDeriv(self):
        capi.check(self.L.wpf_calc_concent_deriv(self.h), "calcConcentDeriv")

    def evolvePhase(self, dtime: float):
        capi.check(self.L.wpf_evolve_phase(self.h, dtime), "evolvePhase")

    def evolveConcent(self, dtime: float):
        capi.check(self.L.wpf_evolve_concent(self.h, dtime), "evolveConcent")

    def next_dtime(self, itime: int) -> float:
        """dt law, wPFAW3D.f90:2227-2230 (taumin lags one step)."""
        p = self.params
        if itime >= 3:
            e2 = p.epsilon * p.epsilon
            return p.tfac * 0.5 * (p.dx * p.dx) / e2 * min(e2 / p.diffusion, self.taumin)
        return self.dtime

    def step_unfused(self) -> capi.StepStats:
        """The main-loop body through the per-routine entry points."""
        self.itime += 1
        self.dtime = self.next_dtime(self.itime)
        self.time += self.dtime
        self.calcPermeability()
        st = self.solvePressure()
        self.calcVelocity()
        self.calcPhaseDeriv()
        self.calcConcentDeriv()
        self.evolvePhase(self.dtime)
        self.evolveConcent(self.dtime)
        self.last = st
        return st

    def step(self, allow_unconverged: bool = False) -> capi.StepStats:
        """One fused step (wpf_step)."""
        self.itime += 1
        st = capi.StepStats()
        dt = C.c_double(self.dtime)
        ok = (capi.WPF_OK, capi.WPF_ERR_NOT_CONVERGED) if allow_unconverged else (capi.WPF_OK,)
        capi.check(self.L.wpf_step(self.h, self.itime, C.byref(dt), C.byref(st)), "wpf_step", ok)
        self.dtime = dt.value
        self.time += self.dtime
        self.taumin = st.taumin
        self.last = st
        return st

    def run(self, nsteps: int):
        stats = []
        for _ in range(nsteps):
            stats.append(self.step())
        return stats

    # -- diagnostics / I/O -------------------------------------------------------------
    def diagnostics(self) -> dict:
        d = capi.Diag()
        capi.check(self.L.wpf_reduce(self.h, C.byref(d)), "wpf_reduce")
        return d.as_dict()

    def getPressure(self, ix: int, iy: int, iz: int) -> float:
        p = self.params
        if not (1 <= ix <= p.nx and 1 <= iy <= p.ny and 1 <= iz <= p.nz):
            return 0.0
        return float(self.download("pressure")[ix, iy, iz])

    def saveField(self, path: str):
        """``saveField`` (wPFAW3D.f90:2096-2141)."""
        d = self.download("phase", "concent")
        kr = self._krock_host()
        write_fld(path, self.time, kr, d["phase"][1:-1, 1:-1, 1:-1], d["concent"][1:-1, 1:-1, 1:-1])

    def _krock_host(self):
        if not hasattr(self, "_kr_cache"):
            raise RuntimeError("permeab_rock is not kept on the host")
        return self._kr_cache
