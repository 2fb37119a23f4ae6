"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Wraps ``wpf_oracle.c`` -- the plain-C restatement of the reference routines
of wPFAW3D.f90 -- behind a class whose methods carry the reference subroutine
names.  Used by tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
legs as the checker; the product package never imports it.

Parity unpinned against the reference binary (not buildable here: Fortran +
Intel MPI + PETSc 3.22); pinned by analytic cases and by a scipy direct solve
of the system the reference assembles (tests/test_oracle_*.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libwpf_oracle.so")

SOLVE_BCGS_SOR = 0
SOLVE_CG = 1
SOLVE_MGCG = 2   # same system and stopping test as SOLVE_CG; faster at 64^3 and up


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (OpenMP, strict FP: -ffp-contract=off)."""
    src = os.path.join(HERE, "wpf_oracle.c")
    hdr = os.path.join(HERE, "wpf_oracle.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class _Params(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("ix_ref", C.c_int32), ("iy_ref", C.c_int32), ("iz_ref", C.c_int32),
                ("dx", C.c_double), ("epsilon", C.c_double), ("lambda_", C.c_double),
                ("porosity", C.c_double), ("viscosity", C.c_double), ("diffusion", C.c_double),
                ("ral", C.c_double), ("rat", C.c_double), ("permeab_hole", C.c_double),
                ("alpha", C.c_double)]


class _Well(C.Structure):
    _fields_ = [("ix", C.c_int32), ("iy", C.c_int32), ("iz", C.c_int32), ("pad", C.c_int32),
                ("pressure", C.c_double), ("injection", C.c_double),
                ("phase", C.c_double), ("concent", C.c_double)]


_DP = C.POINTER(C.c_double)


class _State(C.Structure):
    _fields_ = [("p", _Params), ("nwell", C.c_int32), ("pad", C.c_int32),
                ("well", C.POINTER(_Well)), ("lw", C.POINTER(C.c_int32)),
                ("permeab_rock", _DP), ("permeab", _DP), ("pressure", _DP), ("velocity", _DP),
                ("phase", _DP), ("concent", _DP), ("dphasedt", _DP), ("dconcentdt", _DP)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("rnorm", C.c_double),
                ("bnorm", C.c_double), ("true_relres", C.c_double)]


class Diag(C.Structure):
    _fields_ = [("pv", C.c_double), ("vcal", C.c_double), ("rwhmax", C.c_double),
                ("phase_max", C.c_double), ("phase_min", C.c_double),
                ("concent_max", C.c_double), ("concent_min", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = LIB_PATH if os.path.exists(LIB_PATH) else build()
        L = C.CDLL(path)
        SP = C.POINTER(_State)
        L.orc_build_lw.argtypes = [SP]
        L.orc_init_fields.argtypes = [SP, C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_apply_well_values.argtypes = [SP]
        L.orc_update_halo.argtypes = [C.POINTER(_Params), _DP]
        L.orc_calc_permeability.argtypes = [SP]
        L.orc_assemble.argtypes = [SP, C.POINTER(C.c_int32), C.POINTER(C.c_int32), _DP, _DP]
        L.orc_assemble.restype = C.c_long
        L.orc_solve_pressure.argtypes = [SP, C.c_int, C.c_double, C.c_int, C.c_int,
                                         C.POINTER(SolveInfo)]
        L.orc_solve_pressure.restype = C.c_int
        L.orc_calc_velocity.argtypes = [SP]
        L.orc_calc_phase_deriv.argtypes = [SP, C.POINTER(C.c_long)]
        L.orc_calc_phase_deriv.restype = C.c_double
        L.orc_calc_concent_deriv.argtypes = [SP]
        L.orc_evolve_phase.argtypes = [SP, C.c_double]
        L.orc_evolve_concent.argtypes = [SP, C.c_double]
        L.orc_next_dtime.argtypes = [C.POINTER(_Params), C.c_double, C.c_int, C.c_double,
                                     C.c_double]
        L.orc_next_dtime.restype = C.c_double
        L.orc_diagnostics.argtypes = [SP, C.POINTER(Diag)]
        L.orc_get_pressure.argtypes = [SP, C.c_int, C.c_int, C.c_int]
        L.orc_get_pressure.restype = C.c_double
        L.orc_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def _ptr(a: np.ndarray, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct))


class OracleSim:
    """The module state of wPFAW3D (wPFAW3D.f90:78-103) on the CPU.

    Fields are halo arrays of shape (nx+2, ny+2, nz+2) in Fortran order, so
    ``phase[i, j, k]`` is the reference's ``phase(i, j, k)``.
    """

    def __init__(self, params, permeab_rock: Optional[np.ndarray] = None,
                 phase: Optional[np.ndarray] = None, concent: Optional[np.ndarray] = None):
        p = params
        self.params = p
        nx, ny, nz = p.nx, p.ny, p.nz
        sh = (nx + 2, ny + 2, nz + 2)
        z = lambda *s: np.zeros(s, dtype=np.float64, order="F")  # noqa: E731
        self.lw = np.zeros(sh, dtype=np.int32, order="F")
        self.permeab_rock = z(*sh)
        self.permeab = z(4, *sh)
        self.pressure = z(*sh)
        self.velocity = z(3, *sh)
        self.phase = z(*sh)
        self.concent = z(*sh)
        self.dphasedt = z(*sh)
        self.dconcentdt = z(*sh)
        ws = (_Well * max(1, len(p.wells)))()
        for n, w in enumerate(p.wells):
            ws[n] = _Well(w.ix, w.iy, w.iz, 0, w.pressure, w.injection, w.phase, w.concent)
        self._wells = ws
        self._cp = _Params(nx, ny, nz, p.ix_ref, p.iy_ref, p.iz_ref, p.dx, p.epsilon, p.lambda_,
                           p.porosity, p.viscosity, p.diffusion, p.ral, p.rat, p.permeab_hole,
                           p.alpha)
        self._st = _State(self._cp, len(p.wells), 0, ws, _ptr(self.lw, C.c_int32),
                          _ptr(self.permeab_rock), _ptr(self.permeab), _ptr(self.pressure),
                          _ptr(self.velocity), _ptr(self.phase), _ptr(self.concent),
                          _ptr(self.dphasedt), _ptr(self.dconcentdt))
        L = lib()
        # loadConfig order, wPFAW3D.f90:452-496
        L.orc_build_lw(C.byref(self._st))
        L.orc_init_fields(C.byref(self._st), p.init_permeab, p.init_phase, p.init_concent, p.pini)
        L.orc_apply_well_values(C.byref(self._st))
        if permeab_rock is not None:          # loadField overrides, :485-486
            self.permeab_rock[1:-1, 1:-1, 1:-1] = permeab_rock
        if phase is not None:
            self.phase[1:-1, 1:-1, 1:-1] = phase
        if concent is not None:
            self.concent[1:-1, 1:-1, 1:-1] = concent
        for f in (self.permeab_rock, self.phase, self.concent):
            L.orc_update_halo(C.byref(self._cp), _ptr(f))
        self.dtime = p.dtime
        self.taumin = 0.0
        self.itime = 0
        self.time = p.time_start
        self.overshoot = 0
        self.last_solve = SolveInfo()

    # --- the reference routines ------------------------------------------------
    def calcPermeability(self):
        lib().orc_calc_permeability(C.byref(self._st))

    def solvePressure(self, mode: int = SOLVE_CG, rtol: float = 1e-13, maxit: int = 100000,
                      nblocks: int = 1) -> SolveInfo:
        info = SolveInfo()
        lib().orc_solve_pressure(C.byref(self._st), mode, rtol, maxit, nblocks, C.byref(info))
        self.last_solve = info
        return info

    def calcVelocity(self):
        lib().orc_calc_velocity(C.byref(self._st))

    def calcPhaseDeriv(self) -> float:
        ov = C.c_long(0)
        self.taumin = lib().orc_calc_phase_deriv(C.byref(self._st), C.byref(ov))
        self.overshoot = ov.value
        return self.taumin

    def calcConcentDeriv(self):
        lib().orc_calc_concent_deriv(C.byref(self._st))

    def evolvePhase(self, dtime: float):
        lib().orc_evolve_phase(C.byref(self._st), dtime)

    def evolveConcent(self, dtime: float):
        lib().orc_evolve_concent(C.byref(self._st), dtime)

    def updateHalo(self, f: np.ndarray):
        lib().orc_update_halo(C.byref(self._cp), _ptr(f))

    def next_dtime(self, itime: int) -> float:
        return lib().orc_next_dtime(C.byref(self._cp), self.params.tfac, itime, self.dtime,
                                    self.taumin)

    def step(self, mode: int = SOLVE_CG, rtol: float = 1e-13, maxit: int = 100000,
             nblocks: int = 1) -> SolveInfo:
        """One pass of the main loop body, wPFAW3D.f90:2226-2280."""
        self.itime += 1
        self.dtime = self.next_dtime(self.itime)
        self.time += self.dtime
        self.calcPermeability()
        info = self.solvePressure(mode, rtol, maxit, nblocks)
        self.calcVelocity()
        self.calcPhaseDeriv()
        self.calcConcentDeriv()
        self.evolvePhase(self.dtime)
        self.evolveConcent(self.dtime)
        return info

    def breakthrough_plane(self) -> int:
        """ix of the plane whose phase maximum signals breakthrough: nx -
        ceil(2 w / dx), at least 1 (outlet wells pin phase = -1 on ix = nx and
        the interface, ~2w wide, cannot cross the pinned plane)."""
        p = self.params
        k = max(1, int(np.ceil(2.0 * p.epsilon / p.dx - 1e-9)))
        return max(1, p.nx - k)

    def inlet_flux(self) -> float:
        """Q_in = sum of u_x over the faces between ix = 1 and 2, times dx^2
        (the velocity of the last calcVelocity)."""
        p = self.params
        return float(self.velocity[0, 1, 1:-1, 1:-1].sum()) * p.dx * p.dx

    def diagnostics(self) -> dict:
        d = Diag()
        lib().orc_diagnostics(C.byref(self._st), C.byref(d))
        return d.as_dict()

    def getPressure(self, ix: int, iy: int, iz: int) -> float:
        return lib().orc_get_pressure(C.byref(self._st), ix, iy, iz)

    def assemble(self):
        """The reference's triplets (irn, jcn, val) and b, wPFAW3D.f90:629-936."""
        L = lib()
        nnz = L.orc_assemble(C.byref(self._st), None, None, None, None)
        irn = np.zeros(nnz, np.int32)
        jcn = np.zeros(nnz, np.int32)
        val = np.zeros(nnz, np.float64)
        b = np.zeros(self.params.nx * self.params.ny * self.params.nz, np.float64)
        L.orc_assemble(C.byref(self._st), _ptr(irn, C.c_int32), _ptr(jcn, C.c_int32), _ptr(val),
                       _ptr(b))
        return irn, jcn, val, b
