"""Seeded synthetic wormholing cases.

No public data set is involved: every input is generated here from a seed.
Permeability is ``K = exp(sigma * g)`` with ``g`` a Gaussian random field of
zero mean and unit variance with squared-exponential covariance
``C(r) = exp(-r^2 / (2 l^2))``, made by filtering white noise in Fourier
space (periodic) and normalising the sample.

Dimensionless convention (dx = 1 via ``w = 2``, ``dxw = 0.5``; ``visco = 1``;
geometric-mean permeability 1; pressure drop 1 from the inlet plane ``ix = 1``
to the outlet plane ``ix = nx``):

* Peclet:  ``D = 1 / Pe``  (advective flux ``K_g dp / mu`` = 1).
* Damkoehler: ``Da = t_adv / tau0`` with ``t_adv = L^2`` (``L = nx``) and
  ``tau0 = 5/3 * alpha * lambda * w^2 / D`` (the relaxation time of the
  phase equation, wPFAW3D.f90:1254), solved for ``lambda``.
* ``alpha = 0.5 / b / kc`` (wPFAW3D.f90:397-399).  Dissolution (acid moving
  the phase field from rock, -1, toward liquid, +1) needs ``lambda < 0``, and
  a positive relaxation time then needs ``alpha < 0``; the cases reach that
  with ``b100 < 0`` so that the reference's own formula yields it.
* The outlet pressure is ``1e-300`` rather than 0 because the reference treats
  a well pressure of exactly 0 as "not Dirichlet" (wPFAW3D.f90:1106).
"""
from __future__ import annotations

import dataclasses
import os
from typing import Optional, Tuple

import numpy as np

from .config import Params, Well, derive, write_config, write_well_file
from .fld import write_fld

__all__ = ["grf", "make_case", "Case", "write_case"]


def grf(shape: Tuple[int, int, int], corr_len: float, seed: int) -> np.ndarray:
    """Zero-mean, unit-variance Gaussian random field (float64, shape
    (nx, ny, nz)) with squared-exponential covariance of length ``corr_len``."""
    rng = np.random.Generator(np.random.PCG64(seed))
    white = rng.standard_normal(shape)
    kx = np.fft.fftfreq(shape[0])[:, None, None]
    ky = np.fft.fftfreq(shape[1])[None, :, None]
    kz = np.fft.rfftfreq(shape[2])[None, None, :]
    k2 = (2 * np.pi) ** 2 * (kx * kx + ky * ky + kz * kz)
    filt = np.exp(-0.25 * k2 * corr_len * corr_len)   # sqrt of exp(-k^2 l^2 / 2)
    g = np.fft.irfftn(np.fft.rfftn(white) * filt, s=shape, axes=(0, 1, 2))
    g -= g.mean()
    sd = g.std()
    if sd > 0:
        g /= sd
    return g


@dataclasses.dataclass
class Case:
    params: Params
    permeab_rock: np.ndarray     # interior (nx, ny, nz)
    phase: np.ndarray
    concent: np.ndarray
    seed: int
    description: str


def make_case(n: Tuple[int, int, int], *, log_var: float = 1.0, corr_len: float = 4.0,
              seed: int = 0, pe: float = 100.0, da: float = 10.0, kwh: float = 20.0,
              tfac: float = 0.025, dt: float = 0.1, porosity: float = 0.225,
              time_total: float = 1.0e30, pini: float = 0.0,
              outlet_pressure: float = 1.0e-300) -> Case:
    """Build the inputs of one synthetic wormholing run (see module docstring)."""
    nx, ny, nz = n
    p = Params(nx=nx, ny=ny, nz=nz)
    p.dtime = dt
    p.tfac = tfac
    p.time_total = time_total
    p.n_res_out = 1
    p.n_dat_out = 1
    p.epsilon = 2.0
    p.dxw = 0.5
    p.porosity = porosity
    p.rhos = 2710.0
    p.rhoa = 1500.0
    p.viscosity = 1.0
    p.cwtp = 1.0
    p.b100 = -1.37
    p.diffusion = 1.0 / pe
    p.ral = 0.0
    p.rat = 0.0
    p.permeab_hole = kwh
    p.pini = pini
    p.ix_ref, p.iy_ref, p.iz_ref = 1, (ny + 1) // 2, (nz + 1) // 2
    derive(p)
    t_adv = float(nx) ** 2
    tau0 = t_adv / da
    p.lambda_ = tau0 * p.diffusion / (5.0 / 3.0 * p.alpha * p.epsilon ** 2)
    sigma = float(np.sqrt(log_var))
    kr = np.exp(sigma * grf((nx, ny, nz), corr_len, seed)) if log_var > 0 else np.ones((nx, ny, nz))
    phase = -np.ones((nx, ny, nz))
    concent = np.zeros((nx, ny, nz))
    wells = []
    for iz in range(1, nz + 1):
        for iy in range(1, ny + 1):
            wells.append(Well(1, iy, iz, pressure=1.0, injection=0.0, phase=1.0, concent=1.0))
    for iz in range(1, nz + 1):
        for iy in range(1, ny + 1):
            wells.append(Well(nx, iy, iz, pressure=outlet_pressure, injection=0.0, phase=-1.0,
                              concent=0.0))
    p.wells = wells
    phase[0, :, :] = 1.0
    concent[0, :, :] = 1.0
    phase[nx - 1, :, :] = -1.0
    concent[nx - 1, :, :] = 0.0
    desc = (f"{nx}x{ny}x{nz} logvar={log_var} corr={corr_len} seed={seed} Pe={pe} Da={da} "
            f"kwh={kwh} tfac={tfac}")
    return Case(p, kr, phase, concent, seed, desc)


def write_case(case: Case, directory: str, name: str = "case") -> str:
    """Write ``<name>.cfg``, ``<name>.well`` and ``<name>.fld``; return the cfg path."""
    os.makedirs(directory, exist_ok=True)
    p = case.params
    write_well_file(os.path.join(directory, name + ".well"), p.wells)
    write_fld(os.path.join(directory, name + ".fld"), 0.0, case.permeab_rock, case.phase,
              case.concent)
    cfg = os.path.join(directory, name + ".cfg")
    write_config(cfg, p, name + ".well", init_file=name + ".fld")
    return cfg
