"""Host-side configuration: the ``.cfg`` + well-file front end of wPFAW3D.

Mirrors ``loadConfig`` (wPFAW3D.f90:264-505): the same ``key = value``
grammar, the same keys, the same derived parameters and the same error
behaviour (an unknown key or a broken line is an error, wPFAW3D.f90:381-384,
500-504).  Two optional keys that the reference does not know are accepted
here only when ``extended=True`` (``nsteps``, ``solver``); configs written
for parity runs never use them, so they stay readable by the reference.
"""
from __future__ import annotations

import dataclasses
import os
import re
from typing import List, Optional, Sequence

__all__ = ["Params", "Well", "ConfigError", "load_config", "read_well_file",
           "write_config", "write_well_file", "derive"]


class ConfigError(ValueError):
    """A config or well file the reference would reject with ``exit(1)``."""


@dataclasses.dataclass
class Well:
    """One well grid point, ``Well_type`` (wPFAW3D.f90:82-90)."""
    ix: int
    iy: int
    iz: int
    pressure: float = 0.0    # Dirichlet iff != 0 (wPFAW3D.f90:1106)
    injection: float = 0.0   # inlet iff != 0 (wPFAW3D.f90:1140)
    phase: float = -1.0
    concent: float = 0.0


@dataclasses.dataclass
class Params:
    """Scalar members of ``Param_type`` (wPFAW3D.f90:27-76), single domain."""
    nx: int = 0
    ny: int = 0
    nz: int = 0
    dtime: float = 0.1e-6          # default, wPFAW3D.f90:286
    tfac: Optional[float] = None   # no default in the reference: required
    time_start: float = 0.0
    time_total: float = 0.0
    time_end: float = 0.0
    n_res_out: int = 1
    n_dat_out: int = 1
    dtime_res: float = 0.0
    dtime_dat: float = 0.0
    epsilon: float = 0.0           # interface width w
    dxw: float = 0.0
    dx: float = 0.0
    lx: float = 0.0
    ly: float = 0.0
    lz: float = 0.0
    lambda_: float = 0.0
    porosity: float = 0.0
    rhos: float = 0.0
    rhoa: float = 0.0
    viscosity: float = 0.0
    cwtp: float = 0.0
    diffusion: float = 0.0
    b100: float = 0.0
    ral: float = 0.0
    rat: float = 0.0
    permeab_hole: float = 0.0
    alpha: float = 0.0
    pini: float = 0.0
    ix_ref: int = 1
    iy_ref: int = 1
    iz_ref: int = 1
    filename_well: str = ""
    filename_init: str = ""
    filename_last: str = ""
    init_permeab: float = 0.0      # "init K phi c" triple, wPFAW3D.f90:372-377
    init_phase: float = -1.0
    init_concent: float = 0.0
    nsteps: Optional[int] = None   # extension: stop after n steps
    solver: Optional[str] = None   # extension: "fp64" | "mixed"
    wells: List[Well] = dataclasses.field(default_factory=list)

    @property
    def ngrid(self) -> int:
        return self.nx * self.ny * self.nz


_FORTRAN_D = re.compile(r"(?<=[0-9.])[dD](?=[+-]?[0-9])")


def _num(tok: str) -> float:
    """Parse a Fortran list-directed real (accepts ``1.0d-3``)."""
    return float(_FORTRAN_D.sub("e", tok))


def _int(tok: str) -> int:
    return int(tok)


def _split(buf: str) -> List[str]:
    return [t for t in re.split(r"[\s,]+", buf.strip()) if t]


def derive(p: Params) -> Params:
    """Derived parameters, wPFAW3D.f90:391-399."""
    if p.n_res_out:
        p.dtime_res = p.time_total / p.n_res_out
    if p.n_dat_out:
        p.dtime_dat = p.time_total / p.n_dat_out
    p.dx = p.dxw * p.epsilon
    p.lx, p.ly, p.lz = p.dx * p.nx, p.dx * p.ny, p.dx * p.nz
    b = p.rhoa / p.rhos
    kc = p.cwtp * p.b100 / (1.0 - p.porosity)
    p.alpha = 0.5 / b / kc
    return p


def read_well_file(path: str) -> List[Well]:
    """Well file, wPFAW3D.f90:402-432: a title line, the count, one line per well
    ``ix iy iz wpq wval phase concent`` with ``wpq`` = +1 (pressure) or -1
    (injection)."""
    try:
        with open(path, "r") as fh:
            lines = fh.read().splitlines()
    except OSError as e:
        raise ConfigError(f"can not open well file: {path}") from e
    if len(lines) < 2:
        raise ConfigError(f"invalid data in well file: {path}")
    nwell = _int(_split(lines[1])[0])
    wells: List[Well] = []
    for n in range(nwell):
        toks = _split(lines[2 + n])
        ix, iy, iz, wpq = (_int(t) for t in toks[:4])
        wval, ph, c = (_num(t) for t in toks[4:7])
        if wpq == 1:
            wells.append(Well(ix, iy, iz, pressure=wval, injection=0.0, phase=ph, concent=c))
        elif wpq == -1:
            wells.append(Well(ix, iy, iz, pressure=0.0, injection=wval, phase=ph, concent=c))
        else:
            raise ConfigError(f"invalid data in well file: {path}")
    return wells


def load_config(path: str, extended: bool = True) -> Params:
    """Parse a ``.cfg`` file as ``loadConfig`` does (wPFAW3D.f90:264-505).

    Relative ``well``/``init`` paths are taken relative to the config file's
    directory (the reference resolves them against its working directory; the
    driver runs from there).
    """
    p = Params()
    try:
        with open(path, "r") as fh:
            text = fh.read().splitlines()
    except OSError as e:
        raise ConfigError(f"can not open config file: {path}") from e
    dxw = 0.0
    for raw in text:
        buf = raw
        if buf[:1] == "#":
            continue
        i = buf.find("#")
        if i >= 0:
            buf = buf[:i]
        if not buf.strip():
            continue
        i = buf.find("=")
        if i >= 0:
            buf = buf[:i] + " " + buf[i + 1:]
        toks = _split(buf)
        key, args = toks[0], toks[1:]
        try:
            if key == "grid":
                p.nx, p.ny, p.nz = (_int(t) for t in args[:3])
            elif key == "dt":
                p.dtime = _num(args[0])
            elif key == "tfac":
                p.tfac = _num(args[0])
            elif key == "time_total":
                p.time_total = _num(args[0])
            elif key == "gid_output":
                p.n_res_out = _int(args[0])
            elif key == "scr_output":
                p.n_dat_out = _int(args[0])
            elif key == "w":
                p.epsilon = _num(args[0])
            elif key == "dxw":
                dxw = _num(args[0])
            elif key == "lambda":
                p.lambda_ = _num(args[0])
            elif key == "poro":
                p.porosity = _num(args[0])
            elif key == "rhos":
                p.rhos = _num(args[0])
            elif key == "rhoa":
                p.rhoa = _num(args[0])
            elif key == "visco":
                p.viscosity = _num(args[0])
            elif key == "cwtp":
                p.cwtp = _num(args[0])
            elif key == "D":
                p.diffusion = _num(args[0])
            elif key == "b100":
                p.b100 = _num(args[0])
            elif key == "ral":
                p.ral = _num(args[0])
            elif key == "rat":
                p.rat = _num(args[0])
            elif key == "kwh":
                p.permeab_hole = _num(args[0])
            elif key == "pini":
                p.pini = _num(args[0])
            elif key == "ref":
                p.ix_ref, p.iy_ref, p.iz_ref = (_int(t) for t in args[:3])
            elif key == "well":
                p.filename_well = args[0]
            elif key == "init":
                try:
                    p.init_permeab, p.init_phase, p.init_concent = (_num(t) for t in args[:3])
                    if len(args) < 3:
                        raise ValueError
                except ValueError:
                    p.filename_init = args[0]
            elif key == "last":
                p.filename_last = args[0]
            elif extended and key == "nsteps":
                p.nsteps = _int(args[0])
            elif extended and key == "solver":
                p.solver = args[0]
            else:
                raise ConfigError(f"unknown key in config file: {path}: {key}")
        except (IndexError, ValueError) as e:
            raise ConfigError(f"broken line in config file: {path}: {raw.strip()}") from e
    p.dxw = dxw
    derive(p)
    if p.tfac is None:
        raise ConfigError("tfac is required (the reference leaves it uninitialised)")
    base = os.path.dirname(os.path.abspath(path))
    wf = p.filename_well if os.path.isabs(p.filename_well) else os.path.join(base, p.filename_well)
    p.wells = read_well_file(wf)
    if p.filename_init and not os.path.isabs(p.filename_init):
        p.filename_init = os.path.join(base, p.filename_init)
    return p


def load_input(path: str) -> Params:
    """Parse a legacy ``.inp`` file as ``loadInput`` does (wPFAW3D.f90:110-259):
    a fixed sequence of comment records and list-directed reads (a read that
    finds too few values on its record continues on the next ones), the wells
    inline, then the uniform initial K, phase and concentration."""
    try:
        with open(path, "r") as fh:
            lines = fh.read().splitlines()
    except OSError as e:
        raise ConfigError(f"can not open input file: {path}") from e
    pos = 0

    def skip(n):
        nonlocal pos
        pos += n

    def read(n):
        nonlocal pos
        out = []
        while len(out) < n:
            if pos >= len(lines):
                raise ConfigError(f"invalid data in input file: {path}")
            out += _split(lines[pos])
            pos += 1
        return out[:n]

    p = Params()
    try:
        skip(5)
        p.nx, p.ny, p.nz = (_int(t) for t in read(3))
        skip(1)
        a = read(2)
        p.dtime, p.tfac = _num(a[0]), _num(a[1])
        skip(1)
        a = read(4)
        p.time_start, p.time_end = _num(a[0]), _num(a[1])
        p.n_res_out, p.n_dat_out = _int(a[2]), _int(a[3])
        skip(2)
        a = read(2)
        p.epsilon, dxw = _num(a[0]), _num(a[1])
        skip(1)
        p.lambda_ = _num(read(1)[0])
        skip(2)
        p.porosity = _num(read(1)[0])
        skip(1)
        p.rhos, p.rhoa = (_num(t) for t in read(2))
        skip(1)
        p.viscosity = _num(read(1)[0])
        skip(1)
        p.cwtp = _num(read(1)[0])
        skip(1)
        p.diffusion = _num(read(1)[0])
        skip(2)
        p.b100 = _num(read(1)[0])
        skip(1)
        p.ral, p.rat = (_num(t) for t in read(2))
        skip(1)
        p.permeab_hole = _num(read(1)[0])
        skip(1)
        p.pini = _num(read(1)[0])
        skip(1)
        p.ix_ref, p.iy_ref, p.iz_ref = (_int(t) for t in read(3))
        skip(2)
        for _ in range(_int(read(1)[0])):
            t = read(7)
            ix, iy, iz, wpq = (_int(x) for x in t[:4])
            wval, ph, c = (_num(x) for x in t[4:7])
            if wpq == 1:
                p.wells.append(Well(ix, iy, iz, pressure=wval, injection=0.0, phase=ph, concent=c))
            elif wpq == -1:
                p.wells.append(Well(ix, iy, iz, pressure=0.0, injection=wval, phase=ph, concent=c))
            else:
                raise ConfigError(f"invalid well data in input file: {path}")
        skip(2)
        p.init_permeab = _num(read(1)[0])
        skip(1)
        p.init_phase = _num(read(1)[0])
        skip(1)
        p.init_concent = _num(read(1)[0])
    except (IndexError, ValueError) as e:
        raise ConfigError(f"invalid data in input file: {path}") from e
    p.time_total = p.time_end - p.time_start
    p.dxw = dxw
    derive(p)
    return p


def write_input(path: str, p: Params) -> None:
    """A legacy ``.inp`` file that load_input / loadInput read back as ``p``."""
    L = ["# wPFAW3D input", "#", "#", "#", "# grid nx ny nz", f"{p.nx} {p.ny} {p.nz}",
         "# dt tfac", f"{p.dtime!r} {p.tfac!r}",
         "# time_start time_end n_res n_dat", f"{p.time_start!r} {p.time_end!r} {p.n_res_out} {p.n_dat_out}",
         "# phase field", "# w dxw", f"{p.epsilon!r} {p.dxw!r}", "# lambda", f"{p.lambda_!r}",
         "# rock and fluid", "# poro", f"{p.porosity!r}", "# rhos rhoa", f"{p.rhos!r} {p.rhoa!r}",
         "# visco", f"{p.viscosity!r}", "# cwtp", f"{p.cwtp!r}", "# D", f"{p.diffusion!r}",
         "# reaction", "# b100", f"{p.b100!r}", "# ral rat", f"{p.ral!r} {p.rat!r}",
         "# kwh", f"{p.permeab_hole!r}", "# pini", f"{p.pini!r}", "# ref", f"{p.ix_ref} {p.iy_ref} {p.iz_ref}",
         "# wells", "# nwell", f"{len(p.wells)}"]
    for w in p.wells:
        wpq, wval = (1, w.pressure) if (w.pressure != 0.0 or w.injection == 0.0) else (-1, w.injection)
        L.append(f"{w.ix} {w.iy} {w.iz} {wpq} {wval!r} {w.phase!r} {w.concent!r}")
    L += ["# initial fields", "# K", f"{p.init_permeab!r}", "# phase", f"{p.init_phase!r}", "# concent",
          f"{p.init_concent!r}"]
    with open(path, "w") as fh:
        fh.write("\n".join(L) + "\n")


def write_well_file(path: str, wells: Sequence[Well]) -> None:
    with open(path, "w") as fh:
        fh.write("# ix iy iz wpq wval phase concent\n")
        fh.write(f"{len(wells)}\n")
        for w in wells:
            if w.pressure != 0.0 or w.injection == 0.0:
                wpq, wval = 1, w.pressure
            else:
                wpq, wval = -1, w.injection
            fh.write(f"{w.ix} {w.iy} {w.iz} {wpq} {wval!r} {w.phase!r} {w.concent!r}\n")


def write_config(path: str, p: Params, well_file: str, init_file: Optional[str] = None,
                 extended: bool = False) -> None:
    """Write a reference-clean ``.cfg`` (plus optional extension keys)."""
    lines = [
        f"grid = {p.nx} {p.ny} {p.nz}",
        f"dt = {p.dtime!r}",
        f"tfac = {p.tfac!r}",
        f"time_total = {p.time_total!r}",
        f"gid_output = {p.n_res_out}",
        f"scr_output = {p.n_dat_out}",
        f"w = {p.epsilon!r}",
        f"dxw = {p.dxw!r}",
        f"lambda = {p.lambda_!r}",
        f"poro = {p.porosity!r}",
        f"rhos = {p.rhos!r}",
        f"rhoa = {p.rhoa!r}",
        f"visco = {p.viscosity!r}",
        f"cwtp = {p.cwtp!r}",
        f"D = {p.diffusion!r}",
        f"b100 = {p.b100!r}",
        f"ral = {p.ral!r}",
        f"rat = {p.rat!r}",
        f"kwh = {p.permeab_hole!r}",
        f"pini = {p.pini!r}",
        f"ref = {p.ix_ref} {p.iy_ref} {p.iz_ref}",
        f"well = {well_file}",
    ]
    if init_file:
        lines.append(f"init = {init_file}")
    else:
        lines.append(f"init = {p.init_permeab!r} {p.init_phase!r} {p.init_concent!r}")
    if p.filename_last:
        lines.append(f"last = {p.filename_last}")
    if extended and p.nsteps is not None:
        lines.append(f"nsteps = {p.nsteps}")
    if extended and p.solver is not None:
        lines.append(f"solver = {p.solver}")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
