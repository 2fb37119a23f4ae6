"""Field restart file (``.fld``), byte-compatible with wPFAW3D.

Layout (``saveField`` wPFAW3D.f90:2096-2141, ``loadField`` :509-557):
a 32-byte header ``{char magic[8] = "wPFAWHFG", char version[8] = "20250304",
float64 time, int16 nx, ny, nz, pad}`` followed by three FP64 arrays over the
global interior grid in Fortran order (x fastest): ``permeab_rock``, ``phase``,
``concent`` (the body subarray of ``MPI__File_{read,write}_body``,
parallel.f90:300-320).  Native byte order, as the reference writes it.
"""
from __future__ import annotations

import dataclasses
import struct

import numpy as np

__all__ = ["FieldFile", "read_fld", "write_fld", "FldError", "MAGIC", "VERSION"]

MAGIC = b"wPFAWHFG"
VERSION = b"20250304"
_HEAD = struct.Struct("=8s8sdhhhh")


class FldError(ValueError):
    pass


@dataclasses.dataclass
class FieldFile:
    time: float
    permeab_rock: np.ndarray   # (nx, ny, nz) float64, Fortran order semantics
    phase: np.ndarray
    concent: np.ndarray

    @property
    def shape(self):
        return self.phase.shape


def write_fld(path: str, time: float, permeab_rock: np.ndarray, phase: np.ndarray,
              concent: np.ndarray) -> None:
    """Write interior arrays (shape (nx, ny, nz), index [ix-1, iy-1, iz-1])."""
    nx, ny, nz = phase.shape
    if max(nx, ny, nz) > 32767:
        raise FldError("grid does not fit the int16 header")
    with open(path, "wb") as fh:
        fh.write(_HEAD.pack(MAGIC, VERSION, float(time), nx, ny, nz, 0))
        for a in (permeab_rock, phase, concent):
            np.asarray(a, dtype=np.float64).ravel(order="F").tofile(fh)


def read_fld(path: str, expect_grid=None) -> FieldFile:
    """Read a ``.fld``; raise ``FldError`` on a bad magic or a grid mismatch
    (the reference's ``exit(1)`` cases, wPFAW3D.f90:526-545)."""
    try:
        fh = open(path, "rb")
    except OSError as e:
        raise FldError(f"can not open field file: {path}") from e
    with fh:
        raw = fh.read(_HEAD.size)
        if len(raw) != _HEAD.size:
            raise FldError(f"truncated field file: {path}")
        magic, _version, time, nx, ny, nz, _pad = _HEAD.unpack(raw)
        if magic != MAGIC:
            raise FldError(f"invalid magic in field file: {path}")
        if expect_grid is not None and tuple(expect_grid) != (nx, ny, nz):
            raise FldError(f"invalid grid in field file: {path}")
        n = nx * ny * nz
        body = np.fromfile(fh, dtype=np.float64, count=3 * n)
        if body.size != 3 * n:
            raise FldError(f"truncated field file: {path}")
    arrs = [body[m * n:(m + 1) * n].reshape((nx, ny, nz), order="F") for m in range(3)]
    return FieldFile(time, *arrs)
