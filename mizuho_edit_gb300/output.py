"""The reference's two output files, written from the device state.

* ``.dat`` progress file -- ``showProgress`` / ``doneProgress``
  (wPFAW3D.f90:1665-1836): the input summary, then one row per call
  (itime, time, injected pore volumes, inlet pressure, wormhole length,
  injected acid, dissolved CaCO3 from the acid balance and from the phase
  field), then the CPU / wall times.  The reductions come from the device
  (``wpf_reduce``); the row layout follows the reference's Fortran formats.
* GiD binary ``.res`` file -- ``saveResult`` (wPFAW3D.f90:1842-2091): the
  hexahedral mesh once, then per call four cell-centred results (pressure,
  phase field, concentration, permeability) in single precision.  The fields
  come from ``wpf_snapshot`` -- packed on the device and copied to pinned
  memory on a side stream while the simulation keeps stepping -- and a
  background thread writes them.
"""
from __future__ import annotations

import ctypes as C
import struct
import threading
import time as _time

import numpy as np

from . import capi


# ---- Fortran edit descriptors ------------------------------------------------------------
def fes(v: float, w: int, d: int) -> str:
    """ESw.d: one digit before the point; a three-digit exponent drops the 'E'."""
    s = format(float(v), f".{d}E")
    mant, exp = s.split("E")
    e = int(exp)
    es = f"E{e:+03d}" if abs(e) < 100 else f"{e:+04d}"
    out = mant + es
    return out.rjust(w) if len(out) <= w else "*" * w


def ff(v: float, w: int, d: int) -> str:
    s = format(float(v), f".{d}f")
    return s.rjust(w) if len(s) <= w else "*" * w


def fi(v: int, w: int) -> str:
    s = str(int(v))
    return s.rjust(w) if len(s) <= w else "*" * w


class ProgressWriter:
    """``showProgress`` to a ``.dat`` file (and, like the reference, a console
    table when ``echo``)."""

    def __init__(self, path: str, params, echo: bool = False):
        self.path, self.p, self.echo = path, params, echo
        self.fh = None
        self.pv = None
        self.t0 = self.c0 = None

    def _w(self, line: str = ""):
        self.fh.write(line + "\n")

    def _out(self, line: str):
        if self.echo:
            print(line)

    def first(self, diag: dict):
        p = self.p
        self.fh = open(self.path, "w")
        self.t0, self.c0 = _time.perf_counter(), _time.process_time()
        self.pv = diag["pv"]
        xchl = p.cwtp * p.b100 * p.rhoa / p.rhos
        b = p.rhoa / p.rhos
        kc = p.cwtp * p.b100 / (1.0 - p.porosity)
        w = self._w
        w(" ***** CALCULATION SUMMARY FOR PFACID PROGRAM *****")
        w(" /// Input data ///")
        w(" *** Grid data")
        w("   Num of grids, nx,ny,nz =" + fi(p.nx, 6) + fi(p.ny, 6) + fi(p.nz, 6))
        w("   Grid size, dx       =" + fes(p.dx, 14, 6) + " [m]")
        w("   Core length, Lx, Ly, Lz =" + ff(p.lx, 10, 4) + ff(p.ly, 10, 4) + ff(p.lz, 10, 4) + " [m]")
        w(" *** Rock and fluid data")
        w("   acid con., cwtp      =" + ff(p.cwtp, 12, 4) + " [kg HCl/kg solution]")
        w("   acid density, rhoa   =" + ff(p.rhoa, 12, 1) + " [kg/m3]")
        w("   rock density, rhos   =" + ff(p.rhos, 12, 1) + " [kg/m3]")
        w("   viscosity, visco     =" + fes(p.viscosity, 14, 6) + " [Pa*s]")
        w("   rock porosity, poro  =" + ff(p.porosity, 12, 6) + " [dec]")
        w("   diffusivity coef. ,d =" + fes(p.diffusion, 12, 4) + " [m2/s]")
        w("   gravimetric dissolving power, b100 =" + ff(p.b100, 8, 3) + " [kg CaCO3/kg HCl]")
        w("   volumetric dissolving power, Xacid =" + ff(xchl, 8, 3) + " [m3 CaCO3/m3 HCl]")
        w(" *** Phase-field related parameters")
        w("   lambda =" + ff(p.lambda_, 12, 6) + " [-]")
        w("   kc     =" + ff(kc, 12, 6) + " [-]")
        w("   b      =" + ff(b, 12, 6) + " [-]")
        w("   alpha  =" + ff(p.alpha, 12, 6) + " [-]")
        w(" *** Injection data")
        w("   time step size, dt     =" + fes(p.dtime, 12, 4) + " [s]")
        w("   initial pressure, pini =" + fes(p.pini, 12, 4) + " [m/s]")
        w(" pore volume =" + fes(self.pv, 20, 6) + " [m3]")
        w()
        w()
        w("/// SIMULATION RESULTS ///")
        w(" " * 13 + "ITIME" + " " * 2 + "TIME" + " " * 15 + "PVINJ" + " " * 13 + "WELL_PRESS" + " " * 10 +
          "WH_LENGTH" + " " * 10 + "INJ_ACID" + " " * 11 + "DISSOLVED_CaCO3" + " " * 10 + "DISS.CaCO3_c")
        w(" " * 13 + "(-)" + " " * 4 + "(sec)" + " " * 15 + "(v/v)" + " " * 15 + "(Pa)" + " " * 16 + "(m)" +
          " " * 14 + "(m3/m)" + " " * 14 + "(m3/m)" + " " * 14 + "(m3/m)")
        w(" " * 5 + "-----" + " " * 2 + "   --------------   " * 6)
        self._out("*** 3D Phase-Field Acid Wormholing Model, wPFAW3D ***")

    def write(self, diag: dict, time: float, itime: int, pinj: float):
        """One showProgress call (diag = Simulation.diagnostics())."""
        p = self.p
        if self.fh is None:
            self.first(diag)
        xchl = p.cwtp * p.b100 * p.rhoa / p.rhos
        qinj = sum(w.injection for w in p.wells if w.injection != 0.0)
        vacid = qinj * time
        vcaco3 = qinj * time * xchl
        row = " " + fi(itime, 8) + " " + "".join(fes(v, 20, 10) for v in (
            time, vacid / self.pv, pinj, diag["rwhmax"], vacid, vcaco3, diag["vcal"]))
        self._w(row)
        self.fh.flush()
        self._out(fi(itime, 8) + fes(time, 13, 5) + fes(vacid / self.pv, 11, 3) + " " +
                  "".join(ff(diag[k], 8, 3) for k in ("phase_max", "phase_min", "concent_max",
                                                       "concent_min")) +
                  fes(pinj, 13, 5) + fes(diag["rwhmax"], 12, 4) + fes(p.dtime, 10, 2))

    def close(self):
        """doneProgress: CPU and wall-clock minutes."""
        if self.fh is None:
            return
        cpu = (_time.process_time() - self.c0) / 60.0
        wall = (_time.perf_counter() - self.t0) / 60.0
        self._w()
        self._w("CPU time =" + fes(cpu, 12, 4) + " [min]")
        self._w("Cal time =" + fes(wall, 12, 4) + " [min]")
        self.fh.close()
        self.fh = None


# ---- GiD binary result file ------------------------------------------------------------------
def _gid_string(s: str) -> bytes:
    b = s.rstrip().encode() + b"\0"
    return struct.pack("<i", len(b)) + b


def gid_mesh(p) -> bytes:
    """Byte-order check, header and the hexahedral mesh (nodes and elements,
    1-based indices with x fastest), as saveResult's first call writes them."""
    nx, ny, nz, dx = p.nx, p.ny, p.nz, p.dx
    out = [struct.pack("<i", 0x091D), _gid_string("GiDPostEx1.1"),
           _gid_string('MESH "quadmesh" dimension 3 ElemType Hexahedra Nnode 8'),
           _gid_string("# color 0.7 0.7 0.4"), _gid_string('Unit "m"'),
           _gid_string("Coordinates -1 Indexed")]
    node = np.dtype([("i", "<i4"), ("x", "<f4"), ("y", "<f4"), ("z", "<f4")])
    iz, iy, ix = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    nodes = np.empty(ix.size, node)
    nodes["i"] = (ix + iy * (nx + 1) + iz * (nx + 1) * (ny + 1) + 1).ravel()
    nodes["x"] = (ix * dx).astype(np.float32).ravel()
    nodes["y"] = (iy * dx).astype(np.float32).ravel()
    nodes["z"] = (iz * dx).astype(np.float32).ravel()
    out += [nodes.tobytes(), _gid_string("End Coordinates"), _gid_string("Elements -1 Indexed")]
    elem = np.dtype([("i", "<i4"), ("n", "<i4", (8,)), ("c", "<i4")])
    ez, ey, ex = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    m = lambda a, b, c: (a + b * (nx + 1) + c * (nx + 1) * (ny + 1) + 1)
    els = np.empty(ex.size, elem)
    els["i"] = (ex + ey * nx + ez * nx * ny + 1).ravel()
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    for q, (a, b, c) in enumerate(corners):
        els["n"][:, q] = m(ex + a, ey + b, ez + c).ravel()
    els["c"] = 1
    out += [els.tobytes(), _gid_string("End Elements"),
            _gid_string('GaussPoints "Cell_Center" ElemType Hexahedra'),
            _gid_string("Number Of Gauss Points: 1"), _gid_string("Natural Coordinates: Given"),
            np.zeros(3, "<f4").tobytes(), _gid_string("End GaussPoints")]
    return b"".join(out)


_RESULTS = (("Pressure", "Pa"), ("Phase-field", "-"), ("Concentration", "-"), ("Permeability", "-"))


def gid_results(time: float, fields: np.ndarray) -> bytes:
    """The four result blocks of one saveResult call; fields = (4, N) float32
    (interior cells, Fortran order)."""
    n = fields.shape[1]
    rec = np.dtype([("i", "<i4"), ("v", "<f4")])
    out = []
    for (name, unit), vals in zip(_RESULTS, fields):
        out.append(_gid_string(f'Result "{name}" "Analysis" {fes(time, 12, 5)} Scalar OnGaussPoints '
                               f'"Cell_Center"'))
        out.append(_gid_string(f'Unit "{unit}"'))
        out.append(_gid_string("Values -1 Indexed"))
        r = np.empty(n, rec)
        r["i"] = np.arange(1, n + 1, dtype=np.int32)
        r["v"] = vals
        out.append(r.tobytes())
        out.append(struct.pack("<i", -1))
        out.append(_gid_string("End Values"))
    return b"".join(out)


class GiDWriter:
    """saveResult to a GiD binary .res file, fed by asynchronous snapshots."""

    def __init__(self, path: str, sim):
        self.path, self.sim = path, sim
        p = sim.params
        self.n = p.nx * p.ny * p.nz
        ptr = C.c_void_p()
        capi.check(sim.L.wpf_host_alloc(4 * 4 * self.n, C.byref(ptr)), "wpf_host_alloc")
        self.ptr = ptr
        self.buf = np.ctypeslib.as_array((C.c_float * (4 * self.n)).from_address(ptr.value)).reshape(4, self.n)
        self.thread = None
        self.error = None
        with open(path, "wb") as fh:
            fh.write(gid_mesh(p))

    def _finish(self, time: float):
        try:
            capi.check(self.sim.L.wpf_snapshot_wait(self.sim.h), "wpf_snapshot_wait")
            with open(self.path, "ab") as fh:
                fh.write(gid_results(time, self.buf))
        except Exception as e:   # reported by the next write / close
            self.error = e

    def write(self, time: float):
        """Queue one saveResult: the copy runs on the device's side stream and
        the file write in a thread; the caller may keep stepping."""
        self.join()
        capi.check(self.sim.L.wpf_snapshot(self.sim.h, self.ptr), "wpf_snapshot")
        self.thread = threading.Thread(target=self._finish, args=(time,), daemon=True)
        self.thread.start()

    def join(self):
        if self.thread is not None:
            self.thread.join()
            self.thread = None
        if self.error is not None:
            e, self.error = self.error, None
            raise e

    def close(self):
        self.join()
        if self.ptr:
            self.sim.L.wpf_host_free(self.ptr)
            self.ptr = None


def read_gid(path: str):
    """Parse a GiD binary .res written by GiDWriter / saveResult: returns the
    node and element arrays and a list of (name, time, values)."""
    data = open(path, "rb").read()
    pos = 0

    def i32():
        nonlocal pos
        v = struct.unpack_from("<i", data, pos)[0]
        pos += 4
        return v

    def string():
        nonlocal pos
        n = i32()
        s = data[pos:pos + n - 1].decode()
        pos += n
        return s

    assert i32() == 0x091D
    head = [string() for _ in range(5)]
    assert head[0] == "GiDPostEx1.1" and head[4] == "Coordinates -1 Indexed"
    nodes, elems, results = [], [], []
    # nodes until the "End Coordinates" string record
    node = np.dtype([("i", "<i4"), ("x", "<f4"), ("y", "<f4"), ("z", "<f4")])
    end = data.find(b"End Coordinates\0", pos) - 4
    nodes = np.frombuffer(data[pos:end], node)
    pos = end
    assert string() == "End Coordinates" and string() == "Elements -1 Indexed"
    elem = np.dtype([("i", "<i4"), ("n", "<i4", (8,)), ("c", "<i4")])
    end = data.find(b"End Elements\0", pos) - 4
    elems = np.frombuffer(data[pos:end], elem)
    pos = end
    assert string() == "End Elements"
    for _ in range(3):
        string()
    pos += 12
    assert string() == "End GaussPoints"
    rec = np.dtype([("i", "<i4"), ("v", "<f4")])
    nel = len(elems)
    while pos < len(data):
        line = string()
        name = line.split('"')[1]
        tok = line.split('"Analysis"')[1].split()[0]
        t = float(tok) if "E" in tok else float(tok[:-4] + "E" + tok[-4:])
        string()
        string()
        vals = np.frombuffer(data[pos:pos + nel * 8], rec)
        pos += nel * 8
        assert i32() == -1 and string() == "End Values"
        results.append((name, t, vals))
    return nodes, elems, results
