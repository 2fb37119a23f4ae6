"""The output writers (showProgress .dat, saveResult GiD .res) on the host:
Fortran edit descriptors, file structure and a GiD round trip."""
import numpy as np

from mizuho_edit_gb300 import output as O
from mizuho_edit_gb300.cases import make_case


def test_fortran_descriptors():
    assert O.fes(1.0, 20, 10) == "    1.0000000000E+00"
    assert O.fes(-0.000123456, 12, 4) == " -1.2346E-04"
    assert O.fes(0.0, 12, 5) == " 0.00000E+00"
    assert O.fes(1.5e123, 14, 6) == "  1.500000+123"    # three-digit exponent drops the E
    assert O.ff(3.14159, 8, 3) == "   3.142"
    assert O.ff(1e9, 6, 2) == "******"
    assert O.fi(42, 8) == "      42"


def test_progress_file_layout(tmp_path):
    case = make_case((8, 6, 4), seed=3)
    p = case.params
    path = str(tmp_path / "run.dat")
    w = O.ProgressWriter(path, p)
    d = dict(pv=1.5, vcal=2.5, rwhmax=0.75, phase_max=1.0, phase_min=-1.0, concent_max=1.0,
             concent_min=0.0, pressure_ref=1.0, inlet_flux=0.0)
    w.write(d, 0.0, 0, 1.0)
    w.write(d, 0.5, 5, 0.9)
    w.close()
    lines = open(path).read().split("\n")
    assert lines[0] == " ***** CALCULATION SUMMARY FOR PFACID PROGRAM *****"
    assert lines[3].startswith("   Num of grids, nx,ny,nz =") and lines[3].endswith("     8     6     4")
    i = lines.index("/// SIMULATION RESULTS ///")
    assert lines[i - 1] == "" and lines[i - 2] == ""
    rows = [l for l in lines[i + 4:] if l.startswith(" ") and len(l) == 1 + 8 + 1 + 7 * 20]
    assert len(rows) == 2
    f = rows[1].split()
    assert int(f[0]) == 5 and float(f[1]) == 0.5
    qinj = sum(wl.injection for wl in p.wells if wl.injection != 0.0)
    assert np.isclose(float(f[2]), qinj * 0.5 / 1.5)     # PVINJ = vacid / pv (first call's pv)
    assert np.isclose(float(f[7]), 2.5)                  # DISS.CaCO3_c = vcal
    assert lines[-3].startswith("CPU time =") and lines[-2].startswith("Cal time =")


def test_gid_round_trip(tmp_path):
    case = make_case((5, 4, 3), seed=4)
    p = case.params
    path = str(tmp_path / "run.res")
    with open(path, "wb") as fh:
        fh.write(O.gid_mesh(p))
        rng = np.random.default_rng(0)
        f1 = rng.standard_normal((4, 60)).astype(np.float32)
        f2 = rng.standard_normal((4, 60)).astype(np.float32)
        fh.write(O.gid_results(0.25, f1))
        fh.write(O.gid_results(1.5e-3, f2))
    nodes, elems, res = O.read_gid(path)
    assert len(nodes) == 6 * 5 * 4 and len(elems) == 60
    assert nodes["i"][0] == 1 and nodes["i"][-1] == 120
    assert np.isclose(nodes["x"][1], p.dx) and np.isclose(nodes["y"][6], p.dx)
    # element 1: nodes (1,1,1),(2,1,1),(2,2,1),(1,2,1),(1,1,2),...
    assert list(elems["n"][0]) == [1, 2, 8, 7, 31, 32, 38, 37]
    assert [r[0] for r in res] == ["Pressure", "Phase-field", "Concentration", "Permeability"] * 2
    assert np.isclose(res[0][1], 0.25) and np.isclose(res[4][1], 1.5e-3)
    assert np.array_equal(res[1][2]["v"], f1[1]) and np.array_equal(res[7][2]["v"], f2[3])
    assert list(res[0][2]["i"][:3]) == [1, 2, 3]
