"""The C++ host program (mizuho_edit_gb300/host/wpf_driver.cpp, the
reference's program main on the C ABI): its .cfg and legacy .inp readers
agree with the Python mirror (CPU, --dry-run), and on the GPU it runs a case
end to end -- .dat, GiD .res and the .fld restart -- with the same fields as
the Python driver of the same library."""
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import rel_l2
from mizuho_edit_gb300 import build, config
from mizuho_edit_gb300.cases import make_case


def _driver():
    build.build()
    return build.DRIVER_PATH


def _write_case(tmp_path, n=(16, 12, 10), seed=5):
    import pathlib
    tmp_path = pathlib.Path(tmp_path)
    case = make_case(n, seed=seed, log_var=1.0, corr_len=3.0)
    p = case.params
    p.time_total = 1000.0                  # --nsteps ends the run
    p.n_res_out, p.n_dat_out = 1000000, 4000   # a result block every step
    p.filename_last = "case.last.fld"
    config.write_well_file(str(tmp_path / "wells.dat"), p.wells)
    from mizuho_edit_gb300.fld import write_fld
    write_fld(str(tmp_path / "init.fld"), 0.0, case.permeab_rock, case.phase, case.concent)
    config.write_config(str(tmp_path / "case.cfg"), p, "wells.dat", "init.fld")
    return case, str(tmp_path / "case.cfg")


def _dry(path):
    r = subprocess.run([_driver(), path, "--dry-run"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return json.loads(r.stdout)


def _same(d, p):
    for k in ("nx", "ny", "nz", "dtime", "tfac", "time_total", "n_res_out", "n_dat_out", "dtime_res",
              "dtime_dat", "epsilon", "dx", "lambda_", "porosity", "rhos", "rhoa", "viscosity", "cwtp",
              "diffusion", "b100", "ral", "rat", "permeab_hole", "alpha", "pini", "ix_ref", "iy_ref",
              "iz_ref"):
        assert d[k] == getattr(p, k), k
    assert len(d["wells"]) == len(p.wells)
    for a, w in zip(d["wells"], p.wells):
        assert a == [w.ix, w.iy, w.iz, w.pressure, w.injection, w.phase, w.concent]


def test_cfg_reader_matches_python(tmp_path):
    _, path = _write_case(tmp_path)
    d = _dry(path)
    p = config.load_config(path)
    _same(d, p)
    assert d["filename_init"].endswith("init.fld")


def test_inp_reader_matches_python(tmp_path):
    case = make_case((10, 8, 6), seed=2)
    p = case.params
    p.time_start, p.time_end, p.n_res_out, p.n_dat_out = 0.5, 3.0, 2, 5
    p.init_permeab, p.init_phase, p.init_concent = 2.5e-12, -1.0, 0.0
    path = str(tmp_path / "legacy.inp")
    config.write_input(path, p)
    q = config.load_input(path)
    d = _dry(path)
    _same(d, q)
    assert q.time_total == 2.5 and d["time_start"] == 0.5 and d["time_end"] == 3.0
    assert d["init_permeab"] == 2.5e-12 and q.wells[0].ix == p.wells[0].ix


def test_bad_inputs_fail_loudly(tmp_path):
    bad = tmp_path / "x.cfg"
    bad.write_text("grid = 4 4 4\nbogus = 1\n")
    r = subprocess.run([_driver(), str(bad), "--dry-run"], capture_output=True, text=True)
    assert r.returncode == 1 and "unknown key" in r.stderr
    r = subprocess.run([_driver(), str(tmp_path / "x.txt")], capture_output=True, text=True)
    assert r.returncode == 1 and "neither inp or cfg" in r.stderr


@pytest.mark.gpu
def test_driver_runs_a_case(tmp_path):
    from mizuho_edit_gb300 import output
    from mizuho_edit_gb300.fld import read_fld
    from mizuho_edit_gb300.sim import Simulation
    case, path = _write_case(tmp_path)
    r = subprocess.run([_driver(), path, "--nsteps", "12", "--quiet"], capture_output=True, text=True,
                       cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    dat = open(tmp_path / "case.dat").read().splitlines()
    assert dat[0].startswith(" ***** CALCULATION SUMMARY")
    assert dat[-2].startswith("CPU time =") and dat[-1].startswith("Cal time =")
    nodes, elems, res = output.read_gid(str(tmp_path / "case.res"))
    assert len(elems) == 16 * 12 * 10 and len(res) % 4 == 0 and len(res) >= 8
    last = read_fld(str(tmp_path / "case.last.fld"), expect_grid=(16, 12, 10))
    # the same steps through the Python mirror of the same library
    p = config.load_config(path)
    with Simulation(p, case.permeab_rock, case.phase, case.concent, solver="fp64", rtol=1e-8) as sim:
        for _ in range(12):
            sim.step()
        f = sim.download("phase", "concent", "pressure")
    assert rel_l2(last.phase, f["phase"][1:-1, 1:-1, 1:-1]) < 1e-10
    assert rel_l2(last.concent, f["concent"][1:-1, 1:-1, 1:-1]) < 1e-10
    assert np.isclose(last.time, sim.time)
    assert len(res) == 4 * 13                    # the initial call + one per step
    # the last .res block holds the final fields in single precision
    perm = [r for r in res if r[0] == "Phase-field"][-1][2]["v"]
    assert np.allclose(perm, f["phase"][1:-1, 1:-1, 1:-1].ravel(order="F").astype(np.float32))
    # the pressure side file: the halo pressure, then a 32-byte step trailer
    assert os.path.getsize(str(tmp_path / "case.last.fld.p")) == 8 * 18 * 14 * 12 + 32


@pytest.mark.gpu
def test_restart_resumes_the_run(tmp_path):
    """N steps, the restart field and its pressure side file (saveField,
    wPFAW3D.f90:2096-2141), a restart from them (loadField, :509-557) and M
    more steps give the fields of N + M continuous steps: same step count,
    time and step size, phase, concentration and pressure within 1e-12."""
    from mizuho_edit_gb300.fld import read_fld
    n, steps_a, steps_b = (16, 12, 10), 9, 7
    G = (n[0] + 2) * (n[1] + 2) * (n[2] + 2)

    def run(cfg, nsteps):
        r = subprocess.run([_driver(), cfg, "--nsteps", str(nsteps), "--rtol", "1e-13", "--quiet"],
                           capture_output=True, text=True, cwd=os.path.dirname(cfg))
        assert r.returncode == 0, r.stderr

    def side(path):
        raw = open(path, "rb").read()
        assert len(raw) == 8 * G + 32 and raw[8 * G:8 * G + 8] == b"WPFSTEP1"
        pr = np.frombuffer(raw[:8 * G], np.float64)
        itime, dt, taumin = np.frombuffer(raw[8 * G + 8:], np.float64)
        return pr, int(itime), dt, taumin

    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    _, cont = _write_case(tmp_path / "a", n)
    run(cont, steps_a + steps_b)
    _, first = _write_case(tmp_path / "b", n)
    run(first, steps_a)
    pr_a, it_a, _, _ = side(str(tmp_path / "b" / "case.last.fld.p"))
    assert it_a == steps_a
    p = config.load_config(first)
    p.filename_last = "case2.last.fld"
    config.write_config(str(tmp_path / "b" / "case2.cfg"), p, "wells.dat", "case.last.fld")
    run(str(tmp_path / "b" / "case2.cfg"), steps_b)
    want = read_fld(str(tmp_path / "a" / "case.last.fld"), expect_grid=n)
    got = read_fld(str(tmp_path / "b" / "case2.last.fld"), expect_grid=n)
    pw, itw, dtw, tmw = side(str(tmp_path / "a" / "case.last.fld.p"))
    pg, itg, dtg, tmg = side(str(tmp_path / "b" / "case2.last.fld.p"))
    assert itg == itw == steps_a + steps_b
    assert dtg == pytest.approx(dtw, rel=1e-12) and tmg == pytest.approx(tmw, rel=1e-12)
    assert got.time == pytest.approx(want.time, rel=1e-12)
    assert rel_l2(got.phase, want.phase) < 1e-12
    assert rel_l2(got.concent, want.concent) < 1e-12
    assert rel_l2(pg, pw) < 1e-12
