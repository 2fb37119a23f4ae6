"""Host front end: .cfg / well-file parsing (loadConfig) and .fld I/O."""
import os

import numpy as np
import pytest

from mizuho_edit_gb300.cases import make_case, write_case
from mizuho_edit_gb300.config import ConfigError, load_config, read_well_file
from mizuho_edit_gb300.fld import FldError, read_fld, write_fld


def test_case_roundtrip(tmp_path):
    case = make_case((6, 5, 4), seed=2)
    cfg = write_case(case, str(tmp_path))
    p = load_config(cfg)
    q = case.params
    for k in ("nx", "ny", "nz", "dtime", "tfac", "epsilon", "dx", "lambda_", "porosity",
              "viscosity", "diffusion", "permeab_hole", "alpha", "ix_ref", "iy_ref", "iz_ref"):
        assert getattr(p, k) == getattr(q, k), k
    assert len(p.wells) == len(q.wells)
    assert p.wells[0] == q.wells[0] and p.wells[-1] == q.wells[-1]
    f = read_fld(p.filename_init, expect_grid=(6, 5, 4))
    assert np.array_equal(f.permeab_rock, case.permeab_rock)
    assert np.array_equal(f.phase, case.phase)


def test_fortran_number_syntax(tmp_path):
    (tmp_path / "w.txt").write_text("title\n2\n1 1 1 1 1.0d0 1.0 1.0\n3 2 1 -1 2.5D-3 -1.0 0.0\n")
    (tmp_path / "c.cfg").write_text(
        "# comment\ngrid = 3 2 1\ntfac=0.1  # trailing\nw 2.0\ndxw 0.5\nrhoa 1\nrhos 1\n"
        "cwtp 1\nb100 1\nporo 0.5\nD 1.0d-2\nvisco 1\nwell w.txt\n")
    p = load_config(str(tmp_path / "c.cfg"))
    assert p.diffusion == 0.01 and p.dx == 1.0 and p.tfac == 0.1
    assert p.wells[0].pressure == 1.0 and p.wells[1].injection == 2.5e-3
    assert p.wells[1].pressure == 0.0
    assert p.alpha == 0.5 / 1.0 / (1.0 * 1.0 / 0.5)


def test_unknown_key_rejected(tmp_path):
    (tmp_path / "c.cfg").write_text("grid 2 2 2\nbogus 1\n")
    with pytest.raises(ConfigError):
        load_config(str(tmp_path / "c.cfg"))
    (tmp_path / "d.cfg").write_text("nsteps 3\n")
    with pytest.raises(ConfigError):
        load_config(str(tmp_path / "d.cfg"), extended=False)


def test_tfac_required(tmp_path):
    (tmp_path / "w.txt").write_text("t\n0\n")
    (tmp_path / "c.cfg").write_text("grid 2 2 2\nw 2\ndxw 0.5\nrhoa 1\nrhos 1\ncwtp 1\nb100 1\n"
                                     "poro 0.5\nwell w.txt\n")
    with pytest.raises(ConfigError):
        load_config(str(tmp_path / "c.cfg"))


def test_bad_well_type(tmp_path):
    (tmp_path / "w.txt").write_text("t\n1\n1 1 1 2 1.0 1.0 1.0\n")
    with pytest.raises(ConfigError):
        read_well_file(str(tmp_path / "w.txt"))


def test_fld_roundtrip_and_errors(tmp_path):
    rng = np.random.default_rng(1)
    a, b, c = rng.random((3, 5, 4, 3))
    path = str(tmp_path / "x.fld")
    write_fld(path, 12.5, a, b, c)
    raw = open(path, "rb").read()
    assert raw[:16] == b"wPFAWHFG20250304" and len(raw) == 32 + 3 * 60 * 8
    f = read_fld(path, expect_grid=(5, 4, 3))
    assert f.time == 12.5 and np.array_equal(f.concent, c)
    # body is the Fortran-order interior (x fastest)
    body = np.frombuffer(raw[32:32 + 60 * 8], dtype=np.float64)
    assert body[1] == a[1, 0, 0] and body[5] == a[0, 1, 0]
    with pytest.raises(FldError):
        read_fld(path, expect_grid=(5, 4, 4))
    bad = str(tmp_path / "bad.fld")
    open(bad, "wb").write(b"XXXXXXXX" + raw[8:])
    with pytest.raises(FldError):
        read_fld(bad)


def test_grf_statistics():
    from mizuho_edit_gb300.cases import grf
    g = grf((32, 32, 32), 4.0, 5)
    assert abs(g.mean()) < 1e-12 and abs(g.std() - 1) < 1e-12
    assert np.array_equal(g, grf((32, 32, 32), 4.0, 5))
    # correlation decays with lag: strong at 1 cell, weak at 3 l
    c1 = np.mean(g * np.roll(g, 1, 0))
    c12 = np.mean(g * np.roll(g, 12, 0))
    assert c1 > 0.9 and abs(c12) < 0.3
