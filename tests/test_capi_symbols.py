"""The C-ABI library builds for sm_103a here (nvcc cross-compiles), loads, and
exports every entry point include/*.h declares.  No compute calls: there is
no GPU in this container, so only the failure path of wpf_create is called."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            txt = re.sub(r"/\*.*?\*/", "", open(os.path.join(inc, f)).read(), flags=re.S)
            names |= set(re.findall(r"\b(wpf_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_header_declares_the_reference_routines():
    names = _declared()
    for n in ("wpf_calc_permeability", "wpf_solve_pressure", "wpf_calc_velocity",
              "wpf_calc_phase_deriv", "wpf_calc_concent_deriv", "wpf_evolve_phase",
              "wpf_evolve_concent", "wpf_step", "wpf_reduce", "wpf_upload", "wpf_download"):
        assert n in names


def test_library_exports_every_symbol():
    from mizuho_edit_gb300 import build, capi
    path = build.build()
    L = C.CDLL(path)
    for n in _declared():
        assert hasattr(L, n), n
        assert n in capi.SIGNATURES, n


def test_no_device_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from mizuho_edit_gb300 import capi
    from mizuho_edit_gb300.cases import make_case
    from mizuho_edit_gb300.sim import Simulation
    case = make_case((4, 4, 4))
    with pytest.raises(capi.WpfError) as e:
        Simulation(case.params, case.permeab_rock, case.phase, case.concent)
    assert e.value.status == capi.WPF_ERR_CUDA
