"""wpf_reduce_noalloc: the allocation-free showProgress diagnostics.

Some callers of this library cannot call cudaMalloc: code whose device memory
belongs to another runtime's pool allocator, and latency-critical code that
cannot take cudaMalloc's implicit synchronisation.  For them
wpf_reduce_noalloc computes the diagnostics from device arrays they already
hold, with a fixed file-scope scratch.  The test holds the fields in device
memory through PyTorch (the caller's allocator here) and checks two calls in
a row against wpf_reduce, the handle-based entry point, and against the CPU
oracle's showProgress reductions (wPFAW3D.f90:1695, 1756-1810), on the
default stream and on a stream of the caller's; a warm call leaves the
device's free memory unchanged.

pytest collects this file last (its name sorts after the others), so that a
run stopping at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("pv", "vcal", "rwhmax", "phase_max", "phase_min", "concent_max", "concent_min")


def _state():
    from mizuho_edit_gb300.cases import grf, make_case
    case = make_case((40, 24, 18), seed=31, log_var=1.0, corr_len=3.0)
    p = case.params
    ph = np.tanh(1.5 * grf((p.nx, p.ny, p.nz), 2.0, 32))
    ph = np.where(ph > 0, ph * 1.05, ph)        # some |phase| > 1 cells
    cc = np.clip(0.5 + 0.5 * grf((p.nx, p.ny, p.nz), 3.0, 33), 0, 1)
    case.phase, case.concent = ph, cc
    return case


def _params(p):
    from mizuho_edit_gb300 import capi
    return capi.Params(p.nx, p.ny, p.nz, p.ix_ref, p.iy_ref, p.iz_ref, p.dx, p.epsilon,
                       p.lambda_, p.porosity, p.viscosity, p.diffusion, p.ral, p.rat,
                       p.permeab_hole, p.alpha, p.tfac)


def test_noalloc_matches_reduce_and_oracle_twice(oracle_mod):
    import torch
    from mizuho_edit_gb300 import capi
    from mizuho_edit_gb300.sim import Simulation
    case = _state()
    p = case.params
    with Simulation(p, case.permeab_rock, case.phase, case.concent) as sim:
        ref = sim.diagnostics()
        f = sim.download("phase", "concent")
    orc = oracle_mod.OracleSim(p, case.permeab_rock, case.phase, case.concent).diagnostics()
    L = capi.load()
    dev_ph = torch.from_numpy(np.ascontiguousarray(f["phase"].ravel(order="F"))).cuda()
    dev_cc = torch.from_numpy(np.ascontiguousarray(f["concent"].ravel(order="F"))).cuda()
    torch.cuda.synchronize()
    cp = _params(p)
    side = torch.cuda.Stream()
    for stream in (None, C.c_void_p(side.cuda_stream)):
        for _ in range(2):
            d = capi.Diag()
            st = L.wpf_reduce_noalloc(C.byref(cp), C.c_void_p(dev_ph.data_ptr()),
                                      C.c_void_p(dev_cc.data_ptr()), C.byref(d), stream)
            assert st == capi.WPF_OK, capi.strerror(st)
            got = d.as_dict()
            for k in KEYS:
                assert got[k] == pytest.approx(ref[k], rel=1e-13, abs=1e-13), k
                assert got[k] == pytest.approx(orc[k], rel=1e-13, abs=1e-13), k


def test_noalloc_takes_no_device_memory():
    """A warm call takes no device memory: the free bytes the driver reports
    are the same before and after it."""
    import torch
    from mizuho_edit_gb300 import capi
    case = _state()
    p = case.params
    G = (p.nx + 2) * (p.ny + 2) * (p.nz + 2)
    dev_ph = torch.zeros(G, dtype=torch.float64, device="cuda")
    dev_cc = torch.zeros(G, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    L = capi.load()
    cp = _params(p)
    d = capi.Diag()
    args = (C.byref(cp), C.c_void_p(dev_ph.data_ptr()), C.c_void_p(dev_cc.data_ptr()), C.byref(d),
            None)
    assert L.wpf_reduce_noalloc(*args) == capi.WPF_OK          # warm: the set-up is done
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert L.wpf_reduce_noalloc(*args) == capi.WPF_OK
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert d.phase_max == 0.0 and d.pv == pytest.approx(p.dx ** 3 * p.porosity * 0.5 *
                                                        p.nx * p.ny * p.nz)


def test_noalloc_rejects_oversized_grid():
    from mizuho_edit_gb300 import capi
    case = _state()
    cp = _params(case.params)
    cp.nz = capi.NOALLOC_MAX_PLANES - 1          # nz + 2 planes exceed the scratch
    d = capi.Diag()
    st = capi.load().wpf_reduce_noalloc(C.byref(cp), None, None, C.byref(d), None)
    assert st == capi.WPF_ERR_TOO_LARGE
    assert "4096" in capi.strerror(st)
