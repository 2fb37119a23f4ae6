"""Host transfers: a kernel reads or writes page-locked caller buffers in
place through their mapped address, 16-byte pairs when the array is aligned
and row by row when it is not (ordinary arrays in place when the device uses
the host page tables, else staged).  Every path must carry the halo arrays
bit for bit, and an upload of unchanged values must keep the incremental
state (the same steps follow as without the upload)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAMES = ("phase", "concent", "pressure")


def _case(shape=(40, 32, 24), seed=5):
    from mizuho_edit_gb300.cases import make_case
    return make_case(shape, seed=seed, log_var=2.0, corr_len=5.0, da=20.0)


def _sim(case, **kw):
    from mizuho_edit_gb300.sim import Simulation
    return Simulation(case.params, case.permeab_rock, case.phase, case.concent, **kw)


class Pinned:
    """Page-locked halo arrays from wpf_host_alloc, `offset` bytes into the
    allocation (8: not 16-byte aligned)."""

    def __init__(self, L, shape, n, offset=0):
        from mizuho_edit_gb300 import capi
        self.L, self.ptrs, self.arrays = L, [], []
        nbytes = int(np.prod(shape)) * 8
        for _ in range(n):
            p = C.c_void_p()
            capi.check(L.wpf_host_alloc(nbytes + 16, C.byref(p)), "wpf_host_alloc")
            self.ptrs.append(p)
            buf = (C.c_char * nbytes).from_address(p.value + offset)
            self.arrays.append(np.frombuffer(buf, dtype=np.float64).reshape(shape, order="F"))

    def dp(self, q):
        from mizuho_edit_gb300 import capi
        return self.arrays[q].ctypes.data_as(capi.DP)

    def free(self):
        self.arrays = []
        for p in self.ptrs:
            self.L.wpf_host_free(p)
        self.ptrs = []


@pytest.mark.parametrize("offset", [0, 8])
def test_pinned_roundtrip_bitwise(offset):
    from mizuho_edit_gb300 import capi
    case = _case()
    with _sim(case, solver="mixed", rtol=1e-8, extrapolate=True, step_graph=True) as sim:
        for _ in range(4):
            sim.step()
        ref = sim.download(*NAMES)
        pin = Pinned(sim.L, sim.halo_shape, 3, offset)
        try:
            for a in pin.arrays:
                a.fill(np.nan)
            capi.check(sim.L.wpf_download(sim.h, pin.dp(0), pin.dp(1), pin.dp(2), None, None, None, None),
                       "wpf_download")
            for q, n in enumerate(NAMES):
                assert np.array_equal(pin.arrays[q].view(np.int64), ref[n].view(np.int64)), n
            # new pressure values through the page-locked path, read back in place
            rng = np.random.default_rng(0)
            new_p = ref["pressure"] + rng.uniform(0.0, 1e-3, ref["pressure"].shape)
            pin.arrays[2][...] = new_p
            capi.check(sim.L.wpf_upload(sim.h, None, None, None, pin.dp(2)), "wpf_upload")
            got = sim.download("pressure")
            fixed = got != new_p   # the Dirichlet well cells keep their pressure
            assert fixed.sum() <= len(case.params.wells)
            assert np.array_equal(got[fixed], ref["pressure"][fixed])
            assert np.array_equal(got[~fixed].view(np.int64), new_p[~fixed].view(np.int64))
        finally:
            pin.free()


def test_pinned_unchanged_upload_keeps_state():
    """Download to page-locked buffers and upload them back before every step:
    the values are unchanged, so the incremental state (graph keys, kept
    residual, quiescent bricks, level-0 marks) stays and the steps are those
    of a run without transfers."""
    from mizuho_edit_gb300 import capi
    from conftest import rel_l2
    case = _case(seed=6)
    kw = dict(solver="mixed", rtol=1e-8, extrapolate=True, step_graph=True)
    with _sim(case, **kw) as sim:
        plain = [sim.step().as_dict() for _ in range(8)]
        f_plain = sim.download(*NAMES)
    with _sim(case, **kw) as sim:
        pin = Pinned(sim.L, sim.halo_shape, 3)
        try:
            io = []
            for s in range(8):
                if s >= 2:
                    capi.check(sim.L.wpf_download(sim.h, pin.dp(0), pin.dp(1), pin.dp(2), None, None, None,
                                                  None), "wpf_download")
                    capi.check(sim.L.wpf_upload(sim.h, None, pin.dp(0), pin.dp(1), pin.dp(2)), "wpf_upload")
                io.append(sim.step().as_dict())
            f_io = sim.download(*NAMES)
        finally:
            pin.free()
    for n in NAMES:
        assert rel_l2(f_io[n], f_plain[n]) <= 1e-11, n
    for a, b in zip(plain, io):
        for key in ("outer_iterations", "inner_iterations", "converged", "warm_start", "kernel_launches"):
            assert a[key] == b[key], (key, a[key], b[key])
