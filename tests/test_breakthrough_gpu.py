"""Breakthrough in pore volumes injected: the GPU forms against the CPU
oracle on identical seeded inputs.

Breakthrough (no counterpart in the reference, whose showProgress cannot
report it under Dirichlet wells, qinj = 0 at wPFAW3D.f90:1784-1790) is the
first step after which a cell of the plane ix = nx - ceil(2 w / dx) has
phase > 0 (wpf_diag.phase_max_outlet).  The outlet wells pin phase = -1 on
ix = nx and the diffuse interface cannot cross that plane, so the dissolved
region's closest approach is about 2w cells; the plane next to the outlet
never reaches phase > 0.  The pore volumes injected are the sum over steps of
Q_in dt / pv, Q_in the inlet-face flux of the step's velocity
(wpf_diag.inlet_flux) and pv the initial pore volume (:1695).

* 64^3, the first benchmark configuration's case (log-K variance 1,
  correlation 4 cells): the plain FP64 form within 0.5 %, the FP32-refined
  form (extrapolated start, one graph launch per step) and the learned start
  within 1 % of the oracle's pore volumes at breakthrough, taken from the
  committed fixture tests/golden/breakthrough_64.json (made by
  tests/golden/make_breakthrough.py: ~3500 oracle steps, too long to rerun
  here).
* Front arrival on a small grid, oracle run in the test: the same measurement
  on the mid plane of a 24x12x12 domain.
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (24, 12, 12)
CASE = dict(da=100.0, seed=3, log_var=1.5, corr_len=3.0)
MAX_STEPS = 6000


def _case():
    from mizuho_edit_gb300.cases import make_case
    return make_case(SHAPE, **CASE)


def _oracle_arrival(oracle_mod, case):
    p = case.params
    ref = oracle_mod.OracleSim(p, case.permeab_rock, case.phase, case.concent)
    pv = ref.diagnostics()["pv"]
    x = p.nx // 2
    vin, q_prev = 0.0, 0.0
    for s in range(1, MAX_STEPS + 1):
        ref.step(oracle_mod.SOLVE_CG, 1e-12)
        q = float(ref.velocity[0, 1, 1:-1, 1:-1].sum()) * p.dx * p.dx   # u_x at the faces 1 -> 2
        vin += 0.5 * (q + q_prev) * ref.dtime
        q_prev = q
        if ref.phase[x, 1:-1, 1:-1].max() > 0.0:
            return s, vin / pv
    return None, vin / pv


def _gpu_arrival(case, **kw):
    from mizuho_edit_gb300.sim import Simulation
    p = case.params
    x = p.nx // 2
    with Simulation(p, case.permeab_rock, case.phase, case.concent, **kw) as sim:
        d = sim.diagnostics()
        pv = d["pv"]
        vin, q_prev = 0.0, d["inlet_flux"]
        for s in range(1, MAX_STEPS + 1):
            st = sim.step()
            d = sim.diagnostics()
            q = d["inlet_flux"]
            vin += 0.5 * (q + q_prev) * st.dtime
            q_prev = q
            if np.max(sim.download("phase")[x, 1:-1, 1:-1]) > 0.0:
                return s, vin / pv
    return None, vin / pv


def test_front_arrival_pore_volumes(oracle_mod):
    case = _case()
    s_ref, pv_ref = _oracle_arrival(oracle_mod, case)
    assert s_ref is not None, "the oracle's front did not reach the mid plane"
    s64, pv64 = _gpu_arrival(case, solver="fp64", rtol=1e-10)
    smx, pvmx = _gpu_arrival(case, solver="mixed", rtol=1e-8, extrapolate=True, step_graph=True,
                             w_from_level=3)
    assert s64 is not None and smx is not None
    print(f"front arrival at ix = nx/2: oracle step {s_ref} PV {pv_ref:.6f}; "
          f"GPU FP64 step {s64} PV {pv64:.6f}; GPU mixed step {smx} PV {pvmx:.6f}")
    assert abs(pv64 - pv_ref) <= 5e-3 * pv_ref, (s_ref, pv_ref, s64, pv64)
    assert abs(pvmx - pv_ref) <= 1e-2 * pv_ref, (s_ref, pv_ref, smx, pvmx)


GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "breakthrough_64.json")


def _gpu_breakthrough(case, max_steps, net_weights=None, **kw):
    from mizuho_edit_gb300 import learned
    from mizuho_edit_gb300.sim import Simulation
    p = case.params
    net = None
    with Simulation(p, case.permeab_rock, case.phase, case.concent, **kw) as sim:
        if net_weights:
            net = learned.WarmStartNet(p.nx // 2, p.ny // 2, p.nz // 2)
            net.set_params(learned.WarmStartNet.load_params(net_weights))
            learned.attach(sim, net)
        try:
            pv = sim.diagnostics()["pv"]
            vin, kept = 0.0, 0
            for s in range(1, max_steps + 1):
                st = sim.step()
                assert st.converged, s
                kept += st.warm_start == 2
                d = sim.diagnostics()
                vin += d["inlet_flux"] * st.dtime
                if d["phase_max_outlet"] > 0.0:
                    return s, vin / pv, kept
            return None, vin / pv, kept
        finally:
            if net is not None:
                learned.attach(sim, None)
                net.close()


def test_breakthrough_64cubed_against_oracle():
    from mizuho_edit_gb300 import learned
    from mizuho_edit_gb300.cases import make_case
    g = json.load(open(GOLDEN))
    c = g["case"]
    n = c["n"]
    case = make_case((n, n, n), log_var=c["log_var"], corr_len=c["corr_len"], seed=c["seed"])
    limit = g["step"] + 500
    s64, pv64, _ = _gpu_breakthrough(case, limit, solver="fp64", rtol=1e-12)
    smx, pvmx, _ = _gpu_breakthrough(case, limit, solver="mixed", rtol=1e-8, extrapolate=True,
                                     step_graph=True)
    sln, pvln, kept = _gpu_breakthrough(case, limit, net_weights=learned.DEFAULT_WEIGHTS,
                                        solver="mixed", rtol=1e-8, extrapolate=True, step_graph=True,
                                        net_always=True)
    print(f"breakthrough 64^3: oracle step {g['step']} PV {g['pv_injected']:.5f}; FP64 step {s64} "
          f"PV {pv64:.5f}; FP32-refined step {smx} PV {pvmx:.5f}; learned step {sln} PV {pvln:.5f} "
          f"(net start kept {kept} times)")
    assert s64 is not None and smx is not None and sln is not None
    ref = g["pv_injected"]
    assert abs(pv64 - ref) <= 5e-3 * ref
    assert abs(pvmx - ref) <= 1e-2 * ref
    assert abs(pvln - ref) <= 1e-2 * ref
    assert kept > 0
