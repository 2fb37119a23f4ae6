"""GPU against the CPU oracle at the sizes and lengths of the benchmark
configurations, every field compared: pressure, face velocity, phase field
and concentration (relative L2 over the halo arrays).

* 64^3, 200 steps, log-K variance 1, correlation length 4 cells: the plain
  FP64 form, the FP32-refined form (1e-8 Darcy residual, extrapolated start,
  one graph launch per step) and the same with the learned start (its
  correction evaluated at every solve), without and with its output as the
  PCG's one-vector coarse space.
* 128^3, 500 steps, log-K variance 2, correlation length 8 cells: the plain
  FP64 form against the FP32-refined form, both against the oracle.

The oracle solves every step's Darcy system to a relative residual of 1e-13
(multigrid-preconditioned CG on the system assembled as wPFAW3D.f90:629-936;
the converged pressure does not depend on that solver); the FP64 form runs
to the same 1e-13.  Accuracy targets, checked after 100 steps and again at
the end of the run: FP64 form -- pressure and velocity <= 1e-10, phase and
concentration <= 1e-9; FP32-refined and learned forms -- pressure <= 1e-6,
phase, concentration and velocity (the pressure's gradient, which a 1e-8
Darcy residual bounds less tightly) <= 1e-5.
The reference's loop body is wPFAW3D.f90:2226-2280.

Velocity is the reference's calcVelocity output, so the last step before
each comparison runs through the per-routine entry points (the fused step
computes face velocities on the fly and keeps none).
"""
import os

import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FP64_TOL = {"pressure": 1e-10, "velocity": 1e-10, "phase": 1e-9, "concent": 1e-9}
MIXED_TOL = {"pressure": 1e-6, "velocity": 1e-5, "phase": 1e-5, "concent": 1e-5}


def _forms(names):
    forms = {
        "fp64": dict(solver="fp64", rtol=1e-13),
        "mixed": dict(solver="mixed", rtol=1e-8, extrapolate=True, step_graph=True),
        # the net evaluated at every solve (not only inside its gate)
        "learned": dict(solver="mixed", rtol=1e-8, extrapolate=True, step_graph=True, net_always=True),
        "learned_coarse": dict(solver="mixed", rtol=1e-8, extrapolate=True, step_graph=True, net_always=True,
                               net_coarse=True),
    }
    return {k: forms[k] for k in names}


def _run(oracle_mod, n, log_var, corr_len, seed, steps, checks, names):
    """Step the oracle and every GPU form side by side from one seeded case;
    at each step in `checks` compare all four fields with the oracle."""
    from mizuho_edit_gb300 import learned
    from mizuho_edit_gb300.cases import make_case
    from mizuho_edit_gb300.sim import Simulation
    O = oracle_mod
    O.set_threads(os.cpu_count() or 1)
    case = make_case((n, n, n), log_var=log_var, corr_len=corr_len, seed=seed)
    p = case.params
    ref = O.OracleSim(p, case.permeab_rock, case.phase, case.concent)
    sims, nets = {}, []
    try:
        for name, kw in _forms(names).items():
            sims[name] = Simulation(p, case.permeab_rock, case.phase, case.concent, **kw)
            if name.startswith("learned"):
                net = learned.WarmStartNet(n // 2, n // 2, n // 2)
                net.set_params(learned.WarmStartNet.load_params(learned.DEFAULT_WEIGHTS))
                learned.attach(sims[name], net)
                nets.append(net)
        errs = {}
        net_kept = 0
        for s in range(1, steps + 1):
            info = ref.step(O.SOLVE_MGCG, 1e-13)
            assert info.converged, f"oracle solve failed at step {s}"
            for name, sim in sims.items():
                st = sim.step_unfused() if s in checks else sim.step()
                assert st.converged, f"{name}: solve did not converge at step {s}"
                net_kept += name.startswith("learned") and st.warm_start == 2
            if s in checks:
                for name, sim in sims.items():
                    assert sim.dtime == pytest.approx(ref.dtime, rel=1e-9), name
                    f = sim.download("pressure", "velocity", "phase", "concent")
                    errs[(name, s)] = {k: rel_l2(f[k], getattr(ref, k)) for k in f}
                    e = errs[(name, s)]
                    print(f"PARITY {n}^3 step {s} {name}: p {e['pressure']:.2e} "
                          f"u {e['velocity']:.2e} phi {e['phase']:.2e} c {e['concent']:.2e}")
        return errs, net_kept, ref.diagnostics(), {k: s.diagnostics() for k, s in sims.items()}
    finally:
        for name, sim in sims.items():
            if name.startswith("learned"):
                learned.attach(sim, None)
            sim.close()
        for net in nets:
            net.close()


def _check(errs, names, checks):
    for name in names:
        tol = FP64_TOL if name == "fp64" else MIXED_TOL
        for s in checks:
            for k, v in errs[(name, s)].items():
                assert v <= tol[k], f"{name} step {s}: {k} rel-L2 {v:.3e} > {tol[k]:.0e}"


def test_config_64cubed_200_steps(oracle_mod):
    """64^3, 200 steps (log-K variance 1, correlation 4 cells): FP64,
    FP32-refined and learned forms (start only, and start + coarse space)
    against the oracle after 100 and 200 steps."""
    names = ("fp64", "mixed", "learned", "learned_coarse")
    checks = (100, 200)
    errs, net_kept, rd, gd = _run(oracle_mod, 64, 1.0, 4.0, 2026, 200, checks, names)
    _check(errs, names, checks)
    # the learned start is exercised, not only attached
    assert net_kept > 0
    for name, d in gd.items():
        for k in ("pv", "vcal", "phase_max", "phase_min", "concent_max", "concent_min"):
            tol = 1e-9 if name == "fp64" else 1e-6
            assert d[k] == pytest.approx(rd[k], rel=tol, abs=1e-12), (name, k)


def test_config_128cubed_500_steps(oracle_mod):
    """128^3, 500 steps (log-K variance 2, correlation 8 cells): plain FP64
    against FP32-refined, both against the oracle after 100 and 500 steps."""
    names = ("fp64", "mixed")
    checks = (100, 500)
    errs, _, rd, gd = _run(oracle_mod, 128, 2.0, 8.0, 2027, 500, checks, names)
    _check(errs, names, checks)
    for name, d in gd.items():
        tol = 1e-9 if name == "fp64" else 1e-6
        for k in ("pv", "vcal"):
            assert d[k] == pytest.approx(rd[k], rel=tol), (name, k)
