"""Regenerate the oracle's breakthrough fixture tests/golden/breakthrough_64.json.

python tests/golden/make_breakthrough.py

The CPU oracle (the plain-C restatement of wPFAW3D.f90) runs the 64^3 case
of the first benchmark configuration (log-K variance 1, correlation length 4
cells, seed 2026, Pe 100, Da 10, kwh 20) until breakthrough: the first step
after which a cell of the plane ix = nx - ceil(2 w / dx) has phase > 0.  The
pore volumes injected are sum over steps of Q_in dt / pv, Q_in the inlet-face
flux of the step's velocity, pv the initial pore volume (wPFAW3D.f90:1695).
Every Darcy solve runs to a relative residual of 1e-12.  About 3500 steps:
10 minutes on 8 cores.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

import oracle as O  # noqa: E402
from mizuho_edit_gb300.cases import make_case  # noqa: E402

CASE = dict(n=64, log_var=1.0, corr_len=4.0, seed=2026)
MAX_STEPS = 20000


def run(case_kw=CASE, max_steps=MAX_STEPS, rtol=1e-12, log=print):
    O.build()
    O.set_threads(os.cpu_count() or 1)
    n = case_kw["n"]
    case = make_case((n, n, n), log_var=case_kw["log_var"], corr_len=case_kw["corr_len"],
                     seed=case_kw["seed"])
    s = O.OracleSim(case.params, case.permeab_rock, case.phase, case.concent)
    pv = s.diagnostics()["pv"]
    ix = s.breakthrough_plane()
    vin = 0.0
    t0 = time.time()
    for step in range(1, max_steps + 1):
        info = s.step(O.SOLVE_MGCG, rtol)
        if not info.converged:
            raise RuntimeError(f"oracle solve failed at step {step}")
        vin += s.inlet_flux() * s.dtime
        if step % 500 == 0:
            log(f"step {step}: PV_inj {vin / pv:.4f} max phase on ix={ix}: "
                f"{float(np.max(s.phase[ix, 1:-1, 1:-1])):.4f} ({time.time() - t0:.0f} s)")
        if float(np.max(s.phase[ix, 1:-1, 1:-1])) > 0.0:
            return {"case": case_kw, "rtol": rtol, "plane_ix": ix, "step": step, "time": s.time,
                    "pv_injected": vin / pv, "pv": pv}
    raise RuntimeError("no breakthrough within the step limit")


def main():
    res = run()
    with open(os.path.join(HERE, "breakthrough_64.json"), "w") as fh:
        json.dump(res, fh, indent=1)
        fh.write("\n")
    print(json.dumps(res))


if __name__ == "__main__":
    main()
