"""Regenerate the golden oracle vectors under tests/golden/.

python tests/golden/make_golden.py

The fixture pins the CPU oracle (the plain-C restatement of wPFAW3D.f90) on a
seeded 12x10x8 wormholing case after 20 steps solved with the tight CG mode,
so that later edits of the oracle that change its results are caught.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

import oracle as O  # noqa: E402
from mizuho_edit_gb300.cases import make_case  # noqa: E402


def main():
    O.build()
    case = make_case((12, 10, 8), seed=1)
    s = O.OracleSim(case.params, case.permeab_rock, case.phase, case.concent)
    steps = 20
    for _ in range(steps):
        s.step(O.SOLVE_CG, 1e-14)
    np.savez_compressed(os.path.join(HERE, "oracle_12x10x8_s1.npz"), steps=steps,
                        permeab_rock=case.permeab_rock, pressure=s.pressure, phase=s.phase,
                        concent=s.concent, dtime=s.dtime, taumin=s.taumin)


if __name__ == "__main__":
    main()
