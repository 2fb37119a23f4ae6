"""The ensemble runner: members of uneven grids stepped together from a pool
of host threads give the same fields as stepping each member alone, and the
autotuner returns one of its candidates per shape."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_ensemble_matches_members_alone():
    from mizuho_edit_gb300 import capi, ensemble
    members = [((24, 20, 16), dict(log_var=1.0, corr_len=4.0, da=5.0, seed=1)),
               ((32, 32, 32), dict(log_var=2.0, corr_len=6.0, da=30.0, seed=2)),
               ((16, 16, 16), dict(log_var=0.5, corr_len=3.0, da=1.0, seed=3))]
    opts = ensemble._opts(ensemble.CANDIDATES[0])
    alone = []
    for shape, kw in members:
        with ensemble._sim(shape, kw, opts) as sim:
            for _ in range(6):
                sim.step()
            alone.append(sim.download("phase", "concent", "pressure"))
    sims = [ensemble._sim(shape, kw, opts) for shape, kw in members]
    try:
        L = sims[0].L
        n = len(sims)
        hs = (C.c_void_p * n)(*[s.h.value for s in sims])
        dt = (C.c_double * n)(*[s.dtime for s in sims])
        stats = (capi.StepStats * n)()
        status = (C.c_int32 * n)()
        capi.check(L.wpf_ensemble_run(hs, n, 1, 6, 2, dt, stats, status), "wpf_ensemble_run")
        assert list(status) == [0, 0, 0] and all(s.converged for s in stats)
        for s, ref in zip(sims, alone):
            got = s.download("phase", "concent", "pressure")
            for k in ("phase", "concent", "pressure"):
                assert rel_l2(got[k], ref[k]) < 1e-9, k
    finally:
        for s in sims:
            s.close()
    # argument checks
    assert L.wpf_ensemble_run(None, 1, 1, 1, 1, dt, None, None) == capi.WPF_ERR_ARG


def test_autotune_picks_a_candidate():
    from mizuho_edit_gb300 import ensemble
    members = ensemble.make_members((1, 0, 0), seed=7)
    best = ensemble.autotune(members, spinup=4, steps=2, log=lambda *a: None)
    (shape, (choice, times)), = best.items()
    assert shape == (64, 64, 64) and choice in ensemble.CANDIDATES
    assert set(times) == set(ensemble.CANDIDATES) and times[choice] == min(times.values())
