"""The learned warm start inside the solve: data generation from the simulator,
training on the GPU, and what the trained network gains over the
extrapolated start without it -- with every solve still finishing at the same
FP64 residual tolerance and the same answer."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _mods():
    from mizuho_edit_gb300 import learned
    from mizuho_edit_gb300.cases import make_case
    from mizuho_edit_gb300.sim import Simulation
    return learned, make_case, Simulation


def test_net_start_same_solution():
    """An attached (untrained) network changes only the start: 12 steps agree
    with the run without it to the solver tolerance, every solve converges."""
    learned, make_case, Simulation = _mods()
    case = make_case((32, 32, 32), log_var=2.0, corr_len=5.0, seed=31)
    out = {}
    for use in (False, True):
        net = learned.WarmStartNet(16, 16, 16, seed=3) if use else None
        with Simulation(case.params, case.permeab_rock, case.phase, case.concent, solver="mixed",
                        rtol=1e-8, extrapolate=True) as sim:
            learned.attach(sim, net)
            st = [sim.step() for _ in range(12)]
            learned.attach(sim, None)
            assert all(s.converged and s.relres <= 1e-8 for s in st)
            out[use] = (st, sim.download("pressure", "phase", "concent"))
        if net is not None:
            codes = [s.warm_start for s in st]
            # no history on the first solve; later: the net's start (2), the
            # extrapolation's (1) or, in the start-up transient, p itself (-1)
            assert codes[0] == 0 and set(codes[3:]) <= {-1, 1, 2}
            net.close()
    for k in ("pressure", "phase", "concent"):
        assert rel_l2(out[True][1][k], out[False][1][k]) < 1e-6, k


def test_trained_net_gains_over_extrapolation():
    """Train on pairs the simulator generates (6 seeded 128^3 runs; cosine
    schedule, the best held-out epoch kept), then on an unseen seed: the
    network predicts the extrapolation's error (held-out loss falls during
    training and ends well below that of predicting zero, which is the start
    without it), its start leaves a smaller initial residual than the
    extrapolation's, and the solves take no more PCG iterations."""
    import torch
    learned, make_case, Simulation = _mods()
    pairs = learned.generate(6, 128, 40, 10, seed0=500, log=lambda *a: None)
    held = learned.generate(1, 128, 12, 30, seed0=900, log=lambda *a: None)
    assert len(pairs) >= 200 and len(held) >= 10
    net = learned.WarmStartNet(64, 64, 64, seed=1)
    hist = learned.train(net, pairs, 6, 1e-3, log=lambda *a: None)
    assert hist["train"][-1] < hist["train"][0]
    assert min(hist["val"]) < hist["val"][0]
    out = torch.empty(64 ** 3, dtype=torch.float32, device="cuda")
    zero, err = [], []
    for x, t in held:
        net.forward(x, out)
        err.append(float(((out - t).double() ** 2).mean()))
        zero.append(float((t.double() ** 2).mean()))
    assert np.mean(err) < 0.5 * np.mean(zero)
    case = make_case((128, 128, 128), log_var=2.0, corr_len=8.0, seed=901)
    base = learned.evaluate(case, None, 10, 30)
    # the net evaluated at every solve (not only inside its gate), so that
    # every step measures its correction
    with_net = learned.evaluate(case, net, 10, 30, net_always=True)
    r_base = np.mean([s[0] for s in base])
    r_net = np.mean([s[0] for s in with_net])
    # the net's correction enters with the residual-minimising step (kept,
    # code 2, only when that step is positive), so the start never gets worse
    assert all(s[2] in (-1, 1, 2) for s in with_net)
    assert any(s[2] == 2 for s in with_net)
    assert r_net < r_base
    assert sum(s[1] for s in with_net) <= sum(s[1] for s in base)
    print(f"unseen seed: initial relative residual {r_base:.3e} -> {r_net:.3e} with the net; "
          f"PCG iterations {sum(s[1] for s in base)} -> {sum(s[1] for s in with_net)}")
    net.close()


def test_net_coarse_space():
    """WPF_SOLVER_NET_COARSE: in the solves where the learned correction is
    evaluated, its output w (predicted on the half-resolution grid and
    prolongated) also becomes the one-vector coarse space of a deflated PCG:
    the start takes the coarse-grid correction w (w.r)/(w.A'w), and every
    search direction is kept A'-orthogonal to w.  On an unseen 96^3 seed with the
    committed weights, host-driven and as one graph launch per step: every
    solve converges to the same 1e-8, the coarse space changes the iterates
    (the pressure differs from the start-only run's by far more than the
    last-bit differences between repeated runs, and by less than the 1e-8
    solves allow), the two step forms agree, and the iteration counts are
    reported."""
    learned, make_case, _ = _mods()
    case = make_case((96, 96, 96), log_var=2.0, corr_len=8.0, seed=903)
    net = learned.WarmStartNet(48, 48, 48)
    net.set_params(learned.WarmStartNet.load_params(learned.DEFAULT_WEIGHTS))
    runs, fields = {}, {}
    for name, kw in (("start", {}), ("coarse", dict(net_coarse=True)),
                     ("coarse_graph", dict(net_coarse=True, step_graph=True))):
        fields[name] = {}
        runs[name] = learned.evaluate(case, net, 10, 20, net_always=True, fields=fields[name], **kw)
    net.close()
    # (the coarse space is on in every solve whose net ran, whether or not the
    # start took the net's correction)
    for name, st in runs.items():
        assert all(s[3] <= 1e-8 for s in st), name
    d = rel_l2(fields["coarse"]["pressure"], fields["start"]["pressure"])
    assert 1e-13 < d < 1e-6
    for k in ("pressure", "phase", "concent"):
        assert rel_l2(fields["coarse"][k], fields["start"][k]) < 1e-6, k
        assert rel_l2(fields["coarse_graph"][k], fields["coarse"][k]) < 1e-6, k
    its = {name: sum(s[1] for s in st) for name, st in runs.items()}
    print(f"learned coarse space, 96^3, 10 steps: PCG iterations start only {its['start']}, "
          f"with the coarse space {its['coarse']} (step graph {its['coarse_graph']})")
