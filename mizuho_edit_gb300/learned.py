"""Learned warm start of the Darcy solve: data generation, training, evaluation.

The network (include/wpf_net.h, kernels in csrc/wpf_net.cu) maps the state at
half resolution -- log K_rock, phase, pressure, the last two pressure
increments, their time extrapolation and the phase change of the last step --
to a correction of the extrapolated increment.  Its training data are pairs
(input, target) that the simulator itself produces: target = (the solve's
increment - the extrapolation), restricted 2x2x2 and scaled by the rms of the
last increment.  The solve always finishes at the same FP64 residual
tolerance and keeps the network's start only when its FP64 residual is the
smallest of the candidates (previous pressure, extrapolation, extrapolation +
network), so the network changes iteration counts, never the answer.

PyTorch only holds device memory here; every kernel is the library's.

    python -m mizuho_edit_gb300.learned train --out weights.npz [--runs 20 --n 128 ...]
    python -m mizuho_edit_gb300.learned time --grid 128      # forward-pass time
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import time

import numpy as np

from . import capi
from .cases import make_case
from .sim import Simulation

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(HERE, "weights", "warm_start_unet.npz")


def _ptr(t):
    return C.c_void_p(t.data_ptr())


class WarmStartNet:
    """One wpf_net for an (nx, ny, nz) net grid (half the simulation grid)."""

    def __init__(self, nx: int, ny: int, nz: int, seed: int = 0):
        self.L = capi.load()
        h = C.c_void_p()
        capi.check(self.L.wpf_net_create(nx, ny, nz, C.byref(h)), "wpf_net_create")
        self.h = h
        self.dims = (nx, ny, nz)
        capi.check(self.L.wpf_net_init(h, seed), "wpf_net_init")
        n = C.c_int64()
        self.L.wpf_net_param_count(h, C.byref(n))
        self.nparam = n.value

    def params(self) -> np.ndarray:
        out = np.zeros(self.nparam, np.float32)
        capi.check(self.L.wpf_net_get_params(self.h, out.ctypes.data_as(C.c_void_p)), "get_params")
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.nparam:
            raise ValueError(f"expected {self.nparam} parameters, got {p.size}")
        capi.check(self.L.wpf_net_set_params(self.h, p.ctypes.data_as(C.c_void_p)), "set_params")

    def train_step(self, x, target, lr: float, mask=None) -> float:
        loss = C.c_float()
        capi.check(self.L.wpf_net_train_step(self.h, _ptr(x), _ptr(target),
                                             _ptr(mask) if mask is not None else None, lr,
                                             C.byref(loss), None), "wpf_net_train_step")
        return loss.value

    def forward(self, x, out):
        capi.check(self.L.wpf_net_forward(self.h, _ptr(x), _ptr(out), None), "wpf_net_forward")

    def save(self, path: str, meta: dict | None = None):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez_compressed(path, params=self.params(), meta=json.dumps(meta or {}))

    @staticmethod
    def load_params(path: str) -> np.ndarray:
        with np.load(path) as z:
            return z["params"]

    def close(self):
        if getattr(self, "h", None):
            self.L.wpf_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def attach(sim: Simulation, net: WarmStartNet | None):
    """Use net (or none) as the learned start of sim's solves."""
    capi.check(sim.L.wpf_set_warm_start_net(sim.h, net.h if net is not None else None),
               "wpf_set_warm_start_net")


def collect_pairs(sim: Simulation, steps: int, store: list, every: int = 1):
    """Advance sim by `steps` steps, appending (input, target) device pairs for
    the steps whose solve had two increments to extrapolate from."""
    import torch
    n = sim.params
    nv = (n.nx // 2) * (n.ny // 2) * (n.nz // 2)
    for s in range(steps):
        take = (s % every == 0)
        x = None
        if take:
            x = torch.empty(nv * 16, dtype=torch.int16, device="cuda")
            rc = sim.L.wpf_ws_features(sim.h, sim.next_dtime(sim.itime + 1), _ptr(x))
            if rc == capi.WPF_ERR_ARG:      # fewer than two increments yet
                x = None
            else:
                capi.check(rc, "wpf_ws_features")
        sim.step()
        if x is not None:
            t = torch.empty(nv, dtype=torch.float32, device="cuda")
            capi.check(sim.L.wpf_ws_target(sim.h, _ptr(t)), "wpf_ws_target")
            store.append((x, t))
    return store


def generate(runs: int, n: int, steps: int, spinup: int, seed0: int = 1000, every: int = 1,
             log=print):
    """Training pairs from `runs` seeded n^3 runs: log-K variance U(1, 3),
    correlation length U(4, 16) cells; `spinup` steps are skipped first."""
    rng = np.random.default_rng(seed0)
    pairs = []
    for r in range(runs):
        lv, cl = float(rng.uniform(1.0, 3.0)), float(rng.uniform(4.0, 16.0))
        case = make_case((n, n, n), log_var=lv, corr_len=cl, seed=seed0 + r)
        with Simulation(case.params, case.permeab_rock, case.phase, case.concent, solver="mixed",
                        rtol=1e-8, extrapolate=True) as sim:
            for _ in range(spinup):
                sim.step()
            before = len(pairs)
            collect_pairs(sim, steps, pairs, every)
        log(f"run {r}: log-K var {lv:.2f} corr {cl:.1f}: {len(pairs) - before} pairs")
    return pairs


def validation_loss(net: WarmStartNet, pairs) -> float:
    """Mean over pairs of the training loss, mean_v (out_v - target_v)^2,
    without a parameter update."""
    import torch
    if not pairs:
        return float("nan")
    out = torch.empty_like(pairs[0][1])
    tot = 0.0
    for x, t in pairs:
        net.forward(x, out)
        tot += float(((out - t).double() ** 2).mean())
    return tot / len(pairs)


def train(net: WarmStartNet, pairs, epochs: int, lr: float, seed: int = 0, val_frac: float = 0.1,
          log=print):
    """Adam over shuffled pairs with a cosine learning-rate schedule; a
    held-out fraction of the pairs is scored after every epoch and the
    parameters of the best held-out epoch are kept.  Returns
    {"train": [mean loss per epoch], "val": [held-out loss per epoch],
    "best_epoch": e}."""
    import math
    rng = np.random.default_rng(seed)
    idx = rng.permutation(len(pairs))
    nval = int(len(pairs) * val_frac) if len(pairs) >= 20 else 0
    val = [pairs[i] for i in idx[:nval]]
    tr = [pairs[i] for i in idx[nval:]]
    hist, vhist = [], []
    best = None
    for ep in range(epochs):
        lr_ep = lr * 0.5 * (1.0 + math.cos(math.pi * ep / max(epochs, 1)))
        tot = 0.0
        for q in rng.permutation(len(tr)):
            x, t = tr[q]
            tot += net.train_step(x, t, lr_ep)
        hist.append(tot / max(len(tr), 1))
        v = validation_loss(net, val) if val else hist[-1]
        vhist.append(v)
        if best is None or v < best[0]:
            best = (v, ep, net.params())
        log(f"epoch {ep}: lr {lr_ep:.2e} train loss {hist[-1]:.4e} held-out loss {v:.4e}")
    if best is not None and best[1] != epochs - 1:
        net.set_params(best[2])
    return {"train": hist, "val": vhist, "best_epoch": best[1] if best else -1}


def evaluate(case, net: WarmStartNet | None, steps: int, spinup: int, net_always: bool = False,
             net_coarse: bool = False, step_graph: bool = False, fields: dict | None = None):
    """Per-step stats of a run with the extrapolated start, with or without
    the network: (relres0, inner iterations, warm_start code, relres) per
    timed step.  net_always evaluates the net at every solve instead of only
    where the extrapolation misses the tolerance by at most 1.02x; net_coarse
    also uses its output as the PCG's one-vector coarse space; step_graph runs
    the steps as one graph launch each.  fields (a dict) receives the final
    phase, concentration and pressure."""
    out = []
    with Simulation(case.params, case.permeab_rock, case.phase, case.concent, solver="mixed",
                    rtol=1e-8, extrapolate=True, net_always=net_always, net_coarse=net_coarse,
                    step_graph=step_graph) as sim:
        attach(sim, net)
        for _ in range(spinup):
            sim.step()
        for _ in range(steps):
            st = sim.step()
            out.append((st.relres0, st.inner_iterations, st.warm_start, st.relres))
        if fields is not None:
            fields.update(sim.download("phase", "concent", "pressure"))
        attach(sim, None)
    return out


def time_forward(m: int, reps: int = 5) -> dict:
    """Forward pass of a seeded net on an m^3 net grid (the solve at (2m)^3
    cells), random BF16 input, one untimed pass, then `reps` timed with CUDA
    events on the default stream."""
    import torch
    net = WarmStartNet(m, m, m, seed=1)
    try:
        gen = torch.Generator(device="cuda").manual_seed(0)
        x = torch.randn(m ** 3 * 16, device="cuda", generator=gen).to(torch.bfloat16).view(torch.int16)
        out = torch.empty(m ** 3, dtype=torch.float32, device="cuda")
        net.forward(x, out)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            net.forward(x, out)
        e1.record()
        torch.cuda.synchronize()
        return {"net_grid": m, "forward_ms": e0.elapsed_time(e1) / max(reps, 1)}
    finally:
        net.close()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--out", default=DEFAULT_WEIGHTS)
    t.add_argument("--runs", type=int, default=20)
    t.add_argument("--n", type=int, default=128)
    t.add_argument("--steps", type=int, default=100)
    t.add_argument("--spinup", type=int, default=10)
    t.add_argument("--epochs", type=int, default=12)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--eval-n", type=int, default=128)
    f = sub.add_parser("time", help="time the forward pass on an m^3 net grid (random input)")
    f.add_argument("--grid", type=int, default=128)
    f.add_argument("--reps", type=int, default=5)
    a = ap.parse_args(argv)
    if a.cmd == "time":
        print(json.dumps(time_forward(a.grid, a.reps)))
        return
    t0 = time.time()
    pairs = generate(a.runs, a.n, a.steps, a.spinup)
    t1 = time.time()
    net = WarmStartNet(a.n // 2, a.n // 2, a.n // 2, seed=a.seed)
    hist = train(net, pairs, a.epochs, a.lr, a.seed)
    t2 = time.time()
    meta = {"runs": a.runs, "n": a.n, "steps": a.steps, "spinup": a.spinup, "epochs": a.epochs,
            "lr": a.lr, "schedule": "cosine", "pairs": len(pairs), "loss": hist["train"],
            "val_loss": hist["val"], "best_epoch": hist["best_epoch"], "gen_s": t1 - t0,
            "train_s": t2 - t1}
    net.save(a.out, meta)
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
