"""CPU restatement of the learned warm start's network (test infrastructure).

The network has no counterpart in the reference (wPFAW3D.f90:980 starts each
pressure solve from the previous pressure); this file restates, in numpy, the
arithmetic the GPU kernels of mizuho_edit_gb300/csrc/wpf_net.cu perform, so
that the tests can check their forward pass and gradients.  It is pinned by
finite differences of its own forward pass (tests/test_net_oracle.py), not by
reference data.  Only tests import it.

Conventions (those of include/wpf_net.h): tensors are (nz, ny, nx, C) with
the channel innermost; a convolution weight is (Cout, 27, Cin) with tap
t = (dz+1)*9 + (dy+1)*3 + (dx+1); "same" zero padding; bf16 storage of
activations, weights and back-propagated gradients (round to nearest even),
products exact and sums in higher precision (the GPU accumulates in FP32).
"""
from __future__ import annotations

import numpy as np

LAYER_CIN = (16, 16, 32, 64, 64, 32, 16)
LAYER_COUT = (16, 32, 64, 64, 32, 16, 16)
LAYER_LEVEL = (0, 1, 2, 3, 2, 1, 0)
TAPS = [(t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1) for t in range(27)]   # (dz, dy, dx)


def bf16(x) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    return (b.astype(np.uint32) << 16).view(np.float32).reshape(a.shape)


def to_bits(x) -> np.ndarray:
    """bfloat16 bit patterns (uint16) of float32 values (nearest even)."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    return ((b + 0x7FFF + ((b >> 16) & 1)) >> 16).astype(np.uint16)


def from_bits(b) -> np.ndarray:
    return (np.asarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def _shift(x, dz, dy, dx):
    """y[z,y,x] = x[z+dz, y+dy, x+dx] with zeros outside."""
    out = np.zeros_like(x)
    nz, ny, nx = x.shape[:3]
    zs = slice(max(0, -dz), nz - max(0, dz))
    ys = slice(max(0, -dy), ny - max(0, dy))
    xs = slice(max(0, -dx), nx - max(0, dx))
    zd = slice(max(0, dz), nz - max(0, -dz))
    yd = slice(max(0, dy), ny - max(0, -dy))
    xd = slice(max(0, dx), nx - max(0, -dx))
    out[zs, ys, xs] = x[zd, yd, xd]
    return out


def conv3d(x, w, b=None):
    """out[v][co] = b[co] + sum_{t,ci} x[v + d_t][ci] w[co][t][ci]  (float64)."""
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    out = np.zeros(x.shape[:3] + (w.shape[0],))
    for t, (dz, dy, dx) in enumerate(TAPS):
        out += _shift(x, dz, dy, dx) @ w[:, t, :].T
    if b is not None:
        out += np.asarray(b, np.float64)
    return out


def conv3d_dgrad(gy, w):
    """d/dx of sum(gy * conv3d(x, w)): gx[v][ci] = sum_{t,co} gy[v - d_t][co] w[co][t][ci]."""
    gy = np.asarray(gy, np.float64)
    w = np.asarray(w, np.float64)
    gx = np.zeros(gy.shape[:3] + (w.shape[2],))
    for t, (dz, dy, dx) in enumerate(TAPS):
        gx += _shift(gy, -dz, -dy, -dx) @ w[:, t, :]
    return gx


def conv3d_wgrad(x, gy):
    """gw[co][t][ci] = sum_v gy[v][co] x[v + d_t][ci];  gb[co] = sum_v gy[v][co]."""
    x = np.asarray(x, np.float64)
    gy = np.asarray(gy, np.float64)
    cin, cout = x.shape[3], gy.shape[3]
    gw = np.zeros((cout, 27, cin))
    g2 = gy.reshape(-1, cout)
    for t, (dz, dy, dx) in enumerate(TAPS):
        gw[:, t, :] = g2.T @ _shift(x, dz, dy, dx).reshape(-1, cin)
    return gw, g2.sum(axis=0)


def pool2(x):
    nz, ny, nx, c = x.shape
    return x.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).mean(axis=(1, 3, 5))


def up2(x):
    return x.repeat(2, axis=0).repeat(2, axis=1).repeat(2, axis=2)


def up2_bwd(g):
    nz, ny, nx, c = g.shape
    return g.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).sum(axis=(1, 3, 5))


def pool2_bwd(g):
    return up2(g) / 8.0


def split_params(p):
    """Flat parameter vector -> [(w (Cout,27,Cin), b (Cout,)) per layer]."""
    out, off = [], 0
    for ci, co in zip(LAYER_CIN, LAYER_COUT):
        n = co * 27 * ci
        out.append((p[off:off + n].reshape(co, 27, ci), p[off + n:off + n + co]))
        off += n + co
    return out


def param_count():
    return sum(co * 27 * ci + co for ci, co in zip(LAYER_CIN, LAYER_COUT))


def forward(params, x, rounding=True):
    """The U-Net forward pass; returns (out fp32 (nz,ny,nx,16), activations).

    rounding=True stores every activation in bf16 as the GPU does (weights
    are rounded to bf16 too); False gives the exact float64 function (for
    finite-difference checks)."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    layers = [(r(w), b) for w, b in
              split_params(np.asarray(params, np.float32 if rounding else np.float64))]
    relu = lambda a: np.maximum(a, 0.0)
    x = r(x)
    y0 = r(relu(conv3d(x, *layers[0])))
    p0 = r(pool2(y0))
    y1 = r(relu(conv3d(p0, *layers[1])))
    p1 = r(pool2(y1))
    y2 = r(relu(conv3d(p1, *layers[2])))
    p2 = r(pool2(y2))
    y3 = r(relu(conv3d(p2, *layers[3])))
    s2 = r(up2(y3) + y2)
    y4 = r(relu(conv3d(s2, *layers[4])))
    s1 = r(up2(y4) + y1)
    y5 = r(relu(conv3d(s1, *layers[5])))
    s0 = r(up2(y5) + y0)
    out = conv3d(s0, *layers[6])
    if rounding:
        out = out.astype(np.float32)
    acts = dict(x=x, y0=y0, p0=p0, y1=y1, p1=p1, y2=y2, p2=p2, y3=y3, s2=s2, y4=y4, s1=s1, y5=y5,
                s0=s0, out=out)
    return out, acts


def loss(out, target, mask=None):
    m = np.ones_like(target) if mask is None else mask
    d = out[..., 0] - target
    return float((m * d * d).sum() / m.sum())


def backward(params, acts, target, mask=None, rounding=True):
    """Gradient of loss() w.r.t. the flat parameters, in the GPU's order of
    operations (bf16 storage of every back-propagated tensor when rounding)."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    layers = [(r(w), b) for w, b in
              split_params(np.asarray(params, np.float32 if rounding else np.float64))]
    m = np.ones_like(target) if mask is None else mask
    a = acts
    gout = np.zeros(a["out"].shape)
    gout[..., 0] = 2.0 * m * (a["out"][..., 0] - target) / m.sum()
    gout = r(gout)
    grads = [None] * 7

    def lay(l, x, g):
        grads[l] = conv3d_wgrad(x, g)

    mask_relu = lambda g, y: np.where(y > 0, g, 0.0)
    lay(6, a["s0"], gout)
    gs0 = r(conv3d_dgrad(gout, layers[6][0]))
    g5 = r(mask_relu(up2_bwd(gs0), a["y5"]))
    lay(5, a["s1"], g5)
    gs1 = r(conv3d_dgrad(g5, layers[5][0]))
    g4 = r(mask_relu(up2_bwd(gs1), a["y4"]))
    lay(4, a["s2"], g4)
    gs2 = r(conv3d_dgrad(g4, layers[4][0]))
    g3 = r(mask_relu(up2_bwd(gs2), a["y3"]))
    lay(3, a["p2"], g3)
    gp2 = r(conv3d_dgrad(g3, layers[3][0]))
    g2 = r(mask_relu(pool2_bwd(gp2) + gs2, a["y2"]))
    lay(2, a["p1"], g2)
    gp1 = r(conv3d_dgrad(g2, layers[2][0]))
    g1 = r(mask_relu(pool2_bwd(gp1) + gs1, a["y1"]))
    lay(1, a["p0"], g1)
    gp0 = r(conv3d_dgrad(g1, layers[1][0]))
    g0 = r(mask_relu(pool2_bwd(gp0) + gs0, a["y0"]))
    lay(0, a["x"], g0)
    flat = []
    for gw, gb in grads:
        flat.append(gw.ravel())
        flat.append(gb.ravel())
    return np.concatenate(flat)


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    p = []
    for l, (ci, co) in enumerate(zip(LAYER_CIN, LAYER_COUT)):
        sd = np.sqrt(2.0 / (27 * ci)) * (0.1 if l == 6 else 1.0)
        p.append(rng.normal(0, sd, co * 27 * ci))
        p.append(rng.normal(0, 0.05, co))
    return np.concatenate(p).astype(np.float32)
