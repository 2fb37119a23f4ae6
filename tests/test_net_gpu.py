"""The tcgen05 BF16 network kernels against the CPU restatement
(oracle/net_oracle.py): convolution forward, weight gradient, the whole U-Net
forward pass and its parameter gradients, and that training on the GPU
lowers the loss."""
import ctypes as C

import numpy as np
import pytest

import net_oracle as N
from conftest import rel_l2

pytestmark = pytest.mark.gpu

PAIRS = [(16, 16), (16, 32), (32, 64), (64, 64), (64, 32), (32, 16)]


def _lib():
    from mizuho_edit_gb300 import capi
    return capi, capi.load()


def _dev_bf16(a):
    import torch
    return torch.from_numpy(N.to_bits(a).view(np.int16).copy()).cuda()


def _dev_f32(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _ptr(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("cin,cout", PAIRS)
def test_conv3d_matches_oracle(cin, cout):
    import torch
    capi, L = _lib()
    rng = np.random.default_rng(cin * 100 + cout)
    nz, ny, nx = 9, 10, 12                      # 1080 voxels: a partial last tile
    x = N.bf16(rng.standard_normal((nz, ny, nx, cin)))
    w = N.bf16(rng.standard_normal((cout, 27, cin)) * 0.2)
    b = rng.standard_normal(cout).astype(np.float32)
    ref = N.conv3d(x, w, b)
    dx, dw, db = _dev_bf16(x), _dev_bf16(w), _dev_f32(b)
    out32 = torch.zeros(nz * ny * nx * cout, dtype=torch.float32, device="cuda")
    capi.check(L.wpf_conv3d(cin, cout, nx, ny, nz, _ptr(dx), _ptr(dw), _ptr(db), 0, None,
                            _ptr(out32), None), "wpf_conv3d")
    got = out32.cpu().numpy().reshape(nz, ny, nx, cout)
    assert rel_l2(got, ref) < 1e-5
    # ReLU + bf16 output
    out16 = torch.zeros(nz * ny * nx * cout, dtype=torch.int16, device="cuda")
    capi.check(L.wpf_conv3d(cin, cout, nx, ny, nz, _ptr(dx), _ptr(dw), _ptr(db), 1,
                            _ptr(out16), None, None), "wpf_conv3d")
    got16 = N.from_bits(out16.cpu().numpy().view(np.uint16)).reshape(nz, ny, nx, cout)
    want16 = N.bf16(np.maximum(ref, 0))
    assert np.mean(got16 != want16) < 0.01      # at most rare one-ulp rounding differences
    assert rel_l2(got16, want16) < 1e-2


# (nx, ny, nz) that route 16-channel inputs to the row-tiled kernel, one per
# brick width: 128 x 1 (one staged 130-voxel row), 64 x 2, 32 x 4, 16 x 8
ROW_SHAPES = [(128, 3, 4), (64, 4, 3), (96, 4, 2), (48, 8, 3)]


@pytest.mark.parametrize("shape", ROW_SHAPES)
@pytest.mark.parametrize("cout", [16, 32])
def test_conv3d_row_tiled_matches_oracle(shape, cout):
    """The TMA-staged row-tiled convolution of the 16-channel layers: zero
    padding by the copies' out-of-range fill, every tap a window of the
    staged halo."""
    import torch
    capi, L = _lib()
    nx, ny, nz = shape
    rng = np.random.default_rng(nx + ny + cout)
    x = N.bf16(rng.standard_normal((nz, ny, nx, 16)))
    w = N.bf16(rng.standard_normal((cout, 27, 16)) * 0.2)
    b = rng.standard_normal(cout).astype(np.float32)
    ref = N.conv3d(x, w, b)
    dx, dw, db = _dev_bf16(x), _dev_bf16(w), _dev_f32(b)
    out32 = torch.zeros(nz * ny * nx * cout, dtype=torch.float32, device="cuda")
    capi.check(L.wpf_conv3d(16, cout, nx, ny, nz, _ptr(dx), _ptr(dw), _ptr(db), 0, None,
                            _ptr(out32), None), "wpf_conv3d")
    got = out32.cpu().numpy().reshape(nz, ny, nx, cout)
    assert rel_l2(got, ref) < 1e-5
    out16 = torch.zeros(nz * ny * nx * cout, dtype=torch.int16, device="cuda")
    capi.check(L.wpf_conv3d(16, cout, nx, ny, nz, _ptr(dx), _ptr(dw), _ptr(db), 1,
                            _ptr(out16), None, None), "wpf_conv3d")
    got16 = N.from_bits(out16.cpu().numpy().view(np.uint16)).reshape(nz, ny, nx, cout)
    want16 = N.bf16(np.maximum(ref, 0))
    assert np.mean(got16 != want16) < 0.01
    assert rel_l2(got16, want16) < 1e-2


@pytest.mark.parametrize("cin,cout", PAIRS)
def test_conv3d_wgrad_matches_oracle(cin, cout):
    import torch
    capi, L = _lib()
    rng = np.random.default_rng(7 + cin + cout)
    nz, ny, nx = 11, 13, 17                     # 2431 voxels: two voxel chunks, ragged stages
    x = N.bf16(rng.standard_normal((nz, ny, nx, cin)))
    gy = N.bf16(rng.standard_normal((nz, ny, nx, cout)))
    gw_ref, gb_ref = N.conv3d_wgrad(x, gy)
    gw = torch.zeros(cout * 27 * cin, dtype=torch.float32, device="cuda")
    gb = torch.zeros(cout, dtype=torch.float32, device="cuda")
    dx, dg = _dev_bf16(x), _dev_bf16(gy)        # held: a freed temporary's memory gets reused
    capi.check(L.wpf_conv3d_wgrad(cin, cout, nx, ny, nz, _ptr(dx), _ptr(dg), _ptr(gw), _ptr(gb),
                                  None), "wpf_conv3d_wgrad")
    assert rel_l2(gw.cpu().numpy().reshape(cout, 27, cin), gw_ref) < 1e-5
    assert rel_l2(gb.cpu().numpy(), gb_ref) < 1e-5


class _Net:
    def __init__(self, n):
        self.capi, self.L = _lib()
        h = C.c_void_p()
        self.capi.check(self.L.wpf_net_create(n, n, n, C.byref(h)), "wpf_net_create")
        self.h = h
        cnt = C.c_int64()
        self.L.wpf_net_param_count(h, C.byref(cnt))
        self.nparam = cnt.value

    def set(self, p):
        p = np.ascontiguousarray(p, np.float32)
        self.capi.check(self.L.wpf_net_set_params(self.h, p.ctypes.data_as(C.c_void_p)), "set")

    def get(self, fn="wpf_net_get_params"):
        out = np.zeros(self.nparam, np.float32)
        self.capi.check(getattr(self.L, fn)(self.h, out.ctypes.data_as(C.c_void_p)), fn)
        return out

    def close(self):
        self.L.wpf_net_destroy(self.h)


def test_unet_forward_and_gradients_match_oracle():
    import torch
    n = 16
    net = _Net(n)
    try:
        assert net.nparam == N.param_count()
        rng = np.random.default_rng(11)
        p = N.init_params(11)
        x = N.bf16(rng.standard_normal((n, n, n, 16)))
        tgt = rng.standard_normal((n, n, n)).astype(np.float32)
        mask = (rng.random((n, n, n)) > 0.2).astype(np.float32)
        net.set(p)
        dx, dt, dm = _dev_bf16(x), _dev_f32(tgt), _dev_f32(mask)
        loss = C.c_float()
        # lr = 0: one forward + backward, parameters unchanged
        net.capi.check(net.L.wpf_net_train_step(net.h, _ptr(dx), _ptr(dt), _ptr(dm), 0.0,
                                                C.byref(loss), None), "train_step")
        out_ref, acts = N.forward(p, x)
        g_ref = N.backward(p, acts, tgt, mask)
        # activations of every convolution
        names = ["y0", "y1", "y2", "y3", "y4", "y5", "out"]
        for layer, name in enumerate(names):
            ref = N.bf16(acts[name])
            buf = np.zeros(ref.size, np.uint16)
            net.capi.check(net.L.wpf_net_get_activation(net.h, layer, buf.ctypes.data_as(C.c_void_p),
                                                        ref.size), "act")
            assert rel_l2(N.from_bits(buf).reshape(ref.shape), ref) < 2e-2, name
        assert abs(loss.value - N.loss(out_ref, tgt, mask)) < 1e-2 * N.loss(out_ref, tgt, mask)
        g = net.get("wpf_net_get_grads")
        off = 0
        for l, (ci, co) in enumerate(zip(N.LAYER_CIN, N.LAYER_COUT)):
            k = co * 27 * ci + co
            assert rel_l2(g[off:off + k], g_ref[off:off + k]) < 5e-2, l
            off += k
        assert np.array_equal(net.get(), p)         # lr = 0 left the parameters alone
        # forward pass alone gives channel 0 of the same output
        out = torch.zeros(n ** 3, dtype=torch.float32, device="cuda")
        net.capi.check(net.L.wpf_net_forward(net.h, _ptr(dx), _ptr(out), None), "forward")
        assert rel_l2(out.cpu().numpy().reshape(n, n, n), out_ref[..., 0]) < 2e-2
    finally:
        net.close()


def test_training_lowers_the_loss():
    n = 16
    net = _Net(n)
    try:
        capi, L = net.capi, net.L
        capi.check(L.wpf_net_init(net.h, 5), "init")
        rng = np.random.default_rng(5)
        x = rng.standard_normal((n, n, n, 16)) * (np.arange(16) < 7)
        # a smooth target that depends on two input channels
        tgt = (0.5 * x[..., 0] - 0.25 * x[..., 3]).astype(np.float32)
        dx, dt = _dev_bf16(x), _dev_f32(tgt)
        losses = []
        for _ in range(150):
            loss = C.c_float()
            capi.check(L.wpf_net_train_step(net.h, _ptr(dx), _ptr(dt), None, 3e-3,
                                            C.byref(loss), None), "train_step")
            losses.append(loss.value)
        assert np.isfinite(losses).all()
        assert losses[-1] < 0.2 * losses[0]
    finally:
        net.close()
