"""The CPU restatement of the warm-start network (oracle/net_oracle.py) pinned
by its own mathematics: adjoint identities of the convolution pieces and
finite differences of the loss through the whole U-Net (float64, no
rounding).  These make it a trustworthy check of the GPU gradients."""
import numpy as np
import pytest

import net_oracle as N


def _rand(rng, *shape):
    return rng.standard_normal(shape)


def test_conv_adjoints():
    rng = np.random.default_rng(0)
    x = _rand(rng, 5, 6, 7, 16)
    w = _rand(rng, 32, 27, 16)
    gy = _rand(rng, 5, 6, 7, 32)
    y = N.conv3d(x, w)
    # <conv(x), gy> = <x, dgrad(gy)> = <w, wgrad(x, gy)>
    a = float((y * gy).sum())
    assert np.isclose(a, float((x * N.conv3d_dgrad(gy, w)).sum()), rtol=1e-12)
    gw, gb = N.conv3d_wgrad(x, gy)
    assert np.isclose(a, float((w * gw).sum()), rtol=1e-12)
    assert np.allclose(gb, gy.reshape(-1, 32).sum(0))


def test_conv_known_answer():
    # a single centre tap of weight 1 is the identity; a +x tap shifts by one
    x = np.arange(4 * 3 * 5 * 16, dtype=float).reshape(4, 3, 5, 16)
    w = np.zeros((16, 27, 16))
    w[:, 13, :] = np.eye(16)
    assert np.array_equal(N.conv3d(x, w), x)
    w2 = np.zeros((16, 27, 16))
    w2[:, 14, :] = np.eye(16)          # tap (0, 0, +1)
    y = N.conv3d(x, w2)
    assert np.array_equal(y[:, :, :-1], x[:, :, 1:])
    assert not y[:, :, -1].any()


def test_pool_up_adjoints():
    rng = np.random.default_rng(1)
    x = _rand(rng, 4, 6, 8, 3)
    g = _rand(rng, 2, 3, 4, 3)
    assert np.isclose((N.pool2(x) * g).sum(), (x * N.pool2_bwd(g)).sum())
    assert np.isclose((N.up2(g) * x).sum(), (g * N.up2_bwd(x)).sum())


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7 + 2 ** -9, -3.14159, 0.0], np.float32)
    r = N.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0            # tie to even
    assert r[2] == np.float32(1.0 + 2 ** -7)
    assert np.array_equal(N.from_bits(N.to_bits(v)), r)


@pytest.mark.parametrize("seed", [3, 4])
def test_unet_gradient_finite_differences(seed):
    rng = np.random.default_rng(seed)
    p = N.init_params(seed).astype(np.float64)
    x = rng.standard_normal((8, 8, 8, 16))
    tgt = rng.standard_normal((8, 8, 8))
    mask = (rng.random((8, 8, 8)) > 0.3).astype(float)
    out, acts = N.forward(p, x, rounding=False)
    g = N.backward(p, acts, tgt, mask, rounding=False)
    assert g.shape == (N.param_count(),)
    idx = rng.choice(p.size, 12, replace=False)
    # include a bias of the last layer and a weight of the first
    idx = np.concatenate([idx, [p.size - 1, 5]])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        lp = N.loss(N.forward(pp, x, rounding=False)[0], tgt, mask)
        lm = N.loss(N.forward(pm, x, rounding=False)[0], tgt, mask)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (i, fd, g[i])
