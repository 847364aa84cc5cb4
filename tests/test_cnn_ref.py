"""CPU checks of the float64 network reference used by the GPU network tests:
its analytic gradient against central finite differences, and its conv /
data-gradient / weight-gradient conventions against each other (adjointness)."""
import numpy as np

import cnn_ref as R


def _case(seed, dims=(5, 4, 3)):
    W, H, D = dims
    rng = np.random.default_rng(seed)
    feat = rng.uniform(-1, 1, (D, H, W, 16))
    params = rng.normal(0, 0.15, R.n_params())
    # only output channel 0 of the last layer is live
    w4 = R.split(params)[3][0]
    off = sum(27 * i * o + o for i, o in R.LAYERS[:3])
    mask = np.zeros((27, 16, 32), bool)
    mask[:, 0, :] = True
    params[off:off + w4.size] *= mask.reshape(-1)
    target = rng.uniform(-0.9, 0.9, (D, H, W))
    active = rng.random((D, H, W)) < 0.6
    return feat, params, target, active


def test_gradient_matches_finite_differences():
    feat, params, target, active = _case(1)
    loss, g = R.loss_and_grad(feat, params, target, active, emulate=False)
    assert loss > 0
    rng = np.random.default_rng(2)
    idx = rng.choice(np.flatnonzero(np.abs(g) > 1e-6), 40, replace=False)
    h = 1e-6
    for i in idx:
        p1, p2 = params.copy(), params.copy()
        p1[i] += h
        p2[i] -= h
        l1, _ = R.loss_and_grad(feat, p1, target, active, emulate=False)
        l2, _ = R.loss_and_grad(feat, p2, target, active, emulate=False)
        fd = (l1 - l2) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, fd, g[i])


def test_conv_adjoint_identities():
    """<conv(x, w), y> = <x, conv_flip(y, w^T)> = <w, wgrad(x, y)>."""
    rng = np.random.default_rng(3)
    x = rng.normal(size=(3, 4, 5, 16))
    y = rng.normal(size=(3, 4, 5, 8))
    w = rng.normal(size=(27, 8, 16))
    a = (R.conv(x, w) * y).sum()
    b = (x * R.conv(y, w.transpose(0, 2, 1), flip=True)).sum()
    c = (w * R.wgrad(x, y)).sum()
    assert abs(a - b) < 1e-9 * abs(a) + 1e-9
    assert abs(a - c) < 1e-9 * abs(a) + 1e-9


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 0.0, 1e-3], np.float64)
    r = R.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0 + 2 ** -6  # 1 + 3/256 rounds up to 1 + 4/256
    assert r[3] == -2.5 and r[4] == 0.0
    assert abs(r[5] - 1e-3) < 1e-3 * 2 ** -8
    assert np.array_equal(R.from_bf16_bits(R.bf16_bits(x)), r)
