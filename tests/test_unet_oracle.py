"""The numpy U-Net oracle pinned by identities that need no GPU: adjointness of the convolution's forward,
input-gradient and weight-gradient restatements, BF16 rounding, and a finite-difference check of the whole
network's gradient in FP32."""
import numpy as np
import pytest

from oracle import unet


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7 + 2 ** -8, -3.0000001, 65504.0, 1e-30], np.float32)
    r = unet.to_bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0  # tie -> even mantissa
    assert r[2] == np.float32(1.0 + 2 ** -6)  # tie -> even (rounds up)
    assert np.all((r.view(np.uint32) & 0xFFFF) == 0)
    assert abs(r[3] + 3.0) < 1e-6


@pytest.mark.parametrize("shape", [(1, 5, 7, 4, 6), (2, 8, 8, 3, 5)])
def test_conv_adjoint_identities(shape):
    n, h, w, cin, cout = shape
    rng = np.random.default_rng(1)
    x = rng.standard_normal((n, h, w, cin)).astype(np.float32)
    wt = rng.standard_normal((cout, 3, 3, cin)).astype(np.float32)
    gy = rng.standard_normal((n, h, w, cout)).astype(np.float32)
    y = unet.conv3x3(x, wt)
    gx = unet.conv3x3_dgrad(gy, wt)
    gw = unet.conv3x3_wgrad(x, gy)
    a = float(np.sum(y.astype(np.float64) * gy))
    assert a == pytest.approx(float(np.sum(x.astype(np.float64) * gx)), rel=1e-4)
    assert a == pytest.approx(float(np.sum(wt.astype(np.float64) * gw)), rel=1e-4)
    # direct definition at one output
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    ref = sum(xp[0, 2 + dy, 3 + dx] @ wt[:, dy, dx, :].T for dy in range(3) for dx in range(3))
    np.testing.assert_allclose(y[0, 2, 3], ref, rtol=1e-5, atol=1e-5)


def test_network_gradient_matches_finite_differences():
    rng = np.random.default_rng(7)
    n, h, w = 1, 16, 16
    layers = []
    for cin, cout, _ in unet.layer_shapes():
        layers.append((rng.standard_normal((cout, 3, 3, cin)).astype(np.float32) * np.sqrt(2.0 / (9 * cin)),
                       rng.standard_normal(cout).astype(np.float32) * 0.05))
    params = unet.pack_params(layers).astype(np.float64)
    feat = rng.uniform(0, 1, (n, h, w, unet.FEATURES)).astype(np.float32)
    target = rng.uniform(0.1, 2.0, (n, h, w, 3)).astype(np.float32)
    loss, grad, _ = unet.gradients(params.astype(np.float32), feat, target, bf16=False)
    # central differences on a few parameters of several layers
    offs = np.cumsum([0] + [cout * 9 * cin + cout for cin, cout, _ in unet.layer_shapes()])
    idx = []
    for li in (0, 5, 9, 12, 17, 18):
        lo, hi = offs[li], offs[li + 1]
        idx += list(rng.integers(lo, hi, 3))
    for i in idx:
        if abs(grad[i]) < 1e-5:
            continue
        eps = 1e-3 * max(1.0, abs(params[i]))
        p1, p2 = params.copy(), params.copy()
        p1[i] += eps
        p2[i] -= eps
        l1 = unet.gradients(p1.astype(np.float32), feat, target, bf16=False)[0]
        l2 = unet.gradients(p2.astype(np.float32), feat, target, bf16=False)[0]
        fd = (l1 - l2) / (2 * eps)
        assert fd == pytest.approx(float(grad[i]), rel=0.05, abs=2e-5), i
