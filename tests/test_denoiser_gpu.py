"""The learned denoiser on the GPU against the numpy oracle (oracle/unet.py):

 * each tcgen05 convolution (forward with bias/ReLU/mask, input gradient, weight gradient) on random BF16
   tensors, including channel slices of wider buffers and image sides that are not tile multiples;
 * the whole network's loss and parameter gradients on a small batch (the oracle rounds to BF16 where the
   device does, so the remaining difference is FP32 accumulation order);
 * training steps lower the loss; inference matches the oracle forward; the per-tile fallback.

Tolerances (written in each test): BF16 conv outputs within 2 BF16 ulps (2^-7 relative) plus a small
absolute floor; FP32 weight gradients within 1e-3 relative L2; network gradients per layer as close to the
FP32 oracle as the BF16-rounding oracle is (1.5x + 0.02) and within 0.1 relative L2 of it.
"""
import numpy as np
import pytest

from oracle import unet
from sparkle_gb300 import native

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dn():
    d = native.Denoiser(0, seed=1)
    yield d
    d.close()


def bf16_tensor(a: np.ndarray):
    return torch.from_numpy(unet.to_bf16(a)).cuda().to(torch.bfloat16)


def host(t) -> np.ndarray:
    return t.float().cpu().numpy()


def assert_bf16_close(got, ref, rel=2 ** -7, abs_floor=None):
    ref = unet.to_bf16(ref)
    scale = float(np.abs(ref).max()) or 1.0
    atol = abs_floor if abs_floor is not None else 1e-3 * scale
    bad = np.abs(got - ref) > rel * np.abs(ref) + atol
    assert bad.mean() < 1e-4, (bad.sum(), bad.size, float(np.abs(got - ref).max()))


CONV_SHAPES = [
    # n, h, w, cin, cout
    (1, 8, 8, 32, 32),
    (2, 16, 24, 64, 96),
    (1, 32, 8, 96, 64),
    (1, 5, 130, 32, 128),
    (1, 4, 4, 256, 32),
    (1, 12, 20, 128, 256),
]
# Layers large enough that the forward kernel stacks 2 or 4 M tiles per CTA (32-64 output rows sharing one
# input box per column tap and one set of weight slices), including ragged bottom tiles and 8-column tiles.
LARGE_SHAPES = [
    (1, 300, 520, 32, 64),   # 2 M tiles
    (1, 1000, 520, 32, 64),  # 4 M tiles
    (1, 600, 520, 64, 128),  # 2 M tiles at 128 output channels
    (20, 1000, 12, 32, 32),  # 4 M tiles of 8 x 16 pixels
]


@pytest.mark.parametrize("shape", CONV_SHAPES + LARGE_SHAPES)
def test_conv_forward(dn, shape):
    n, h, w, cin, cout = shape
    rng = np.random.default_rng(hash(shape) & 0xFFFF)
    x = unet.to_bf16(rng.standard_normal((n, h, w, cin)).astype(np.float32))
    wt = unet.to_bf16((rng.standard_normal((cout, 3, 3, cin)) / np.sqrt(9 * cin)).astype(np.float32))
    b = rng.standard_normal(cout).astype(np.float32) * 0.1
    y = torch.zeros((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
    dn.conv3x3(0, bf16_tensor(x), cin, bf16_tensor(wt), y, cout, n, h, w, bias=torch.from_numpy(b).cuda(), relu=True)
    ref = np.maximum(unet.conv3x3(x, wt, b), 0)
    assert_bf16_close(host(y), ref)


def test_conv_forward_channel_slices(dn):
    """Input channels [16, 16 + 64) of an 96-channel buffer into channels [32, 32 + 64) of a 128-channel one."""
    n, h, w, cin, cout = 1, 16, 16, 64, 64
    rng = np.random.default_rng(3)
    big = unet.to_bf16(rng.standard_normal((n, h, w, 96)).astype(np.float32))
    wt = unet.to_bf16((rng.standard_normal((cout, 3, 3, cin)) / 24).astype(np.float32))
    xb = bf16_tensor(big)
    out = torch.full((n, h, w, 128), 7.0, dtype=torch.bfloat16, device="cuda")
    x_view = xb[..., 16:]
    y_view = out[..., 32:]
    dn.conv3x3(0, x_view, cin, bf16_tensor(wt), y_view, cout, n, h, w, x_ld=96, y_ld=128)
    ref = unet.conv3x3(big[..., 16:16 + cin], wt)
    got = host(out)
    assert_bf16_close(got[..., 32:96], ref)
    assert np.all(got[..., :32] == 7.0) and np.all(got[..., 96:] == 7.0)  # untouched channels


@pytest.mark.parametrize("shape", CONV_SHAPES[:4] + LARGE_SHAPES[1:3])
def test_conv_dgrad_with_mask(dn, shape):
    n, h, w, cin, cout = shape
    rng = np.random.default_rng(11 + cin)
    gy = unet.to_bf16(rng.standard_normal((n, h, w, cout)).astype(np.float32))
    wt = unet.to_bf16((rng.standard_normal((cout, 3, 3, cin)) / np.sqrt(9 * cout)).astype(np.float32))
    mask = unet.to_bf16(rng.standard_normal((n, h, w, cin)).astype(np.float32))
    gx = torch.zeros((n, h, w, cin), dtype=torch.bfloat16, device="cuda")
    dn.conv3x3(1, bf16_tensor(gy), cout, bf16_tensor(wt), gx, cin, n, h, w, mask=bf16_tensor(mask), mask_ld=cin)
    ref = unet.conv3x3_dgrad(gy, wt) * (mask > 0)
    assert_bf16_close(host(gx), ref)


@pytest.mark.parametrize("shape", CONV_SHAPES)
def test_conv_wgrad_accumulates(dn, shape):
    n, h, w, cin, cout = shape
    rng = np.random.default_rng(21 + cout)
    x = unet.to_bf16(rng.standard_normal((n, h, w, cin)).astype(np.float32))
    gy = unet.to_bf16(rng.standard_normal((n, h, w, cout)).astype(np.float32))
    dw = torch.zeros((cout, 3, 3, cin), dtype=torch.float32, device="cuda")
    xt, gt = bf16_tensor(x), bf16_tensor(gy)
    dn.conv3x3(2, xt, cin, None, gt, cout, n, h, w, dw=dw)
    dn.conv3x3(2, xt, cin, None, gt, cout, n, h, w, dw=dw)  # += a second time
    ref = 2.0 * unet.conv3x3_wgrad(x, gy).astype(np.float64)
    got = dw.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(got - ref) <= 1e-3 * np.linalg.norm(ref)


def test_conv_rejects_bad_shapes(dn):
    x = torch.zeros((1, 8, 8, 48), dtype=torch.bfloat16, device="cuda")
    y = torch.zeros((1, 8, 8, 32), dtype=torch.bfloat16, device="cuda")
    w = torch.zeros((32, 3, 3, 48), dtype=torch.bfloat16, device="cuda")
    with pytest.raises(native.SpkError):
        dn.conv3x3(0, x, 48, w, y, 32, 1, 8, 8)  # 48 channels: not a multiple of 32


def random_batch(n, h, w, seed):
    rng = np.random.default_rng(seed)
    hdr = rng.gamma(1.0, 0.6, (n, h, w, 4)).astype(np.float32)
    nd = np.concatenate([rng.standard_normal((n, h, w, 3)), rng.uniform(0, 20, (n, h, w, 1))], -1).astype(np.float32)
    alb = rng.uniform(0, 1, (n, h, w, 4)).astype(np.float32)
    feat = unet.pack_features(hdr, nd, alb)
    target = (hdr[..., :3] * rng.uniform(0.7, 1.3, (n, h, w, 3))).astype(np.float32)
    return feat, target


def test_network_gradients_match_oracle(dn):
    """Per layer, the device gradient is as close to the FP32 oracle as the BF16-rounding oracle is (a
    wrong kernel or a wrong wiring lands far outside), and close to the BF16-rounding oracle itself.
    Bounds: err(device, fp32) <= 1.5 err(bf16 oracle, fp32) + 0.02; err(device, bf16 oracle) <= 0.1;
    cosine(device, bf16 oracle) >= 0.995 (relative L2 errors)."""
    dn.init(5)
    params = dn.get_params()
    feat, target = random_batch(1, 64, 64, 3)
    loss, grad = dn.gradients(torch.from_numpy(feat).cuda(), torch.from_numpy(target).cuda())
    ref_loss, g16, _ = unet.gradients(params, feat, target, bf16=True)
    _, g32, _ = unet.gradients(params, feat, target, bf16=False)
    assert loss == pytest.approx(ref_loss, rel=1e-2)
    off, rows, bad = 0, [], []
    for li, (cin, cout, _) in enumerate(unet.layer_shapes()):
        nw = cout * 9 * cin
        for name, lo, hi in (("w", off, off + nw), ("b", off + nw, off + nw + cout)):
            d, r16, r32 = (x[lo:hi].astype(np.float64) for x in (grad, g16, g32))
            n32, n16 = np.linalg.norm(r32), np.linalg.norm(r16)
            if n32 == 0 or n16 == 0:
                continue
            e_dev, e_ref = np.linalg.norm(d - r32) / n32, np.linalg.norm(r16 - r32) / n32
            e_16 = np.linalg.norm(d - r16) / n16
            cos = float(d @ r16 / (np.linalg.norm(d) * n16 + 1e-30))
            rows.append(f"{li}{name}: dev-fp32 {e_dev:.4f} bf16ref-fp32 {e_ref:.4f} dev-bf16ref {e_16:.4f} cos {cos:.5f}")
            if not (e_dev <= 1.5 * e_ref + 0.02 and e_16 <= 0.1 and cos >= 0.995):
                bad.append(rows[-1])
        off += nw + cout
    assert off == grad.size
    assert not bad, "\n".join(["failing:"] + bad + ["all:"] + rows)


def test_inference_matches_oracle_forward_with_padding(dn):
    """A 40 x 50 image is padded to 48 x 64 by edge replication: bit-identical to inferring the padded
    image and cropping. Against the BF16-rounding oracle forward: relMSE < 1e-3 and median relative
    error < 1% (an untrained 19-layer network amplifies single BF16 rounding flips, so no per-pixel bound)."""
    dn.init(9)
    params = dn.get_params()
    feat, _ = random_batch(1, 40, 50, 4)
    out = dn.infer(torch.from_numpy(feat).cuda()).cpu().numpy()
    hp, wp = 48, 64
    fp = np.pad(feat, ((0, 0), (0, hp - 40), (0, wp - 50), (0, 0)), mode="edge")
    out_p = dn.infer(torch.from_numpy(np.ascontiguousarray(fp)).cuda()).cpu().numpy()
    assert np.array_equal(out, out_p[:, :40, :50])
    assert np.all(out[..., 3] == 1.0)
    ref_out, _, _ = unet.forward(params, fp, bf16=True)
    ref = unet.decode(ref_out)[:, :40, :50]
    got = out[..., :3]
    relmse = float(np.mean((got - ref) ** 2 / (ref ** 2 + 1e-2)))
    med = float(np.median(np.abs(got - ref) / (np.abs(ref) + 1e-2)))
    assert relmse < 1e-3 and med < 1e-2, (relmse, med)


def test_training_lowers_the_loss(dn):
    dn.init(2)
    feat, target = random_batch(4, 64, 64, 8)
    f, t = torch.from_numpy(feat).cuda(), torch.from_numpy(target).cuda()
    losses = [dn.train_step(f, t, 1e-3) for _ in range(40)]
    assert all(np.isfinite(losses))
    assert losses[-1] < 0.5 * losses[0], losses[::8]
    assert dn.last_ms() > 0


def test_fallback_tiles(dn):
    h, w, tile = 40, 70, 16
    rng = np.random.default_rng(1)
    den = rng.uniform(0.5, 1.0, (h, w, 4)).astype(np.float32)
    plain = rng.uniform(0.5, 1.0, (h, w, 4)).astype(np.float32)
    a = den.copy()
    b = den.copy()
    # disagreement in tile (1, 2) only
    b[16:32, 32:48, :3] += 0.5
    out, count = dn.fallback(*(torch.from_numpy(v).cuda() for v in (den, a, b, plain)), tile=tile, threshold=0.01)
    got = out.cpu().numpy()
    assert count == 1
    np.testing.assert_array_equal(got[16:32, 32:48], plain[16:32, 32:48])
    mask = np.ones((h, w), bool)
    mask[16:32, 32:48] = False
    np.testing.assert_array_equal(got[mask], den[mask])
