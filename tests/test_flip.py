"""Image evaluators: the device LDR-FLIP (spk_flip) against the float64 restatement in oracle/flip.py, the
device relMSE against numpy, and the reference's screenshot comparison flow (PNG in, mean FLIP out).

FLIP is floating point: per-pixel errors within 2e-4 (absolute, errors lie in [0, 1]) and means within
2e-5 of the float64 oracle."""
import numpy as np
import pytest

from oracle import flip as oflip


def structured(h, w, seed):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w] / max(h, w)
    img = np.stack([0.5 + 0.5 * np.sin(9 * xx), yy, 0.3 + 0.2 * np.cos(13 * xx * yy)], -1)
    img[h // 3: h // 2, w // 4: w // 2] = [0.9, 0.1, 0.1]  # a hard-edged block
    img += rng.normal(0, 0.02, img.shape)
    return np.clip(img, 0, 1)


def test_oracle_kernels_and_limits():
    for ch in ("A", "RG", "BY"):
        k = oflip.spatial_kernel(ch, oflip.PPD)
        assert k.shape == (21, 21) and abs(k.sum() - 1) < 1e-12 and np.allclose(k, k.T)
    for k in oflip.feature_kernels(oflip.PPD):
        assert k.shape == (19, 19)
        assert abs(k[k > 0].sum() - 1) < 1e-12 and abs(k[k < 0].sum() + 1) < 1e-12
    a = structured(24, 32, 1)
    assert oflip.flip_mean(a, a) == 0.0
    black, white = np.zeros((16, 16, 3)), np.ones((16, 16, 3))
    assert 0.96 < oflip.flip_mean(black, white) < 0.975  # colour error near its top, no features
    noisy = [oflip.flip_mean(a, np.clip(a + np.random.default_rng(2).normal(0, s, a.shape), 0, 1))
             for s in (0.01, 0.05, 0.2)]
    assert noisy[0] < noisy[1] < noisy[2]


@pytest.mark.gpu
@pytest.mark.parametrize("h,w,ppd", [(48, 64, oflip.PPD), (37, 53, oflip.PPD), (40, 40, 30.0)])
def test_device_flip_matches_oracle(h, w, ppd):
    from sparkle_gb300 import evaluate
    ref = structured(h, w, 3)
    rng = np.random.default_rng(4)
    test = np.clip(ref + rng.normal(0, 0.06, ref.shape), 0, 1)
    test[5:9, 5:30] = 0.0  # a dark stroke: feature differences
    mean, emap = evaluate.flip(ref, test, pixels_per_degree=ppd, return_map=True)
    omap = oflip.flip_map(ref.astype(np.float32).astype(np.float64), test.astype(np.float32).astype(np.float64), ppd)
    assert np.max(np.abs(emap - omap)) < 2e-4
    assert abs(mean - omap.mean()) < 2e-5
    assert evaluate.flip(ref, ref) == 0.0


@pytest.mark.gpu
def test_device_relmse_and_compare_images(tmp_path, cornell):
    from sparkle_gb300 import abi, evaluate, native, scenes
    rng = np.random.default_rng(5)
    x = rng.lognormal(0, 1, 100_003).astype(np.float32)
    r = rng.lognormal(0, 1, 100_003).astype(np.float32)
    ref = np.mean((x.astype(np.float64) - r) ** 2 / (r.astype(np.float64) ** 2 + 0.01))
    assert abs(evaluate.rel_mse(x, r) - ref) < 1e-6 * ref  # fp32 terms, float64 sum
    # the reference's screenshot test flow: two renders at different sample counts written as PNGs
    scene, cam_args = cornell
    W, H = 96, 72
    shots = []
    for frames in (2, 64):
        ctx = native.Context(0)
        ctx.set_scene(scene)
        ctx.set_config(abi.make_config(W, H, spp=1, bounce=5, seed=7))
        ctx.set_camera(scenes.make_camera(cam_args, W, H))
        ctx.render(frames)
        p = tmp_path / f"shot{frames}.png"
        ctx.save_image(p, abi.SPK_IMAGE_PNG)
        shots.append((p, ctx.read_rgba8()))
        ctx.close()
    score = evaluate.compare_images(shots[1][0], shots[0][0])
    a = shots[1][1][..., :3] / np.float32(255)
    b = shots[0][1][..., :3] / np.float32(255)
    assert abs(score - oflip.flip_mean(a.astype(np.float64), b.astype(np.float64))) < 2e-5
    assert 0.01 < score < 0.5
    assert evaluate.compare_images(shots[1][0], shots[1][0]) == 0.0
