"""What the trained network gains: on procedural scenes outside its training and hold-out seeds, rendered
at 4 samples per pixel, the denoised image with the committed weights is scored against a 1024-spp render
by relMSE, next to the plain 4-spp render and the same network untrained.

Bounds (written here): trained relMSE <= 0.25 x plain relMSE, and <= 0.25 x untrained relMSE, averaged
over the scenes."""
import os

import numpy as np
import pytest

from sparkle_gb300 import denoise, native, scenes

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.skipif(not os.path.exists(denoise.WEIGHTS), reason="no trained weights committed")
def test_trained_network_beats_plain_and_untrained():
    ctx = native.Context(0)
    dn = native.Denoiser(0, seed=123)
    size = 128
    plain, trained, untrained = [], [], []
    feats = torch.empty((1, size, size, native.Denoiser.FEATURES), dtype=torch.float32, device="cuda")
    for seed in (90001, 90002, 90003):
        scene, cam_args = scenes.random_training_scene(seed)
        camera = scenes.make_camera(cam_args, size, size)
        ctx.set_scene(scene)
        ctx.set_config(denoise.render_config(size, size, seed=seed))
        ctx.set_camera(camera)
        ctx.render(4)
        hdr = denoise.framebuffer_tensor(ctx)
        nd, al = denoise.guides_tensors(ctx)
        dn.pack_features(hdr[None], nd[None], al[None], feats)
        ctx.set_config(denoise.render_config(size, size, seed=seed + 500000))
        ctx.set_camera(camera)
        ctx.render(1024)
        ref, _ = ctx.framebuffer()
        dn.init(123)
        untrained.append(denoise.relmse(dn.infer(feats)[0].cpu().numpy(), ref))
        denoise.load_weights(dn)
        trained.append(denoise.relmse(dn.infer(feats)[0].cpu().numpy(), ref))
        plain.append(denoise.relmse(hdr.cpu().numpy(), ref))
    p, t, u = np.mean(plain), np.mean(trained), np.mean(untrained)
    print(f"relMSE vs 1024 spp: plain 4 spp {p:.4f}, untrained {u:.4f}, trained {t:.4f}")
    assert t <= 0.25 * p and t <= 0.25 * u, (p, t, u)
    dn.close()
    ctx.close()


@pytest.mark.skipif(not os.path.exists(denoise.WEIGHTS), reason="no trained weights committed")
def test_trained_network_on_an_out_of_family_scene():
    """The Cornell box is nothing like the training scenes (a closed room lit by one small area light, no
    sky, inward-facing walls): the trained network must still cut the plain 4-spp render's relMSE at least
    four times there (measured: 0.166 -> 0.013)."""
    ctx = native.Context(0)
    dn = native.Denoiser(0, seed=123)
    size = 128
    feats = torch.empty((1, size, size, native.Denoiser.FEATURES), dtype=torch.float32, device="cuda")
    scene, cam_args = scenes.cornell_box(0)
    camera = scenes.make_camera(cam_args, size, size)
    ctx.set_scene(scene)
    ctx.set_config(denoise.render_config(size, size, seed=4242, bounce=5))
    ctx.set_camera(camera)
    ctx.render(4)
    hdr = denoise.framebuffer_tensor(ctx)
    nd, al = denoise.guides_tensors(ctx)
    dn.pack_features(hdr[None], nd[None], al[None], feats)
    ctx.set_config(denoise.render_config(size, size, seed=4243, bounce=5))
    ctx.set_camera(camera)
    ctx.render(1024)
    ref, _ = ctx.framebuffer()
    untrained = denoise.relmse(dn.infer(feats)[0].cpu().numpy(), ref)
    denoise.load_weights(dn)
    trained = denoise.relmse(dn.infer(feats)[0].cpu().numpy(), ref)
    plain = denoise.relmse(hdr.cpu().numpy(), ref)
    print(f"Cornell box relMSE vs 1024 spp: plain 4 spp {plain:.4f}, untrained {untrained:.4f}, trained {trained:.4f}")
    assert trained <= 0.25 * plain and trained < untrained, (plain, trained, untrained)
    dn.close()
    ctx.close()
