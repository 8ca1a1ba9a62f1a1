"""Next-event estimation (not part of the reference cpu pipeline; its GPU shader samples only the sky): the
device schedules match the CPU oracle's NEE on the same seeds, and NEE converges to the plain path tracer.

Tolerances: the image parity of tests/parity.py against the oracle after a few frames (>= 99.5% of pixels
within 1e-4 relative, relMSE < 1e-4, tonemapped pixels bit-identical where the frame buffer is); converged
NEE vs plain (bounce limit lifted, emission below the 6.0 sample clamp) mean within 0.5% and relMSE < 2e-4."""
import numpy as np
import pytest

import oracle
from sparkle_gb300 import abi, native, scenes

from parity import assert_image_parity, compare_images, rel_mse

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


def render_gpu(ctx, scene, camera, cfg, frames):
    ctx.set_scene(scene)
    ctx.set_config(cfg)
    ctx.set_camera(camera)
    ctx.render(frames)
    st = ctx.stats()
    assert st["error_flags"] == 0, st
    hdr, out = ctx.framebuffer()
    return hdr, st, out


@pytest.mark.parametrize("kernel,spatial", [(abi.SPK_KERNEL_MEGAKERNEL, False), (abi.SPK_KERNEL_WAVEFRONT, False),
                                            (abi.SPK_KERNEL_WAVEFRONT, True)])
def test_cornell_nee_matches_oracle(ctx, cornell, kernel, spatial):
    scene, cam_args = cornell
    W, H, frames = 48, 40, 4
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=5, enable_nee=True, spatial_denoise=spatial,
                          rng=abi.SPK_RNG_XOSHIRO256SS, seed=3, kernel=kernel)
    g, st, g_out = render_gpu(ctx, scene, camera, cfg, frames)
    r = oracle.OracleRenderer(oracle.OracleScene(scene), cfg, camera)
    r.render(frames, traversal=oracle.PRUNED)
    o, o_out = r.framebuffer()
    ext, shadow, _ = r.counts()
    print(f"kernel={kernel} spatial={spatial} shadow gpu={st['shadow_rays']} oracle={shadow}")
    assert shadow > 0 and abs(st["shadow_rays"] - shadow) <= 0.02 * shadow
    assert_image_parity(compare_images(g, g_out, o, o_out), f"cornell nee kernel={kernel} spatial={spatial}")


def test_sky_nee_matches_oracle(ctx, small_terrain):
    scene, cam_args = small_terrain
    W, H, frames = 64, 48, 2
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=6, enable_nee=True, rng=abi.SPK_RNG_XOSHIRO256SS, seed=1)
    g, st, g_out = render_gpu(ctx, scene, camera, cfg, frames)
    r = oracle.OracleRenderer(oracle.OracleScene(scene), cfg, camera)
    r.render(frames, traversal=oracle.PRUNED)
    o, o_out = r.framebuffer()
    assert st["shadow_rays"] > 0
    assert_image_parity(compare_images(g, g_out, o, o_out), "sky nee")


def test_nee_is_unbiased_and_reduces_noise(ctx, cornell):
    scene, cam_args = cornell
    scene = abi.Scene(scene.meshes, scene.instances, list(scene.materials), scene.sky)
    scene.materials[7] = abi.Material.light((2.0, 2.0, 2.0))  # below the 6.0 sample clamp
    W, H = 32, 32
    camera = scenes.make_camera(cam_args, W, H)
    img = {}
    for nee in (False, True):
        for seed in (1, 2):
            cfg = abi.make_config(W, H, spp=1, max_spp=1 << 20, bounce=24, enable_nee=nee,
                                  rng=abi.SPK_RNG_XOSHIRO256SS, seed=seed)
            img[(nee, seed)] = render_gpu(ctx, scene, camera, cfg, 16384)[0][..., :3].astype(np.float64)
    plain = 0.5 * (img[(False, 1)] + img[(False, 2)])
    nee = 0.5 * (img[(True, 1)] + img[(True, 2)])
    noise_plain = rel_mse(img[(False, 1)], img[(False, 2)])
    noise_nee = rel_mse(img[(True, 1)], img[(True, 2)])
    ratio = nee.mean() / plain.mean()
    print(f"mean ratio {ratio:.5f} relmse nee-plain {rel_mse(nee, plain):.2e} noise plain {noise_plain:.2e} "
          f"nee {noise_nee:.2e}")
    assert abs(ratio - 1.0) < 5e-3
    assert rel_mse(nee, plain) < 2e-4
    assert noise_nee < 0.25 * noise_plain


@pytest.mark.parametrize("spatial", [False, True])
def test_shadow_stage_equals_inline_walks(ctx, small_terrain, cornell, spatial):
    """The wavefront's shadow stage (occlusion rays queued by shade, walked by their own persistent kernel,
    radiance added light before sky) renders the same bits as walking them inline in the shade kernel and
    as the one-kernel schedule, with the same shadow-ray count, on the frame-by-frame (spatial fill) and the
    multi-frame schedules; sky NEE on the terrain, triangle lights and sky-less on the Cornell box."""
    for scene, cam_args in (small_terrain, cornell):
        W, H = 64, 48
        camera = scenes.make_camera(cam_args, W, H)
        res = []
        for kernel, stage in ((abi.SPK_KERNEL_WAVEFRONT, 1), (abi.SPK_KERNEL_WAVEFRONT, 0),
                              (abi.SPK_KERNEL_MEGAKERNEL, 1)):
            ctx.set_tuning(shadow_stage=stage)
            cfg = abi.make_config(W, H, spp=1, bounce=6, enable_nee=True, spatial_denoise=spatial,
                                  rng=abi.SPK_RNG_XOSHIRO256SS, seed=4, kernel=kernel)
            g, st, out = render_gpu(ctx, scene, camera, cfg, 5)
            res.append((g, out, st["shadow_rays"], st["extension_rays"]))
        ctx.set_tuning(shadow_stage=1)
        assert res[0][2] > 0
        for g, out, shadow, ext in res[1:]:
            assert np.array_equal(g.view(np.uint32), res[0][0].view(np.uint32))
            assert np.array_equal(out, res[0][1])
            assert (shadow, ext) == (res[0][2], res[0][3])
