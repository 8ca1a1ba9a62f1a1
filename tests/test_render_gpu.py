"""Image parity of the device BasePass/DenoisePass/ToneMappingPass (spk_render through the C ABI) against the
CPU oracle on the same scenes, cameras and per-pixel seeds.

The device and the oracle draw the same random numbers in the same order and round every multiply and
add the same way; they differ only in the last bits of cosf/sinf/powf, so a path can occasionally take
another branch (a Fresnel or roulette coin lands on the other side). Tolerances (tests/parity.py, per
image): >= 99.5% of pixels agree to 1e-4 relative, relMSE < 1e-3 for renders of at most 16 frames and
< 1e-4 for converged renders (256 frames), and every pixel whose frame-buffer value is bit-identical has a
bit-identical tonemapped RGBA16F pixel (ACES, clamp, vertical flip, RNE half); the counts of identical and
differing pixels are printed. The one-kernel and wavefront schedules are bit-identical to each other.
"""
import numpy as np
import pytest

import oracle
from sparkle_gb300 import abi, native, scenes

from parity import MAX_RELMSE_CONVERGED, assert_image_parity, close_fraction, compare_images, rel_mse

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


def gpu_render(ctx, scene, camera, cfg, frames):
    ctx.set_scene(scene)
    ctx.set_config(cfg)
    ctx.set_camera(camera)
    ctx.render(frames)
    hdr, out = ctx.framebuffer()
    st = ctx.stats()
    assert st["error_flags"] == 0, st
    return hdr, out, st


def oracle_render(scene, camera, cfg, frames, osc=None):
    osc = osc or oracle.OracleScene(scene)
    r = oracle.OracleRenderer(osc, cfg, camera)
    r.render(frames, traversal=oracle.PRUNED)
    hdr, out = r.framebuffer()
    return hdr, out, r


@pytest.mark.parametrize("rng", [abi.SPK_RNG_XOSHIRO128P, abi.SPK_RNG_XOSHIRO256SS])
@pytest.mark.parametrize("spatial", [False, True])
def test_cornell_matches_oracle(ctx, cornell, rng, spatial):
    scene, cam_args = cornell
    W, H, frames = 64, 48, 4
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=5, spatial_denoise=spatial, rng=rng, seed=7)
    g_hdr, g_out, st = gpu_render(ctx, scene, camera, cfg, frames)
    o_hdr, o_out, r = oracle_render(scene, camera, cfg, frames)
    assert_image_parity(compare_images(g_hdr, g_out, o_hdr, o_out), f"cornell rng={rng} spatial={spatial}")
    assert ctx.sample_counts() == r.sample_counts()
    # accumulated validity channel and the tonemapped alpha
    assert np.all(g_out[..., 3] == 0x3C00)
    ext_o = r.counts()[0]
    assert abs(st["extension_rays"] - ext_o) <= 0.02 * ext_o


@pytest.mark.parametrize("rng,spatial", [(abi.SPK_RNG_XOSHIRO128P, False), (abi.SPK_RNG_XOSHIRO256SS, False),
                                         (abi.SPK_RNG_XOSHIRO128P, True)])
def test_cornell_full_size_matches_oracle(ctx, cornell, rng, spatial):
    """The Cornell workload at its stated size: 256x256, 16 frames of 1 spp, depth 5, against the oracle on
    the same seeds (both generators without the spatial DenoisePass; the reference generator with it,
    as the reference's default pipeline runs); then the same accumulation continued to 256 frames, where
    the two converged renders must agree to relMSE < 1e-4."""
    scene, cam_args = cornell
    W, H, frames = 256, 256, 16
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=5, spatial_denoise=spatial, rng=rng, seed=0)
    g_hdr, g_out, st = gpu_render(ctx, scene, camera, cfg, frames)
    o_hdr, o_out, r = oracle_render(scene, camera, cfg, frames)
    assert_image_parity(compare_images(g_hdr, g_out, o_hdr, o_out), f"cornell 256x256x16 rng={rng} spatial={spatial}")
    assert ctx.sample_counts() == r.sample_counts() == (15, 16)
    ext_o = r.counts()[0]
    assert abs(st["extension_rays"] - ext_o) <= 0.01 * ext_o
    ctx.render(256 - frames)
    r.render(256 - frames, traversal=oracle.PRUNED)
    g_hdr, g_out = ctx.framebuffer()
    o_hdr, o_out = r.framebuffer()
    assert ctx.sample_counts() == r.sample_counts() == (255, 256)
    assert_image_parity(compare_images(g_hdr, g_out, o_hdr, o_out), f"cornell 256x256x256 rng={rng} spatial={spatial}",
                        min_close=0.9, max_relmse=MAX_RELMSE_CONVERGED)


@pytest.mark.parametrize("spatial", [False, True])
def test_wavefront_equals_megakernel(ctx, small_terrain, spatial):
    scene, cam_args = small_terrain
    W, H = 96, 64
    camera = scenes.make_camera(cam_args, W, H)
    outs = []
    for kernel in (abi.SPK_KERNEL_MEGAKERNEL, abi.SPK_KERNEL_WAVEFRONT):
        cfg = abi.make_config(W, H, spp=1, bounce=8, spatial_denoise=spatial, rng=abi.SPK_RNG_XOSHIRO256SS,
                              kernel=kernel)
        hdr, out, st = gpu_render(ctx, scene, camera, cfg, 3)
        outs.append((hdr, out, st["extension_rays"]))
    assert np.array_equal(outs[0][0].view(np.uint32), outs[1][0].view(np.uint32))
    assert np.array_equal(outs[0][1], outs[1][1])
    assert outs[0][2] == outs[1][2]


def test_terrain_matches_oracle(ctx, small_terrain):
    scene, cam_args = small_terrain
    W, H, frames = 80, 60, 2
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=8, rng=abi.SPK_RNG_XOSHIRO256SS, kernel=abi.SPK_KERNEL_WAVEFRONT)
    g_hdr, g_out, _ = gpu_render(ctx, scene, camera, cfg, frames)
    o_hdr, o_out, _ = oracle_render(scene, camera, cfg, frames)
    assert_image_parity(compare_images(g_hdr, g_out, o_hdr, o_out), "terrain")


def test_converged_cornell_relmse(ctx, cornell):
    scene, cam_args = cornell
    W, H, frames = 48, 48, 256
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=5, rng=abi.SPK_RNG_XOSHIRO256SS, kernel=abi.SPK_KERNEL_WAVEFRONT)
    g_hdr, _, _ = gpu_render(ctx, scene, camera, cfg, frames)
    o_hdr, _, _ = oracle_render(scene, camera, cfg, frames)
    rm = rel_mse(g_hdr, o_hdr)
    print(f"converged relmse={rm:.3e}")
    assert rm < 1e-4


@pytest.mark.parametrize("kernel", [abi.SPK_KERNEL_MEGAKERNEL, abi.SPK_KERNEL_WAVEFRONT])
def test_accumulation_cap_and_reset(ctx, cornell, kernel):
    """max_spp caps the cumulated count (then the lerp becomes an EMA); a camera change clears. Frames split
    over several calls accumulate exactly like one call."""
    scene, cam_args = cornell
    W, H = 16, 16
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, max_spp=3, bounce=3, rng=abi.SPK_RNG_XOSHIRO256SS, kernel=kernel)
    hdr6, _, _ = gpu_render(ctx, scene, camera, cfg, 6)
    r = oracle.OracleRenderer(oracle.OracleScene(scene), cfg, camera)
    r.render(6, traversal=oracle.PRUNED)
    assert ctx.sample_counts() == r.sample_counts() == (3, 6)
    assert ctx.is_converged()
    o_hdr, _ = r.framebuffer()
    assert close_fraction(hdr6, o_hdr) >= 0.99
    ctx.set_camera(camera)
    ctx.render(2)
    ctx.render(4)
    split, _ = ctx.framebuffer()
    assert np.array_equal(split.view(np.uint32), hdr6.view(np.uint32))
    ctx.set_camera(camera)
    ctx.render(1)
    assert ctx.sample_counts() == (0, 1)


def test_full_hd_frame_is_consistent(ctx):
    """One 1920x1080 frame of the stress scene, both schedules: identical images and ray counts, no
    device error flags, finite output."""
    scene, cam_args = scenes.terrain_spheres(0)
    W, H = 1920, 1080
    camera = scenes.make_camera(cam_args, W, H)
    res = []
    for kernel in (abi.SPK_KERNEL_MEGAKERNEL, abi.SPK_KERNEL_WAVEFRONT):
        cfg = abi.make_config(W, H, spp=1, bounce=8, rng=abi.SPK_RNG_XOSHIRO256SS, kernel=kernel)
        hdr, out, st = gpu_render(ctx, scene, camera, cfg, 1)
        assert np.all(np.isfinite(hdr))
        res.append((hdr, st["extension_rays"]))
    assert np.array_equal(res[0][0].view(np.uint32), res[1][0].view(np.uint32))
    assert res[0][1] == res[1][1]
    assert res[0][1] >= W * H


def test_full_hd_stress_rows_match_oracle(ctx):
    """The benchmark workload itself (stress scene, 1920x1080, depth 8, xoshiro256**, seed 0) rendered for
    4 frames in one call (the multi-frame wavefront schedule the benchmark times); the oracle renders
    three bands of rows of the same frames (rows are independent without the spatial DenoisePass). Same
    tolerances as the small scenes, per band, tonemapped pixels included."""
    scene, cam_args = scenes.terrain_spheres(0)
    W, H, frames = 1920, 1080, 4
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=8, rng=abi.SPK_RNG_XOSHIRO256SS, seed=0,
                          kernel=abi.SPK_KERNEL_WAVEFRONT)
    g_hdr, g_out, _ = gpu_render(ctx, scene, camera, cfg, frames)
    osc = oracle.OracleScene(scene)
    for r0, r1 in ((0, 6), (H // 2 - 4, H // 2 + 4), (H - 6, H)):
        r = oracle.OracleRenderer(osc, cfg, camera)
        r.render(frames, traversal=oracle.PRUNED, rows=(r0, r1))
        o_hdr, o_out = r.framebuffer()
        res = compare_images(g_hdr[r0:r1], g_out[H - r1:H - r0], o_hdr[r0:r1], o_out[H - r1:H - r0])
        assert_image_parity(res, f"stress rows {r0}-{r1}")
    assert np.all(g_out[..., 3] == 0x3C00)
