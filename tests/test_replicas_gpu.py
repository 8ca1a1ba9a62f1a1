"""Replicas on the device: contexts that render consecutive frames of one view from their own sample
offsets (spk_config.sample_offset) merge, by the sample-weighted mean of their frame buffers, to the image one
context renders with all the frames -- on both schedules and both generators -- and an offset render matches
the oracle rendering the same frames (parity tolerances of tests/parity.py)."""
import numpy as np
import pytest

from sparkle_gb300 import abi, native, replicas, scenes

from parity import assert_image_parity, compare_images, oracle_image

pytestmark = pytest.mark.gpu

FRAMES = (5, 3, 8)  # uneven frames per replica


def _render(scene, camera, cfg, frames):
    ctx = native.Context(0)
    try:
        ctx.set_scene(scene)
        ctx.set_config(cfg)
        ctx.set_camera(camera)
        ctx.render(frames)
        assert ctx.stats()["error_flags"] == 0
        return ctx.framebuffer()
    finally:
        ctx.close()


@pytest.mark.parametrize("kernel", [abi.SPK_KERNEL_WAVEFRONT, abi.SPK_KERNEL_MEGAKERNEL])
@pytest.mark.parametrize("rng", [abi.SPK_RNG_XOSHIRO128P, abi.SPK_RNG_XOSHIRO256SS])
def test_replicas_merge_to_one_renderer(small_terrain, kernel, rng):
    scene, cam_args = small_terrain
    W, H = 64, 48
    camera = scenes.make_camera(cam_args, W, H)
    parts, offset = [], 0
    for frames in FRAMES:
        cfg = abi.make_config(W, H, spp=1, bounce=6, rng=rng, seed=3, kernel=kernel, sample_offset=offset)
        parts.append((_render(scene, camera, cfg, frames)[0].astype(np.float64), frames))
        offset += frames
    merged = sum(h * f for h, f in parts) / sum(FRAMES)
    whole, _ = _render(scene, camera, abi.make_config(W, H, spp=1, bounce=6, rng=rng, seed=3, kernel=kernel),
                       sum(FRAMES))
    np.testing.assert_allclose(merged.astype(np.float32), whole, rtol=2e-5, atol=1e-6)
    assert not np.array_equal(parts[0][0], parts[1][0])  # disjoint samples


def test_offset_render_matches_oracle(small_terrain):
    scene, cam_args = small_terrain
    W, H, frames = 64, 48, 4
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=6, rng=abi.SPK_RNG_XOSHIRO128P, seed=0,
                          sample_offset=replicas.replica_sample_offset(3, frames))
    hdr, out = _render(scene, camera, cfg, frames)
    o_hdr, o_out = oracle_image(scene, camera, cfg, frames)
    assert_image_parity(compare_images(hdr, out, o_hdr, o_out), "offset render vs oracle")
