"""spk_render_noalloc, the entry point for callers that cannot allocate device memory while they render (a
frame loop that must not stall on the allocator, code running under stream capture, a host whose memory is
already reserved by its own pool). It renders into buffers the caller owns and keeps its scratch in a static
device array, so its output must equal spk_render's with the one-kernel schedule -- checked bit for bit on
two calls in a row (a fresh accumulation, then a continued one) -- and configs larger than the array must be
refused. This file is collected last on purpose."""
import numpy as np
import pytest
import torch

from sparkle_gb300 import abi, native, scenes

pytestmark = pytest.mark.gpu


def test_noalloc_render_matches_spk_render(cornell):
    scene, cam_args = cornell
    W, H = 64, 48
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=5, rng=abi.SPK_RNG_XOSHIRO256SS, seed=9,
                          kernel=abi.SPK_KERNEL_MEGAKERNEL)
    ctx = native.Context(0)
    try:
        ctx.set_scene(scene)
        ctx.set_config(cfg)
        # existing entry point: 3 frames, then 6 frames from a fresh accumulation
        ctx.set_camera(camera)
        ctx.render(3)
        ref3 = ctx.framebuffer()
        ctx.set_camera(camera)
        ctx.render(6)
        ref6 = ctx.framebuffer()
        # the no-allocation entry point: call 1 renders 3 frames from a fresh accumulation, call 2 adds 3 more
        hdr = torch.full((H, W, 4), float("nan"), dtype=torch.float32, device="cuda")
        out = torch.zeros((H, W, 4), dtype=torch.int16, device="cuda")
        ctx.set_camera(camera)
        ctx.render_noalloc(3, hdr.data_ptr(), out.data_ptr())
        ctx.synchronize()
        got3 = (hdr.cpu().numpy(), out.cpu().numpy().view(np.uint16))
        assert ctx.sample_counts() == (2, 3)
        ctx.render_noalloc(3, hdr.data_ptr(), out.data_ptr())
        ctx.synchronize()
        got6 = (hdr.cpu().numpy(), out.cpu().numpy().view(np.uint16))
        assert ctx.sample_counts() == (5, 6)
        for got, ref in ((got3, ref3), (got6, ref6)):
            assert np.array_equal(got[0].view(np.uint32), ref[0].view(np.uint32))
            assert np.array_equal(got[1], ref[1])
    finally:
        ctx.close()


def test_noalloc_rejects_configs_beyond_its_array(cornell):
    scene, cam_args = cornell
    ctx = native.Context(0)
    try:
        ctx.set_scene(scene)
        ctx.set_config(abi.make_config(1024, 512, spp=1, bounce=2))
        ctx.set_camera(scenes.make_camera(cam_args, 1024, 512))
        hdr = torch.zeros((512, 1024, 4), dtype=torch.float32, device="cuda")
        out = torch.zeros((512, 1024, 4), dtype=torch.int16, device="cuda")
        with pytest.raises(native.SpkError, match="at most 262144 pixels"):
            ctx.render_noalloc(1, hdr.data_ptr(), out.data_ptr())
    finally:
        ctx.close()
