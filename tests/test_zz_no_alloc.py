"""spk_render_noalloc, the entry point for callers that cannot allocate device memory while they render (a
frame loop that must not stall on the allocator, code running under stream capture, a host whose memory is
already reserved by its own pool). It renders into buffers the caller owns and keeps its scratch in a static
device array, so:

* its output must equal spk_render's with the one-kernel schedule -- checked bit for bit on two calls in a
  row (a fresh accumulation, then a continued one) -- while the library's allocation hook stays armed and
  untouched (the hook then fails the next allocation another call makes, which shows it would have caught
  one here);
* the sample bookkeeping follows one frame buffer: switching between the context's buffer and caller
  buffers starts the accumulation over, and the context's own buffer is not handed out while it is stale;
* the walk's error flags reach spk_get_stats;
* configs larger than the array are refused.

This file is collected last on purpose."""
import numpy as np
import pytest
import torch

from sparkle_gb300 import abi, native, scenes

pytestmark = pytest.mark.gpu

W, H = 64, 48


def _setup(cornell, kernel=abi.SPK_KERNEL_MEGAKERNEL):
    scene, cam_args = cornell
    camera = scenes.make_camera(cam_args, W, H)
    ctx = native.Context(0)
    ctx.set_scene(scene)
    ctx.set_config(abi.make_config(W, H, spp=1, bounce=5, rng=abi.SPK_RNG_XOSHIRO256SS, seed=9, kernel=kernel))
    ctx.set_camera(camera)
    return ctx, camera


def _buffers():
    hdr = torch.full((H, W, 4), float("nan"), dtype=torch.float32, device="cuda")
    out = torch.zeros((H, W, 4), dtype=torch.int16, device="cuda")
    return hdr, out


def _host(hdr, out):
    torch.cuda.synchronize()
    return hdr.cpu().numpy(), out.cpu().numpy().view(np.uint16)


def _same(got, ref):
    return np.array_equal(got[0].view(np.uint32), ref[0].view(np.uint32)) and np.array_equal(got[1], ref[1])


def test_noalloc_render_matches_spk_render_without_allocating(cornell):
    ctx, camera = _setup(cornell)
    # a second context, made ready before the hook is armed: its first wavefront render allocates path state
    other, other_cam = _setup(cornell, kernel=abi.SPK_KERNEL_WAVEFRONT)
    try:
        # existing entry point: 3 frames, then 6 frames from a fresh accumulation
        ctx.render(3)
        ref3 = ctx.framebuffer()
        ctx.set_camera(camera)
        ctx.render(6)
        ref6 = ctx.framebuffer()
        hdr, out = _buffers()
        ctx.set_camera(camera)
        native.debug_fail_allocation(1)  # the next device allocation of the library fails
        try:
            # call 1 renders 3 frames from a fresh accumulation, call 2 adds 3 more
            ctx.render_noalloc(3, hdr.data_ptr(), out.data_ptr())
            got3 = _host(hdr, out)
            assert ctx.sample_counts() == (2, 3)
            ctx.render_noalloc(3, hdr.data_ptr(), out.data_ptr())
            got6 = _host(hdr, out)
            assert ctx.sample_counts() == (5, 6)
            st = ctx.stats()
            assert st["error_flags"] == 0 and st["extension_rays"] >= 3 * W * H and st["kernel_launches"] == 6
            # the hook is still armed: the other context's first render allocates and gets the failure
            with pytest.raises(native.SpkError):
                other.render(1)
        finally:
            native.debug_fail_allocation(0)
        assert _same(got3, ref3) and _same(got6, ref6)
        other.set_camera(other_cam)
        other.render(1)  # and renders once the hook is disarmed
    finally:
        ctx.close()
        other.close()


def test_noalloc_and_spk_render_restart_each_others_accumulation(cornell):
    ctx, camera = _setup(cornell)
    try:
        ctx.render(3)
        fresh = ctx.framebuffer()
        # spk_render, then noalloc into a caller buffer: the caller buffer starts from zero
        a_hdr, a_out = _buffers()
        ctx.render_noalloc(3, a_hdr.data_ptr(), a_out.data_ptr())
        assert _same(_host(a_hdr, a_out), fresh)
        assert ctx.sample_counts() == (2, 3)
        # the context's own buffer does not hold those frames: reading it is refused
        with pytest.raises(native.SpkError, match="spk_render_noalloc"):
            ctx.framebuffer()
        # another caller buffer starts over too
        b_hdr, b_out = _buffers()
        ctx.render_noalloc(3, b_hdr.data_ptr(), b_out.data_ptr())
        assert _same(_host(b_hdr, b_out), fresh)
        # and spk_render afterwards starts over in the context's buffer
        ctx.render(3)
        assert _same(ctx.framebuffer(), fresh)
        assert ctx.sample_counts() == (2, 3)
    finally:
        ctx.close()


def test_noalloc_reports_walk_errors(cornell):
    ctx, _ = _setup(cornell)
    try:
        hdr, out = _buffers()
        ctx.debug_walk_budget(2)  # every walk may take two node steps: most run out
        ctx.render_noalloc(1, hdr.data_ptr(), out.data_ptr())
        assert ctx.stats()["error_flags"] & 2  # iteration budget
        ctx.debug_walk_budget(0)
        ctx.render_noalloc(1, hdr.data_ptr(), out.data_ptr())
        assert ctx.stats()["error_flags"] == 0
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
