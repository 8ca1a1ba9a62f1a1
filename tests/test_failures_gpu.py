"""Checkpoint / resume and failure handling, tested without any GPU fault.

* A render checkpoint (frame buffer, output image, CameraRenderProxy / CPURenderer sample bookkeeping)
  resumes bit for bit on every schedule; a checkpoint of another config is refused.
* A denoiser training checkpoint (parameters, Adam moments, step) resumes training.
* Host-side fault injection: a device allocation made to fail (spk_debug_fail_allocation) is reported as
  SPK_ERR_OUT_OF_MEMORY by the entry point that made it, and the context or denoiser stays usable.
* Device-side bounds: a walk budget that runs out sets the iteration-budget flag and ends the walk; an
  mbarrier wait that nothing completes gives up after its 1 s limit and reports the time-out bit.
"""
import time

import numpy as np
import pytest

from sparkle_gb300 import abi, native, scenes
from oracle import unet

pytestmark = pytest.mark.gpu

OOM, DEVICE_LIMIT = 3, 5


def setup(ctx, scene_cam, W, H, **cfg):
    scene, cam_args = scene_cam
    ctx.set_scene(scene)
    ctx.set_config(abi.make_config(W, H, **cfg))
    ctx.set_camera(scenes.make_camera(cam_args, W, H))


@pytest.mark.parametrize("kw", [dict(kernel=abi.SPK_KERNEL_WAVEFRONT), dict(kernel=abi.SPK_KERNEL_MEGAKERNEL),
                                dict(kernel=abi.SPK_KERNEL_WAVEFRONT, spatial_denoise=1),
                                dict(kernel=abi.SPK_KERNEL_WAVEFRONT, enable_nee=True, spp=4)])
def test_render_checkpoint_resumes_bit_for_bit(cornell, kw):
    cfg = dict(dict(spp=1, bounce=5, seed=3, max_spp=64), **kw)
    a = native.Context(0)
    setup(a, cornell, 48, 40, **cfg)
    a.render(5)
    ckpt = a.save_checkpoint()
    a.render(7)
    ref_hdr, ref_out = a.framebuffer()
    b = native.Context(0)
    setup(b, cornell, 48, 40, **cfg)
    b.load_checkpoint(ckpt)
    hdr0, _ = b.framebuffer()
    b.render(7)
    hdr, out = b.framebuffer()
    assert np.array_equal(hdr.view(np.uint32), ref_hdr.view(np.uint32))
    assert np.array_equal(out, ref_out)
    assert b.sample_counts() == a.sample_counts()
    assert not np.array_equal(hdr0, hdr)  # the load restored the 5-frame state, the renders went on
    # the same state cannot be loaded into another config
    c = native.Context(0)
    setup(c, cornell, 48, 40, **dict(cfg, seed=4))
    with pytest.raises(native.SpkError):
        c.load_checkpoint(ckpt)
    with pytest.raises(native.SpkError):
        c.load_checkpoint(ckpt[:100])
    for x in (a, b, c):
        x.close()


def test_allocation_failures_are_reported_and_recovered(cornell, small_terrain):
    ctx = native.Context(0)
    for nth in (1, 2, 5):
        native.debug_fail_allocation(nth)
        with pytest.raises(native.SpkError) as e:
            ctx.set_scene(small_terrain[0])
        assert e.value.status == OOM
    native.debug_fail_allocation(0)
    setup(ctx, cornell, 32, 24, spp=1, bounce=4, seed=1)
    ctx.render(2)
    good, _ = ctx.framebuffer()
    native.debug_fail_allocation(1)
    with pytest.raises(native.SpkError) as e:
        ctx.set_config(abi.make_config(64, 48, spp=1, bounce=4, seed=1))
    assert e.value.status == OOM
    setup(ctx, cornell, 32, 24, spp=1, bounce=4, seed=1)  # usable again: same image as before
    ctx.render(2)
    assert np.array_equal(ctx.framebuffer()[0], good)
    ctx.set_tuning(bvh_builder=1)  # the device BVH builder's scratch
    native.debug_fail_allocation(3)
    with pytest.raises(native.SpkError) as e:
        ctx.set_scene(small_terrain[0])
    assert e.value.status == OOM
    ctx.set_scene(cornell[0])
    ctx.render(2)
    assert np.array_equal(ctx.framebuffer()[0], good)
    native.debug_fail_allocation(0)
    ctx.close()


def test_walk_budget_sets_the_error_flag(small_terrain):
    ctx = native.Context(0)
    scene, _ = small_terrain
    ctx.set_scene(scene)
    rays = scenes.random_rays(*scene.world_bounds(), 4096, seed=1)
    ref = ctx.trace(rays)
    assert ctx.stats()["error_flags"] == 0
    ctx.debug_walk_budget(3)
    ctx.trace(rays)
    assert ctx.stats()["error_flags"] & 2  # kErrIterationBudget
    ctx.debug_walk_budget(0)
    got = ctx.trace(rays)
    assert ctx.stats()["error_flags"] == 0
    for f in ("t", "prim", "face"):
        assert np.array_equal(got[f].view(np.uint32), ref[f].view(np.uint32))
    ctx.close()


def batch(seed, n=2, h=32, w=32):
    import torch
    rng = np.random.default_rng(seed)
    hdr = rng.gamma(1.0, 0.6, (n, h, w, 4)).astype(np.float32)
    nd = np.concatenate([rng.standard_normal((n, h, w, 3)), rng.uniform(0, 20, (n, h, w, 1))], -1).astype(np.float32)
    alb = rng.uniform(0, 1, (n, h, w, 4)).astype(np.float32)
    target = (hdr[..., :3] * rng.uniform(0.7, 1.3, (n, h, w, 3))).astype(np.float32)
    return torch.from_numpy(unet.pack_features(hdr, nd, alb)).cuda(), torch.from_numpy(target).cuda()


def test_denoiser_training_checkpoint():
    f, t = batch(1)
    a = native.Denoiser(0, seed=5)
    for _ in range(3):
        a.train_step(f, t, 1e-3)
    state = a.save_state()
    la = [a.train_step(f, t, 1e-3) for _ in range(3)]
    pa = a.get_params()
    b = native.Denoiser(0, seed=9)  # other initial weights: the state replaces them
    b.load_state(state)
    assert b.save_state() == state
    lb = [b.train_step(f, t, 1e-3) for _ in range(3)]
    pb = b.get_params()
    # weight gradients accumulate with atomics, so runs agree to rounding, not to the bit
    np.testing.assert_allclose(lb, la, rtol=1e-4)
    np.testing.assert_allclose(pb, pa, rtol=1e-3, atol=1e-6)
    with pytest.raises(native.SpkError):
        b.load_state(state[:64])
    a.close()
    b.close()


def test_bounded_wait_times_out_and_the_denoiser_recovers():
    f, _ = batch(2, n=1, h=64, w=64)
    dn = native.Denoiser(0, seed=1)
    ref = dn.infer(f).cpu().numpy()
    t0 = time.perf_counter()
    with pytest.raises(native.SpkError) as e:
        dn.debug_wait_timeout()
    dt = time.perf_counter() - t0
    assert e.value.status == DEVICE_LIMIT and "0x1" in str(e.value)
    assert 0.9 < dt < 10.0
    got = dn.infer(f).cpu().numpy()
    assert np.array_equal(got, ref)
    native.debug_fail_allocation(1)  # a failed activation allocation in inference, then recovery
    g2, _ = batch(3, n=2, h=96, w=96)
    with pytest.raises(native.SpkError) as e:
        dn.infer(g2)
    assert e.value.status == OOM
    native.debug_fail_allocation(0)
    dn.infer(g2)
    assert np.array_equal(dn.infer(f).cpu().numpy(), ref)
    dn.close()


def test_training_run_resumes_from_its_checkpoint(tmp_path):
    import torch
    from sparkle_gb300 import denoise
    f, t = batch(4, n=4, h=64, w=64)
    data = denoise.DataSet(f, t)
    kw = dict(batch=2, crop=32, lr=1e-3, seed=3)
    a = native.Denoiser(0, seed=5)
    la, _, _ = denoise.train(a, data, 6, **kw)
    ck = str(tmp_path / "train.ckpt")
    b = native.Denoiser(0, seed=5)
    lb, _, _ = denoise.train(b, data, 6, checkpoint=ck, checkpoint_every=2, stop_at=3, **kw)
    assert len(lb) == 3
    c = native.Denoiser(0, seed=11)  # other initial weights: the checkpoint replaces them
    lc, _, _ = denoise.train(c, data, 6, checkpoint=ck, resume=True, **kw)
    assert len(lc) == 6
    np.testing.assert_allclose(lc, la, rtol=1e-4)
    np.testing.assert_allclose(c.get_params(), a.get_params(), rtol=1e-3, atol=1e-6)
    for d in (a, b, c):
        d.close()
