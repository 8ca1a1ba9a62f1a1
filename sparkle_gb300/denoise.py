"""Learned denoiser pipeline: training data from the path tracer, the training loop, denoised rendering
with the per-tile fallback, and the equal-accuracy comparison against plain path tracing.

Every pixel is computed by the library's CUDA kernels: the wavefront path tracer renders inputs, targets
and guides (spk_render / spk_render_guides), the U-Net packs features, trains and infers on the tcgen05
convolutions (include/spk_denoise.h). PyTorch only holds device buffers and cuts training crops.

relMSE is mean over pixels and colour channels of (x - ref)^2 / (ref^2 + 0.01).
"""
from __future__ import annotations

import os
import time
from dataclasses import dataclass, field

import numpy as np

from . import abi, native, scenes

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "unet.npz")


def relmse(x: np.ndarray, ref: np.ndarray) -> float:
    x = np.asarray(x, np.float64)[..., :3]
    ref = np.asarray(ref, np.float64)[..., :3]
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + 0.01)))


def _torch():
    import torch
    return torch


def render_config(width, height, seed, bounce=8, nee=True):
    return abi.make_config(width, height, spp=1, max_spp=1 << 24, bounce=bounce, enable_nee=nee,
                           rng=abi.SPK_RNG_XOSHIRO256SS, seed=seed, kernel=abi.SPK_KERNEL_WAVEFRONT)


def framebuffer_tensor(ctx: native.Context):
    """The context's HDR frame buffer as a (H, W, 4) float32 CUDA tensor (a copy)."""
    torch = _torch()
    w, h = ctx.config.width, ctx.config.height
    out = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    ctx.read_framebuffer_into(out.data_ptr(), 0)  # device-to-device copy, waits for the render
    return out


def guides_tensors(ctx: native.Context):
    """Renders the primary-hit guides and returns (normal_depth, albedo) (H, W, 4) CUDA tensors."""
    torch = _torch()
    w, h = ctx.config.width, ctx.config.height
    nd = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    al = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    ctx.render_guides()
    ctx.guides_into(nd.data_ptr(), al.data_ptr())
    return nd, al


@dataclass
class DataSet:
    features: object  # (N, H, W, 10) float32 CUDA tensor
    targets: object   # (N, H, W, 3) float32 CUDA tensor
    render_s: float = 0.0
    rays: int = 0
    info: dict = field(default_factory=dict)


def generate(ctx: native.Context, dn: native.Denoiser, num_scenes: int, size: int = 256, spp_in: int = 4,
             spp_target: int = 4096, seed: int = 0, bounce: int = 8) -> DataSet:
    """Renders `num_scenes` procedural scenes (scenes.random_training_scene) at size x size: the input at
    `spp_in` samples per pixel with its guides, the target at `spp_target` with an independent seed."""
    torch = _torch()
    feats = torch.empty((num_scenes, size, size, native.Denoiser.FEATURES), dtype=torch.float32, device="cuda")
    targets = torch.empty((num_scenes, size, size, 3), dtype=torch.float32, device="cuda")
    t0 = time.perf_counter()
    rays = 0
    for k in range(num_scenes):
        scene, cam_args = scenes.random_training_scene(seed + k)
        camera = scenes.make_camera(cam_args, size, size)
        ctx.set_scene(scene)
        ctx.set_config(render_config(size, size, seed=2 * (seed + k), bounce=bounce))
        ctx.set_camera(camera)
        ctx.render(spp_in)
        rays += ctx.stats()["extension_rays"]
        hdr = framebuffer_tensor(ctx)
        nd, al = guides_tensors(ctx)
        dn.pack_features(hdr[None], nd[None], al[None], feats[k:k + 1])
        ctx.set_config(render_config(size, size, seed=2 * (seed + k) + 1, bounce=bounce))
        ctx.set_camera(camera)
        ctx.render(spp_target)
        rays += ctx.stats()["extension_rays"]
        targets[k] = framebuffer_tensor(ctx)[..., :3]
    torch.cuda.synchronize()
    return DataSet(feats, targets, time.perf_counter() - t0, rays,
                   dict(scenes=num_scenes, size=size, spp_in=spp_in, spp_target=spp_target, seed=seed))


def save_checkpoint(path: str, dn: native.Denoiser, generator, step: int, losses):
    """Training checkpoint: the denoiser state (parameters, Adam moments, step), the crop generator's state,
    the step reached and the losses so far; written to a temporary file, then renamed."""
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        np.savez(f, dn_state=np.frombuffer(dn.save_state(), np.uint8), generator=generator.get_state().numpy(),
                 step=np.int64(step), losses=np.asarray(losses, np.float64))
    os.replace(tmp, path)


def train(dn: native.Denoiser, data: DataSet, steps: int, batch: int = 16, crop: int = 128, lr: float = 1e-3,
          seed: int = 0, log_every: int = 0, checkpoint: str = None, checkpoint_every: int = 0, resume: bool = False,
          stop_at: int = None):
    """Adam on random crops; returns (losses, seconds, device ms per step). With `checkpoint`, the state is
    saved every `checkpoint_every` steps and at the end (or at `stop_at`); `resume` continues from it, so an
    interrupted run ends where the uninterrupted one would (to the rounding of the atomic gradient sums)."""
    torch = _torch()
    g = torch.Generator(device="cpu").manual_seed(seed)
    n, h, w, _ = data.features.shape
    losses, dev_ms = [], []
    first = 0
    if resume and checkpoint and os.path.exists(checkpoint):
        z = np.load(checkpoint)
        dn.load_state(z["dn_state"].tobytes())
        g.set_state(torch.from_numpy(z["generator"]))
        first = int(z["step"])
        losses = [float(x) for x in z["losses"]]
    t0 = time.perf_counter()
    last = steps if stop_at is None else min(steps, stop_at)
    for step in range(first, last):
        idx = torch.randint(0, n, (batch,), generator=g)
        ys = torch.randint(0, h - crop + 1, (batch,), generator=g)
        xs = torch.randint(0, w - crop + 1, (batch,), generator=g)
        f = torch.stack([data.features[i, y:y + crop, x:x + crop] for i, y, x in zip(idx, ys, xs)]).contiguous()
        t = torch.stack([data.targets[i, y:y + crop, x:x + crop] for i, y, x in zip(idx, ys, xs)]).contiguous()
        step_lr = lr * (0.1 if step >= int(0.8 * steps) else 1.0)
        losses.append(dn.train_step(f, t, step_lr))
        dev_ms.append(dn.last_ms())
        if log_every and (step + 1) % log_every == 0:
            print(f"step {step + 1}: loss {np.mean(losses[-log_every:]):.5f}", flush=True)
        if checkpoint and checkpoint_every and (step + 1) % checkpoint_every == 0:
            save_checkpoint(checkpoint, dn, g, step + 1, losses)
    if checkpoint and last > first:
        save_checkpoint(checkpoint, dn, g, last, losses)
    return losses, time.perf_counter() - t0, float(np.median(dev_ms)) if dev_ms else 0.0


def save_weights(dn: native.Denoiser, path: str = WEIGHTS, **meta):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez_compressed(path, params=dn.get_params(), **{k: np.asarray(v) for k, v in meta.items()})


def load_weights(dn: native.Denoiser, path: str = WEIGHTS) -> dict:
    z = np.load(path)
    dn.set_params(z["params"])
    return {k: z[k] for k in z.files if k != "params"}


# --------------------------------------------------------------------------------------------------
# Denoised rendering with the per-tile fallback
# --------------------------------------------------------------------------------------------------
@dataclass
class DenoisedFrame:
    image: np.ndarray
    plain: np.ndarray
    fallback_tiles: int
    tiles: int
    wall_s: float
    render_s: float
    denoise_s: float


def render_denoised(ctx: native.Context, dn: native.Denoiser, camera, spp: int, tile: int = 16,
                    threshold: float = 0.02) -> DenoisedFrame:
    """Renders `spp` samples per pixel in two halves (the second half continues the same accumulation),
    denoises the mean and each half, and replaces the tiles whose two denoised halves disagree by more
    than `threshold` (spk_dn_fallback) with the plain mean. With spp == 1 there are no halves and no
    fallback. Wall time covers everything from the camera upload to the final image on the device."""
    torch = _torch()
    w, h = ctx.config.width, ctx.config.height
    # the mean and the two halves as one batch of three images: a single inference
    feats = torch.empty((3, h, w, native.Denoiser.FEATURES), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx.set_camera(camera)
    half = spp // 2
    a = None
    if half >= 1:
        ctx.render(half)
        a = framebuffer_tensor(ctx)
        ctx.render(spp - half)
    else:
        ctx.render(spp)
    full = framebuffer_tensor(ctx)
    nd, al = guides_tensors(ctx)
    t_render = time.perf_counter()
    dn.pack_features(full[None], nd[None], al[None], feats[0:1])
    fb_tiles = 0
    tiles = ((w + tile - 1) // tile) * ((h + tile - 1) // tile)
    if a is not None:
        dn.pack_halves(full[None], a[None], nd[None], al[None], feats[1:2], feats[2:3])  # half B = 2 * full - half A
        den3 = dn.infer(feats)
        den, fb_tiles = dn.fallback(den3[0], den3[1], den3[2], full, tile, threshold)
    else:
        den = dn.infer(feats[0:1])[0]
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    return DenoisedFrame(den.cpu().numpy(), full.cpu().numpy(), fb_tiles, tiles, t1 - t0, t_render - t0,
                         t1 - t_render)


def plain_curve(ctx: native.Context, camera, spps, ref: np.ndarray):
    """Plain path tracing to each spp of `spps` (ascending) in one accumulation; returns
    [(spp, relMSE, wall seconds from the start)]."""
    torch = _torch()
    out = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx.set_camera(camera)
    done = 0
    for s in spps:
        ctx.render(s - done)
        done = s
        ctx.synchronize()
        t = time.perf_counter() - t0
        hdr, _ = ctx.framebuffer()
        out.append((s, relmse(hdr, ref), t))
        t0 += time.perf_counter() - t0 - t  # exclude the read-back and the relMSE from the clock
    return out


def time_to(curve, target: float):
    """Wall time at which a (spp, relMSE, seconds) curve first reaches `target` relMSE, log-log
    interpolated between measured points; None if never."""
    prev = None
    for spp, err, t in curve:
        if err <= target:
            if prev is None:
                return t
            (s0, e0, t0) = prev
            f = (np.log(e0) - np.log(target)) / max(1e-12, np.log(e0) - np.log(err))
            return float(np.exp(np.log(t0) + f * (np.log(t) - np.log(t0))))
        prev = (spp, err, t)
    return None
