"""Trains the learned denoiser on path-tracer-generated pairs and saves its weights.

    python -m sparkle_gb300.train_denoiser --scenes 128 --steps 2000 --out sparkle_gb300/weights/unet.npz

Data: `--scenes` + `--holdout` seeded procedural scenes (scenes.random_training_scene) at --size^2, inputs
at --spp-in samples per pixel (log1p HDR + albedo, normal, depth guides), targets at --spp-target. Training:
Adam (lr --lr, x0.1 for the last 20% of steps) on --batch random --crop^2 crops, relMSE loss. The held-out
scenes are scored by relMSE against their targets: the plain --spp-in render, the untrained network and
the trained network. Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import denoise, native


def holdout_scores(dn, data, start):
    import torch
    out = {"plain": [], "denoised": []}
    for k in range(start, data.features.shape[0]):
        f = data.features[k:k + 1].contiguous()
        t = data.targets[k].cpu().numpy()
        plain = np.expm1(f[0, ..., :3].cpu().numpy())
        den = dn.infer(f)[0].cpu().numpy()
        out["plain"].append(denoise.relmse(plain, t))
        out["denoised"].append(denoise.relmse(den, t))
        torch.cuda.synchronize()
    return {k: float(np.mean(v)) for k, v in out.items()}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=128)
    ap.add_argument("--holdout", type=int, default=8)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--spp-in", type=int, default=4)
    ap.add_argument("--spp-target", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--crop", type=int, default=128)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=denoise.WEIGHTS)
    ap.add_argument("--checkpoint", default=None, help="training checkpoint file (written every --checkpoint-every)")
    ap.add_argument("--checkpoint-every", type=int, default=500)
    ap.add_argument("--resume", action="store_true", help="continue from --checkpoint")
    args = ap.parse_args(argv)

    ctx = native.Context(0)
    dn = native.Denoiser(0, seed=args.seed)
    t0 = time.perf_counter()
    data = denoise.generate(ctx, dn, args.scenes + args.holdout, size=args.size, spp_in=args.spp_in,
                            spp_target=args.spp_target, seed=1000 + args.seed)
    train_data = denoise.DataSet(data.features[:args.scenes], data.targets[:args.scenes])
    untrained = holdout_scores(dn, data, args.scenes)
    losses, train_s, step_ms = denoise.train(dn, train_data, args.steps, batch=args.batch, crop=args.crop,
                                             lr=args.lr, seed=args.seed, log_every=max(1, args.steps // 10),
                                             checkpoint=args.checkpoint, checkpoint_every=args.checkpoint_every,
                                             resume=args.resume)
    trained = holdout_scores(dn, data, args.scenes)
    meta = dict(scenes=args.scenes, holdout=args.holdout, size=args.size, spp_in=args.spp_in,
                spp_target=args.spp_target, steps=args.steps, batch=args.batch, crop=args.crop, lr=args.lr,
                seed=args.seed, final_loss=float(np.mean(losses[-50:])),
                holdout_plain_relmse=trained["plain"], holdout_untrained_relmse=untrained["denoised"],
                holdout_denoised_relmse=trained["denoised"])
    denoise.save_weights(dn, args.out, **meta)
    line = dict(meta, data_render_s=round(data.render_s, 2), data_rays=int(data.rays), train_s=round(train_s, 2),
                train_step_device_ms=round(step_ms, 3), total_s=round(time.perf_counter() - t0, 2),
                loss_curve=[round(float(np.mean(losses[i:i + 50])), 5) for i in range(0, len(losses), max(50, len(losses) // 20))],
                weights=args.out)
    print(json.dumps(line), flush=True)
    dn.close()
    ctx.close()


if __name__ == "__main__":
    main()
