"""Denoised vs plain path tracing at equal accuracy, on the incoherent-ray stress scene.

    python -m sparkle_gb300.eval_denoiser --width 1920 --height 1080 --ref-spp 16384

Renders a --ref-spp plain reference, then (1) plain path tracing accumulated to 1, 2, 4, ... --plain-max
spp, timing each point, and (2) denoised rendering at each --den-spp (samples in two halves, U-Net on the
mean and on each half, per-tile fallback to the plain mean where the halves disagree, spk_dn_fallback).
Every image is scored by relMSE against the reference; the wall time to reach each --targets relMSE is
reported for both (plain: log-log interpolation between measured spp points). Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import denoise, native, scenes


def run(width=1920, height=1080, ref_spp=16384, plain_max=4096, den_spp=(1, 4, 16), targets=(0.01, 0.003),
        threshold=0.02, tile=16, weights=denoise.WEIGHTS, scene_seed=0, ctx=None, dn=None):
    import torch
    own = ctx is None
    ctx = ctx or native.Context(0)
    dn = dn or native.Denoiser(0)
    meta = denoise.load_weights(dn, weights) if weights else {}
    scene, cam_args = scenes.terrain_spheres(scene_seed)
    camera = scenes.make_camera(cam_args, width, height)
    ctx.set_scene(scene)
    # reference
    ctx.set_config(denoise.render_config(width, height, seed=7001))
    ctx.set_camera(camera)
    t0 = time.perf_counter()
    ctx.render(ref_spp)
    ref, _ = ctx.framebuffer()
    ref_s = time.perf_counter() - t0
    # plain curve
    ctx.set_config(denoise.render_config(width, height, seed=7002))
    spps = [1 << k for k in range(0, int(np.log2(plain_max)) + 1)]
    denoise.plain_curve(ctx, camera, [1], ref)  # warm-up (allocations, first launch)
    ctx.set_config(denoise.render_config(width, height, seed=7003))
    curve = denoise.plain_curve(ctx, camera, spps, ref)
    # denoised
    den = []
    for k, s in enumerate(den_spp):
        ctx.set_config(denoise.render_config(width, height, seed=7100 + k))
        if k == 0:
            denoise.render_denoised(ctx, dn, camera, s, tile, threshold)  # warm-up
            ctx.set_config(denoise.render_config(width, height, seed=7200))
        fr = denoise.render_denoised(ctx, dn, camera, s, tile, threshold)
        den.append(dict(spp=s, relmse=denoise.relmse(fr.image, ref), plain_relmse=denoise.relmse(fr.plain, ref),
                        wall_s=round(fr.wall_s, 4), render_s=round(fr.render_s, 4), denoise_s=round(fr.denoise_s, 4),
                        fallback_tiles=fr.fallback_tiles, tiles=fr.tiles))
    out = dict(scene="terrain_spheres(%d)" % scene_seed, width=width, height=height, ref_spp=ref_spp,
               ref_render_s=round(ref_s, 2), threshold=threshold, tile=tile,
               plain=[dict(spp=s, relmse=e, wall_s=round(t, 4)) for s, e, t in curve], denoised=den,
               weights_meta={k: (v.item() if hasattr(v, "item") else v) for k, v in meta.items()})
    for tgt in targets:
        tp = denoise.time_to(curve, tgt)
        ok = [d["wall_s"] for d in den if d["relmse"] <= tgt]
        out[f"time_to_{tgt}"] = dict(plain_s=tp, denoised_s=min(ok) if ok else None,
                                     speedup=(tp / min(ok)) if (tp and ok) else None)
    if own:
        dn.close()
        ctx.close()
    torch.cuda.synchronize()
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--ref-spp", type=int, default=16384)
    ap.add_argument("--plain-max", type=int, default=4096)
    ap.add_argument("--den-spp", default="1,4,16")
    ap.add_argument("--threshold", type=float, default=0.02)
    ap.add_argument("--tile", type=int, default=16)
    ap.add_argument("--weights", default=denoise.WEIGHTS)
    args = ap.parse_args(argv)
    out = run(args.width, args.height, args.ref_spp, args.plain_max,
              tuple(int(x) for x in args.den_spp.split(",")), threshold=args.threshold, tile=args.tile,
              weights=args.weights)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
