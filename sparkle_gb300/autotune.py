"""Autotuner for the path tracer's launch shapes and schedule (spk_tuning): queue capacity (batch path
slots), CTAs per SM of the traversal and shading stages, BVH node width and leaf size, material sort on
or off, CUDA-graph replay on or off, NEE occlusion rays in their own shadow stage or inline, primary rays
walked in warp packets or one by one.

No knob changes a result (spk_tuning), so the tuner only measures: it runs a caller's workload under each
candidate setting and keeps the fastest by device time. The search is coordinate descent from the
defaults, one knob at a time in SPACE order, for `rounds` passes; BVH knobs rebuild the scene(s) through
the caller's `rebuild` hook.

    best, log = autotune(ctx, workload, rebuild=lambda: ctx.set_scenes(scene_list))
    ctx.set_tuning(**best)
"""
from __future__ import annotations

import time

SPACE = {
    "batch_slots": [1 << 27, 1 << 25, 1 << 23, 1 << 21],
    "path_slots_per_pixel": [64, 16, 4, 1],
    "shade_blocks_per_sm": [4, 8, 16],
    "extend_blocks_per_sm": [0, 6],
    "material_sort": [0, 1],
    "cuda_graph": [1, 0],
    "bvh_width": [8, 4],
    "bvh_leaf_size": [3, 2],
    "bvh_collapse": [0, 1],
    "bvh_builder": [0, 1, 2],
    "shadow_stage": [1, 0],
    "primary_packets": [1, 0],
}
SCENE_KNOBS = ("bvh_width", "bvh_leaf_size", "bvh_collapse", "bvh_builder")


def measure(ctx, workload, repeats: int = 2):
    """Best-of-`repeats` (rays, device ms) of `workload(ctx)`, which renders and returns ctx.stats()."""
    best = None
    for _ in range(repeats):
        st = workload(ctx)
        if st["error_flags"]:
            return None
        rays = st["extension_rays"] + st["shadow_rays"]
        cand = (rays, st["device_ms"])
        if best is None or cand[1] < best[1]:
            best = cand
    return best


def autotune(ctx, workload, rebuild=None, space=None, rounds: int = 1, repeats: int = 2, log=print):
    """Coordinate-descent search; returns (best knob dict, [(knobs, Mrays/s)] of every evaluation)."""
    space = dict(space or SPACE)
    if rebuild is None:
        for k in SCENE_KNOBS:
            space.pop(k, None)
    current = ctx.tuning()
    history = []

    def evaluate(knobs):
        ctx.set_tuning(**knobs)
        if rebuild is not None and any(knobs[k] != current_scene[k] for k in SCENE_KNOBS if k in knobs):
            rebuild()
            for k in SCENE_KNOBS:
                current_scene[k] = knobs[k]
        m = measure(ctx, workload, repeats)
        rate = None if m is None else m[0] / (m[1] * 1e3)
        history.append((dict(knobs), rate))
        if log:
            log(f"autotune {knobs} -> {rate if rate is None else round(rate, 1)} Mrays/s")
        return rate

    current_scene = {k: current[k] for k in SCENE_KNOBS}
    best_rate = evaluate(current)
    t0 = time.perf_counter()
    for _ in range(rounds):
        for knob, values in space.items():
            for v in values:
                if v == current[knob]:
                    continue
                cand = dict(current, **{knob: v})
                rate = evaluate(cand)
                if rate is not None and (best_rate is None or rate > best_rate):
                    best_rate, current = rate, cand
    ctx.set_tuning(**current)
    if rebuild is not None and any(current[k] != current_scene[k] for k in SCENE_KNOBS):
        rebuild()
    if log:
        log(f"autotune best {current} -> {best_rate} Mrays/s ({time.perf_counter() - t0:.1f} s)")
    return current, history
