"""Generates the committed golden fixtures of tests/test_golden.py from the CPU oracle.

The reference ships no golden vectors for this path (its only pinned test compares a screenshot to a remote
PNG that is not available), so these fixtures pin the oracle itself: later changes to it must reproduce them.

  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from sparkle_gb300 import abi, scenes  # noqa: E402


def render_case(rng_kind, spatial):
    scene, cam_args = scenes.cornell_box(0)
    W, H, frames = 24, 18, 4
    cam = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=5, spatial_denoise=spatial, rng=rng_kind, seed=7)
    r = oracle.OracleRenderer(oracle.OracleScene(scene), cfg, cam)
    r.render(frames)
    hdr, out = r.framebuffer()
    return hdr, out, np.array(r.counts(), np.uint64)


def main():
    out = {}
    for name, kind in (("x128p", abi.SPK_RNG_XOSHIRO128P), ("x256ss", abi.SPK_RNG_XOSHIRO256SS)):
        for seed in (0, 1, 2 ** 33 + 17):
            u, f = oracle.rng_fill(kind, seed, 32)
            out[f"rng_{name}_{seed}"] = u
    for name, kind in (("x128p", abi.SPK_RNG_XOSHIRO128P), ("x256ss", abi.SPK_RNG_XOSHIRO256SS)):
        for spatial in (False, True):
            hdr, img, counts = render_case(kind, spatial)
            key = f"cornell_{name}_{'spatial' if spatial else 'plain'}"
            out[key + "_hdr"] = hdr
            out[key + "_out"] = img
            out[key + "_counts"] = counts
    scene, _ = scenes.cornell_box(0)
    rays = scenes.random_rays(*scene.world_bounds(), 3000, seed=99)
    hits, _ = oracle.OracleScene(scene).trace(rays)
    out["cornell_rays"] = rays
    out["cornell_hits"] = hits.view(np.uint8).reshape(len(hits), -1)
    ter, _ = scenes.terrain_spheres(seed=3, grid=32, num_spheres=4, sphere_level=1, size=20.0, cube_size=8)
    trays = scenes.random_rays(*ter.world_bounds(), 3000, seed=98)
    thits, _ = oracle.OracleScene(ter).trace(trays)
    out["terrain_rays"] = trays
    out["terrain_hits"] = thits.view(np.uint8).reshape(len(thits), -1)
    np.savez_compressed(os.path.join(HERE, "oracle_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "oracle_golden.npz"))


if __name__ == "__main__":
    main()
