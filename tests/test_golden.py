"""The oracle reproduces its committed golden fixtures (tests/golden/oracle_golden.npz, made by
tests/golden/make_golden.py): RNG streams and hit records bit for bit, images to 1e-6 relative (the
images pass through the C library's cos/sin/pow, whose last bits may differ between hosts)."""
import os

import numpy as np
import pytest

import oracle
from sparkle_gb300 import abi, scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_golden.npz")
HIT_BYTES = 20


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def test_rng_streams(golden):
    for name, kind in (("x128p", abi.SPK_RNG_XOSHIRO128P), ("x256ss", abi.SPK_RNG_XOSHIRO256SS)):
        for seed in (0, 1, 2 ** 33 + 17):
            u, _ = oracle.rng_fill(kind, seed, 32)
            assert np.array_equal(u, golden[f"rng_{name}_{seed}"])


def test_ray_sets(golden):
    scene, _ = scenes.cornell_box(0)
    hits, _ = oracle.OracleScene(scene).trace(golden["cornell_rays"])
    assert np.array_equal(hits.view(np.uint8).reshape(len(hits), HIT_BYTES), golden["cornell_hits"])
    ter, _ = scenes.terrain_spheres(seed=3, grid=32, num_spheres=4, sphere_level=1, size=20.0, cube_size=8)
    thits, _ = oracle.OracleScene(ter).trace(golden["terrain_rays"])
    assert np.array_equal(thits.view(np.uint8).reshape(len(thits), HIT_BYTES), golden["terrain_hits"])


@pytest.mark.parametrize("name,kind", [("x128p", abi.SPK_RNG_XOSHIRO128P), ("x256ss", abi.SPK_RNG_XOSHIRO256SS)])
@pytest.mark.parametrize("spatial", [False, True])
def test_cornell_images(golden, name, kind, spatial):
    scene, cam_args = scenes.cornell_box(0)
    W, H, frames = 24, 18, 4
    cam = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=5, spatial_denoise=spatial, rng=kind, seed=7)
    r = oracle.OracleRenderer(oracle.OracleScene(scene), cfg, cam)
    r.render(frames)
    hdr, out = r.framebuffer()
    key = f"cornell_{name}_{'spatial' if spatial else 'plain'}"
    np.testing.assert_allclose(hdr, golden[key + "_hdr"], rtol=1e-6, atol=1e-7)
    assert np.abs(out.astype(np.int32) - golden[key + "_out"].astype(np.int32)).max() <= 1
    assert np.array_equal(np.array(r.counts(), np.uint64), golden[key + "_counts"])
