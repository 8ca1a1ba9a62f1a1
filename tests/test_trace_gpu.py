"""Ray-set parity of the device BVH walk (spk_trace through the C ABI) against the CPU oracle.

Closest hits must be bit-identical (primitive, face, t, u, v) except where two hits have bit-identical
t (order-dependent ties, counted) or a box test grazes (counted, bounded); any-hit must agree on hit/miss.
"""
import json

import numpy as np
import pytest

import oracle
from sparkle_gb300 import abi, native, scenes

from parity import INVALID, axis_parallel, classify_hits, oracle_hits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


def sphere_field(seed=0, n=24):
    """Analytic spheres (SphereRenderProxy) over a ground quad, plus a transformed cube."""
    rng = np.random.default_rng(seed)
    ground = scenes._quad((-10, -10, 0), (10, -10, 0), (10, 10, 0), (-10, 10, 0), (0, 0, 1), (1, 0, 0))
    meshes = [ground, scenes.unit_cube()]
    mats = [abi.Material.lambertian((0.5, 0.5, 0.5)), abi.Material.metal((0.9, 0.8, 0.7), 0.2),
            abi.Material.glass()]
    inst = [abi.Instance(0, 0)]
    for k in range(n):
        c = rng.uniform(-8, 8, 3)
        c[2] = rng.uniform(0.5, 3)
        r = float(rng.uniform(0.3, 1.2))
        inst.append(abi.Instance(0, int(k % 3), scenes._affine(np.eye(3), c), sphere=True, radius=r))
    lin = scenes._rot_z(0.7) @ np.diag([2.0, 1.0, 3.0])
    inst.append(abi.Instance(1, 1, scenes._affine(lin, (1.0, -2.0, 1.5))))
    return abi.Scene(meshes, inst, mats, abi.Sky(abi.SPK_SKY_GRADIENT, (0.3, 0.5, 0.9)), name="spheres")


def _check_closest(ctx, scene, rays, max_bad_frac=2e-5, min_hit_frac=0.2):
    ctx.set_scene(scene)
    ref_scene = oracle.OracleScene(scene)
    got = ctx.trace(rays)
    st = ctx.stats()
    assert st["error_flags"] == 0, st
    assert st["extension_rays"] == len(rays)
    ref, _ = oracle_hits(ref_scene, rays, oracle.PRUNED)
    c = classify_hits(got, ref)
    print(scene.name, {k: v for k, v in c.items() if k != "mismatch_idx"})
    assert c["hits"] > min_hit_frac * c["n"]
    assert c["other"] == 0
    assert c["exact"] + c["tie"] + c["gpu_closer"] + c["ref_closer"] == c["n"]
    # every disagreement is a tie (bit-identical t, order-dependent winner) or a rare grazing box test
    assert c["gpu_closer"] + c["ref_closer"] <= max(2, max_bad_frac * c["n"])
    assert c["exact"] + c["tie"] >= (1 - max_bad_frac) * c["n"] - 2
    return got, ref, c


def test_cornell_closest(ctx, cornell):
    scene, _ = cornell
    rays = scenes.random_rays(*scene.world_bounds(), 200_000, seed=11)
    _check_closest(ctx, scene, rays)


def test_sphere_field_closest(ctx):
    scene = sphere_field()
    lo, hi = scene.world_bounds()
    rays = scenes.random_rays(lo, hi, 200_000, seed=12)
    got, ref, _ = _check_closest(ctx, scene, rays)
    sph = np.array([scene.instances[p].sphere if p != INVALID else False for p in ref["prim"]])
    assert sph.sum() > 1000
    assert np.all(got["face"][sph] == INVALID)


def test_small_terrain_closest(ctx, small_terrain):
    scene, _ = small_terrain
    rays = scenes.random_rays(*scene.world_bounds(), 300_000, seed=13)
    _check_closest(ctx, scene, rays)


def test_axis_aligned_and_degenerate_rays(ctx, cornell):
    """d.x == 0 rays never hit a triangle (world t is NaN, Ray::InverseAt divides by d.x); spheres still
    hit. Axis-aligned directions exercise the zero-component slab test (checked against brute force)."""
    scene = sphere_field(seed=4)
    lo, hi = scene.world_bounds()
    rng = np.random.default_rng(5)
    n = 20_000
    o = lo + (hi - lo) * rng.random((n, 3))
    d = np.zeros((n, 3))
    axis = rng.integers(0, 3, n)
    d[np.arange(n), axis] = np.where(rng.random(n) < 0.5, -1.0, 1.0)
    rays = abi.rays_to_array(o.astype(np.float32), d.astype(np.float32))
    got, ref, _ = _check_closest(ctx, scene, rays, min_hit_frac=0.02)
    tri_hits = (got["prim"] != INVALID) & (got["face"] != INVALID)
    assert not np.any(tri_hits & (rays[:, 3] == 0.0))


def test_any_hit_agrees_on_hit_or_miss(ctx, small_terrain):
    scene, _ = small_terrain
    ctx.set_scene(scene)
    rays = scenes.random_rays(*scene.world_bounds(), 200_000, seed=14)
    got = ctx.trace(rays, any_hit=True)
    ref, _ = oracle.OracleScene(scene).trace(rays, any_hit=True)
    agree = (got["prim"] != INVALID) == (ref["prim"] != INVALID)
    assert agree.mean() >= 1 - 1e-4, agree.mean()


def test_empty_scene_and_empty_ray_set(ctx):
    scene = abi.Scene([], [], [abi.Material()], abi.Sky())
    ctx.set_scene(scene)
    rays = scenes.random_rays((-1, -1, -1), (1, 1, 1), 1000, seed=1)
    got = ctx.trace(rays)
    assert np.all(got["prim"] == INVALID)
    assert len(ctx.trace(rays[:0])) == 0


def test_full_size_random_rays(ctx):
    """16M random rays on the full stress scene (2,097,152 terrain + 64 x 20,480 icosphere triangles):
    every ray compared against the oracle, and a second launch reproduces the first bit for bit."""
    scene, _ = scenes.terrain_spheres(0)
    ctx.set_scene(scene)
    rays = scenes.random_rays(*scene.world_bounds(), 16 * 1024 * 1024, seed=21)
    got = ctx.trace(rays)
    again = ctx.trace(rays)
    assert np.array_equal(got.view(np.uint8), again.view(np.uint8))
    osc = oracle.OracleScene(scene)
    ref, quirk = oracle_hits(osc, rays, oracle.PRUNED)
    c = classify_hits(got, ref)
    # near ties: mismatches whose two hit distances are within 1e-5 relative (a grazing box test or an
    # order-dependent tie), against the ones farther apart
    mi = c["mismatch_idx"]
    both = (got["prim"][mi] != INVALID) & (ref["prim"][mi] != INVALID)
    gt, rt = got["t"][mi].astype(np.float64), ref["t"][mi].astype(np.float64)
    near = both & (np.abs(gt - rt) <= 1e-5 * np.maximum(np.abs(rt), 1e-30))
    record = {k: v for k, v in c.items() if k != "mismatch_idx"}
    record.update(axis_parallel=int(quirk.sum()), axis_parallel_hits=int((ref["prim"][quirk] != INVALID).sum()),
                  near_tie_mismatches=int(near.sum()), far_mismatches=int(len(mi) - near.sum()),
                  exact_fraction=c["exact"] / c["n"])
    print("RAYSET_PARITY " + json.dumps(record))
    assert c["other"] == 0
    assert c["gpu_closer"] + c["ref_closer"] <= 2e-6 * c["n"] + 4
    assert c["exact"] + c["tie"] >= (1 - 2e-6) * c["n"] - 4
