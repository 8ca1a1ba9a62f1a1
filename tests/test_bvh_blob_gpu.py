"""BVH blobs (spk_save_bvh / spk_set_bvh): a scene rebuilt from a blob takes every matching mesh's BLAS
from it -- the same nodes as the original build, the same hits -- and builds the meshes whose geometry or
BVH knobs differ; damaged blobs are refused."""
import copy

import numpy as np
import pytest

from sparkle_gb300 import native, scenes

pytestmark = pytest.mark.gpu


def hits_equal(a, b):
    for f in ("t", "u", "v", "prim", "face"):
        assert np.array_equal(a[f].view(np.uint32), b[f].view(np.uint32)), f


def test_reload_reuses_every_blas(small_terrain):
    scene, _ = small_terrain
    a = native.Context(0)
    a.set_scene(scene)
    assert a.stats()["blas_reused"] == 0
    blob = a.save_bvh()
    rays = scenes.random_rays(*scene.world_bounds(), 30_000, seed=5)
    b = native.Context(0)
    b.set_bvh(blob)
    b.set_scene(scene)
    assert b.stats()["blas_reused"] == len(scene.meshes)
    assert np.array_equal(b.bvh_nodes(), a.bvh_nodes())
    hits_equal(b.trace(rays), a.trace(rays))
    b.set_bvh(None)
    b.set_scene(scene)
    assert b.stats()["blas_reused"] == 0
    a.close()
    b.close()


def test_changed_geometry_or_knobs_rebuild(small_terrain):
    scene, _ = small_terrain
    a = native.Context(0)
    a.set_scene(scene)
    blob = a.save_bvh()
    moved = copy.deepcopy(scene)
    moved.meshes[1].positions = (moved.meshes[1].positions * np.float32(1.1)).astype(np.float32)
    b = native.Context(0)
    b.set_bvh(blob)
    b.set_scene(moved)
    assert b.stats()["blas_reused"] == 1  # the terrain, not the changed sphere
    fresh = native.Context(0)
    fresh.set_scene(moved)
    assert np.array_equal(b.bvh_nodes(), fresh.bvh_nodes())
    b.set_tuning(bvh_leaf_size=2)  # other knobs: nothing reused
    b.set_scene(scene)
    assert b.stats()["blas_reused"] == 0
    for c in (a, b, fresh):
        c.close()


def test_blob_of_a_refitted_scene(small_terrain):
    scene, _ = small_terrain
    a = native.Context(0)
    a.set_scene(scene)
    moved = copy.deepcopy(scene)
    p = moved.meshes[0].positions.copy()
    p[:, 2] += np.float32(0.8) * np.sin(p[:, 0]).astype(np.float32)
    moved.meshes[0].positions = p
    a.update_mesh(0, p)
    blob = a.save_bvh()
    b = native.Context(0)
    b.set_bvh(blob)
    b.set_scene(moved)
    assert b.stats()["blas_reused"] == 2
    rays = scenes.random_rays(*moved.world_bounds(), 30_000, seed=6)
    hits_equal(b.trace(rays), a.trace(rays))
    a.close()
    b.close()


def test_damaged_blobs_are_refused(small_terrain):
    scene, _ = small_terrain
    a = native.Context(0)
    a.set_scene(scene)
    blob = bytearray(a.save_bvh())
    with pytest.raises(native.SpkError):
        a.set_bvh(bytes(blob[:40]))
    bad = bytearray(blob)
    bad[0] ^= 0xFF
    with pytest.raises(native.SpkError):
        a.set_bvh(bytes(bad))
    # a node whose child base points past its BLAS
    header, meta = 8 + 4 * 2 + 4 * 4, 24
    nodes_at = header + len(scene.meshes) * meta
    bad = bytearray(blob)
    bad[nodes_at + 16:nodes_at + 20] = (0x7FFFFFFF).to_bytes(4, "little")
    with pytest.raises(native.SpkError):
        a.set_bvh(bytes(bad))
    a.set_bvh(bytes(blob))  # the intact blob is accepted
    a.close()
