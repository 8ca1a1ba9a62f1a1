"""Incremental scene changes (spk_set_instances, spk_set_instance_transforms, spk_update_mesh) against a
fresh spk_set_scene of the changed scene, and against the CPU oracle on the changed scene.

SceneRenderProxy::UpdateBVH rebuilds the TLAS on every primitive change and keeps each mesh's BLAS
(SceneRenderProxy.cpp:269-297); here a deformed mesh keeps its tree too and the device refits it. Hits and
images never depend on the tree's shape, so every update must give the same bits as building the changed
scene from scratch; a refit with unchanged positions must reproduce the node array byte for byte. The
updated context's hits and images are also compared with the oracle's for the changed scene (parity
tolerances of tests/parity.py).
"""
import copy

import numpy as np
import pytest

from sparkle_gb300 import abi, native, scenes

from parity import assert_hits_match_oracle, assert_image_parity, compare_images, oracle_image

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


def hits_equal(a, b):
    for f in ("t", "u", "v", "prim", "face"):
        assert np.array_equal(a[f].view(np.uint32), b[f].view(np.uint32)), f


def render(c, scene_cam, cfg, frames=3, scene=None, with_image=False):
    sc, cam_args = scene_cam
    camera = scenes.make_camera(cam_args, cfg.width, cfg.height)
    if scene is not None:
        c.set_scene(scene)
    c.set_config(cfg)
    c.set_camera(camera)
    c.render(frames)
    assert c.stats()["error_flags"] == 0
    hdr, out = c.framebuffer()
    return (hdr, out) if with_image else hdr


def assert_render_matches_oracle(hdr, out, scene, cam_args, cfg, frames, label):
    camera = scenes.make_camera(cam_args, cfg.width, cfg.height)
    o_hdr, o_out = oracle_image(scene, camera, cfg, frames)
    assert_image_parity(compare_images(hdr, out, o_hdr, o_out), label)


def deform(positions, seed, amount):
    rng = np.random.default_rng(seed)
    p = positions.astype(np.float32).copy()
    p[:, 2] += (amount * np.sin(p[:, 0] * 0.7) * np.cos(p[:, 1] * 0.5)).astype(np.float32)
    p += rng.normal(0, amount * 0.05, p.shape).astype(np.float32)
    return p


def test_identity_refit_reproduces_nodes(ctx, small_terrain):
    scene, _ = small_terrain
    ctx.set_scene(scene)
    before = ctx.bvh_nodes()
    for m, mesh in enumerate(scene.meshes):
        ctx.update_mesh(m, mesh.positions)
    after = ctx.bvh_nodes()
    assert before.shape == after.shape
    assert np.array_equal(before, after)


def test_deformed_mesh_equals_fresh_build(ctx, small_terrain):
    scene, cam_args = small_terrain
    moved = copy.deepcopy(scene)
    moved.meshes[0].positions = deform(scene.meshes[0].positions, 1, 3.0)   # terrain: big bumps
    moved.meshes[1].positions = deform(scene.meshes[1].positions, 2, 0.3)   # icosphere: wobble
    rays = scenes.random_rays(*moved.world_bounds(), 60_000, seed=4)
    fresh = native.Context(0)
    fresh.set_scene(moved)
    ref = fresh.trace(rays)
    ctx.set_scene(scene)
    ctx.update_mesh(0, moved.meshes[0].positions)
    ctx.update_mesh(1, moved.meshes[1].positions)
    got = ctx.trace(rays)
    hits_equal(got, ref)
    assert (got["prim"] != 0xFFFFFFFF).mean() > 0.2  # the rays do hit geometry
    assert_hits_match_oracle(got, moved, rays, "refit vs oracle")
    # the refitted tree is a valid tree for the new geometry: same images as the fresh build
    cfg = abi.make_config(64, 48, spp=2, bounce=4, seed=3)
    a, a_out = render(ctx, (scene, cam_args), cfg, with_image=True)
    b = render(fresh, (moved, cam_args), cfg)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert_render_matches_oracle(a, a_out, moved, cam_args, cfg, 3, "refit render vs oracle")
    fresh.close()


def test_normals_update(ctx, small_terrain):
    scene, cam_args = small_terrain
    moved = copy.deepcopy(scene)
    n = moved.meshes[0].normals.copy()
    n[:, :2] += 0.3 * np.sin(np.arange(n.shape[0]))[:, None]
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    moved.meshes[0].normals = n.astype(np.float32)
    cfg = abi.make_config(64, 48, spp=1, bounce=3, seed=8)
    ctx.set_scene(scene)
    ctx.update_mesh(0, scene.meshes[0].positions, normals=moved.meshes[0].normals)
    a = render(ctx, (scene, cam_args), cfg)
    fresh = native.Context(0)
    b = render(fresh, (moved, cam_args), cfg, scene=moved)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    fresh.close()


def test_transforms_equal_fresh_build(ctx, small_terrain):
    scene, cam_args = small_terrain
    moved = copy.deepcopy(scene)
    rng = np.random.default_rng(5)
    new = []
    for inst in moved.instances[1:]:
        t = inst.transform.copy()
        t[:, 3] += rng.uniform(-4, 4, 3).astype(np.float32)
        t[:, :3] = (scenes._rot_z(float(rng.uniform(0, 6.28))) @ t[:, :3]).astype(np.float32)
        inst.transform = t
        new.append(t)
    ctx.set_scene(scene)
    ctx.set_instance_transforms(1, np.stack(new))
    fresh = native.Context(0)
    fresh.set_scene(moved)
    rays = scenes.random_rays(*moved.world_bounds(), 40_000, seed=6)
    got = ctx.trace(rays)
    hits_equal(got, fresh.trace(rays))
    assert_hits_match_oracle(got, moved, rays, "moved instances vs oracle")
    assert ctx.stats()["bvh_nodes"] == fresh.stats()["bvh_nodes"]
    assert np.array_equal(ctx.bvh_nodes(), fresh.bvh_nodes())  # same TLAS build from the same boxes
    cfg = abi.make_config(64, 48, spp=2, bounce=4, seed=2)
    a, a_out = render(ctx, (scene, cam_args), cfg, with_image=True)
    b = render(fresh, (moved, cam_args), cfg)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert_render_matches_oracle(a, a_out, moved, cam_args, cfg, 3, "moved instances render vs oracle")
    fresh.close()


@pytest.mark.parametrize("nee", [False, True])
def test_instance_list_changes_equal_fresh_build(ctx, cornell, nee):
    """New / Remove / Move: drop a box, duplicate the light (the light table grows), swap two entries."""
    scene, cam_args = cornell
    changed = copy.deepcopy(scene)
    insts = changed.instances
    light = next(i for i in insts if np.linalg.norm(changed.materials[i.material_id].emissive) > 0)
    extra = copy.deepcopy(light)
    extra.transform = extra.transform.copy()
    extra.transform[:, 3] += np.array([0.15, 0.1, -0.05], np.float32)
    insts = insts[:6] + insts[7:] + [extra]  # remove the short box, add a second light
    insts[0], insts[2] = insts[2], insts[0]
    changed.instances = insts
    cfg = abi.make_config(48, 48, spp=2, bounce=5, enable_nee=nee, seed=9)
    ctx.set_scene(scene)
    render(ctx, (scene, cam_args), cfg, frames=2)
    ctx.set_instances(changed.instances)
    a, a_out = render(ctx, (scene, cam_args), cfg, with_image=True)
    fresh = native.Context(0)
    b = render(fresh, (changed, cam_args), cfg, scene=changed)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert_render_matches_oracle(a, a_out, changed, cam_args, cfg, 3, f"instance list nee={nee} vs oracle")
    # the change cleared the accumulation: 3 frames after the update, not 5
    assert ctx.sample_counts()[0] == fresh.sample_counts()[0]
    fresh.close()


def test_emissive_mesh_deformation_updates_lights(ctx, cornell):
    scene, cam_args = cornell
    light_inst = next(i for i in scene.instances if np.linalg.norm(scene.materials[i.material_id].emissive) > 0)
    m = light_inst.mesh_id
    moved = copy.deepcopy(scene)
    p = moved.meshes[m].positions.copy()
    c = p.mean(axis=0)
    moved.meshes[m].positions = (c + (p - c) * np.array([1.6, 0.7, 1.0], np.float32)).astype(np.float32)
    cfg = abi.make_config(48, 48, spp=2, bounce=4, enable_nee=True, seed=4)
    ctx.set_scene(scene)
    ctx.update_mesh(m, moved.meshes[m].positions)
    a = render(ctx, (scene, cam_args), cfg)
    fresh = native.Context(0)
    b = render(fresh, (moved, cam_args), cfg, scene=moved)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    fresh.close()


def test_update_validation(ctx, small_terrain, cornell):
    scene, _ = small_terrain
    ctx.set_scene(scene)
    with pytest.raises(native.SpkError):
        ctx.update_mesh(0, scene.meshes[0].positions[:-1])  # vertex count differs
    with pytest.raises(native.SpkError):
        ctx.update_mesh(7, scene.meshes[0].positions)  # no such mesh
    with pytest.raises(native.SpkError):
        ctx.set_instance_transforms(len(scene.instances), np.eye(3, 4)[None])  # past the end
    bad = copy.deepcopy(scene.instances)
    bad[0].material_id = 999
    with pytest.raises(native.SpkError):
        ctx.set_instances(bad)
    ctx.set_scenes([scene, cornell[0]])  # several scenes: no incremental updates
    with pytest.raises(native.SpkError):
        ctx.set_instance_transforms(0, np.eye(3, 4)[None])


def test_empty_instance_list_and_back(ctx, cornell):
    scene, cam_args = cornell
    cfg = abi.make_config(32, 24, spp=1, bounce=3, seed=5)
    ctx.set_scene(scene)
    ref = render(ctx, (scene, cam_args), cfg)
    ctx.set_instances([])
    empty = render(ctx, (scene, cam_args), cfg)
    assert np.all(empty[..., :3] == 0)  # no geometry, no sky
    hits = ctx.trace(scenes.random_rays(np.zeros(3), np.ones(3), 1000, seed=1))
    assert np.all(hits["prim"] == 0xFFFFFFFF)
    ctx.set_instances(scene.instances)
    assert np.array_equal(render(ctx, (scene, cam_args), cfg).view(np.uint32), ref.view(np.uint32))
    # a mesh with no faces updates without a BLAS
    empty_mesh = abi.Mesh(np.zeros((3, 3), np.float32), np.tile([[0, 0, 1]], (3, 1)).astype(np.float32),
                          np.zeros((0, 3), np.uint32))
    sc = abi.Scene(scene.meshes + [empty_mesh], scene.instances + [abi.Instance(len(scene.meshes), 0, np.eye(3, 4))],
                   scene.materials, scene.sky)
    ctx.set_scene(sc)
    ctx.update_mesh(len(scene.meshes), np.ones((3, 3), np.float32))
    assert np.array_equal(render(ctx, (sc, cam_args), cfg).view(np.uint32), ref.view(np.uint32))
