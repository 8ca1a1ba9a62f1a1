"""Device BLAS builders (spk_tuning.bvh_builder = 1: Karras LBVH over Morton codes; 2: PLOC clustering over
the same order), collapsed to the same 8-wide node format as the host builder. Results never depend on the tree, so hits and images must equal
the host-built scene's bit for bit; the build is deterministic, and a refit of a device-built tree with
unchanged positions reproduces it."""
import time

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


@pytest.mark.parametrize("builder", [1, 2])
@pytest.mark.parametrize("width,leaf", [(8, 3), (4, 2), (2, 1), (8, 1)])
def test_device_build_hits_equal_host_build(ctx, small_terrain, width, leaf, builder):
    scene, _ = small_terrain
    rays = scenes.random_rays(*scene.world_bounds(), 50_000, seed=12)
    ctx.set_tuning(bvh_builder=0, bvh_width=8, bvh_leaf_size=3, bvh_collapse=0)
    ctx.set_scene(scene)
    ref = ctx.trace(rays)
    ctx.set_tuning(bvh_builder=builder, bvh_width=width, bvh_leaf_size=leaf)
    ctx.set_scene(scene)
    got = ctx.trace(rays)
    assert ctx.stats()["error_flags"] == 0
    hits_equal(got, ref)
    if width == 8 and leaf == 3:
        assert_hits_match_oracle(got, scene, rays, f"device builder {builder} vs oracle")
    ctx.set_tuning(bvh_builder=0, bvh_width=8, bvh_leaf_size=3)


@pytest.mark.parametrize("builder", [1, 2])
def test_device_build_is_deterministic_and_refits(ctx, small_terrain, builder):
    scene, _ = small_terrain
    ctx.set_tuning(bvh_builder=builder)
    ctx.set_scene(scene)
    a = ctx.bvh_nodes()
    ctx.set_scene(scene)
    b = ctx.bvh_nodes()
    assert np.array_equal(a, b)
    for m, mesh in enumerate(scene.meshes):
        ctx.update_mesh(m, mesh.positions)
    assert np.array_equal(ctx.bvh_nodes(), a)
    ctx.set_tuning(bvh_builder=0)


@pytest.mark.parametrize("builder", [1, 2])
@pytest.mark.parametrize("n", [1, 2, 3, 4, 9, 25])
def test_tiny_meshes(ctx, n, builder):
    """Meshes of a few triangles: a single leaf root, a root with only leaf children, one level below."""
    rng = np.random.default_rng(n)
    pos = rng.uniform(-1, 1, (3 * n, 3)).astype(np.float32)
    mesh = abi.Mesh(pos, np.tile(np.array([[0, 0, 1]], np.float32), (3 * n, 1)),
                    np.arange(3 * n, dtype=np.uint32).reshape(n, 3))
    scene = abi.Scene([mesh], [abi.Instance(0, 0, np.eye(3, 4))], [abi.Material.lambertian((0.5, 0.5, 0.5))],
                      abi.Sky())
    rays = scenes.random_rays(np.full(3, -1.5), np.full(3, 1.5), 20_000, seed=n)
    ctx.set_tuning(bvh_builder=0)
    ctx.set_scene(scene)
    ref = ctx.trace(rays)
    ctx.set_tuning(bvh_builder=builder)
    ctx.set_scene(scene)
    hits_equal(ctx.trace(rays), ref)
    assert (ref["prim"] != 0xFFFFFFFF).any()
    ctx.set_tuning(bvh_builder=0)


@pytest.mark.parametrize("builder", [1, 2])
def test_large_mesh_builds_fast_and_equal(ctx, builder):
    """A 512x512 heightfield (524,288 triangles): same hits as the host build, built in far less time."""
    mesh = scenes.heightfield(512, 100.0, 6.0, seed=2)
    scene = abi.Scene([mesh], [abi.Instance(0, 0, np.eye(3, 4))], [abi.Material.lambertian((0.5, 0.5, 0.5))],
                      abi.Sky())
    rays = scenes.random_rays(*scene.world_bounds(), 200_000, seed=3)
    ctx.set_tuning(bvh_builder=0)
    t0 = time.perf_counter()
    ctx.set_scene(scene)
    host_s = time.perf_counter() - t0
    ref = ctx.trace(rays)
    ctx.set_tuning(bvh_builder=builder)
    ctx.set_scene(scene)  # warm
    t0 = time.perf_counter()
    ctx.set_scene(scene)
    dev_s = time.perf_counter() - t0
    got = ctx.trace(rays)
    hits_equal(got, ref)
    print(f"set_scene 524k triangles: host SAH {host_s * 1e3:.0f} ms, device builder {builder}: {dev_s * 1e3:.0f} ms")
    assert dev_s < host_s
    ctx.set_tuning(bvh_builder=0)


def test_device_built_render_equals_host_built(ctx, small_terrain):
    scene, cam_args = small_terrain
    camera = scenes.make_camera(cam_args, 64, 48)
    cfg = abi.make_config(64, 48, spp=2, bounce=4, seed=1)
    out = []
    for builder in (0, 1, 2):
        ctx.set_tuning(bvh_builder=builder)
        ctx.set_scene(scene)
        ctx.set_config(cfg)
        ctx.set_camera(camera)
        ctx.render(3)
        out.append(ctx.framebuffer())
    assert np.array_equal(out[0][0].view(np.uint32), out[1][0].view(np.uint32))
    assert np.array_equal(out[0][0].view(np.uint32), out[2][0].view(np.uint32))
    o_hdr, o_out = oracle_image(scene, camera, cfg, 3)
    assert_image_parity(compare_images(out[1][0], out[1][1], o_hdr, o_out), "device-built render vs oracle")
    ctx.set_tuning(bvh_builder=0)
