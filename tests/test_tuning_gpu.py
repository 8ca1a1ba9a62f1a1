"""Performance knobs (spk_set_tuning) never change a result: every setting renders the same bits as the
defaults, on both schedules, and closest-hit queries return the same hits for every BVH shape.

The tie-break between equal hit distances is (instance, face), independent of the tree, and every sample
draws its random numbers from its own (pixel, sample) seed, independent of which slot or launch runs it.
"""
import numpy as np
import pytest

from sparkle_gb300 import abi, native, scenes

pytestmark = pytest.mark.gpu

DEFAULTS = dict(cuda_graph=1, material_sort=0, bvh_width=8, bvh_leaf_size=3, extend_blocks_per_sm=0,
                shade_blocks_per_sm=8, batch_slots=0, ray_sort=0, bvh_collapse=0, bvh_builder=0,
                path_slots_per_pixel=64, shadow_stage=1, multi_frame=1, primary_packets=1)

VARIANTS = [
    dict(cuda_graph=0),
    dict(material_sort=1),
    dict(bvh_width=2),
    dict(bvh_width=4, bvh_leaf_size=1),
    dict(bvh_leaf_size=2, extend_blocks_per_sm=2),
    dict(shade_blocks_per_sm=3, material_sort=1, cuda_graph=0),
    dict(ray_sort=1),
    dict(bvh_collapse=1),
    dict(bvh_collapse=1, bvh_width=4, bvh_leaf_size=2),
    dict(ray_sort=1, material_sort=1),
    dict(bvh_builder=1),
    dict(bvh_builder=1, bvh_width=4, bvh_leaf_size=1),
    dict(bvh_builder=2),
    dict(path_slots_per_pixel=1),
    dict(path_slots_per_pixel=4, cuda_graph=0),
    dict(path_slots_per_pixel=3, material_sort=1),
    dict(shadow_stage=0),
    dict(shadow_stage=0, material_sort=1, path_slots_per_pixel=2),
    dict(multi_frame=0),
    dict(multi_frame=0, shadow_stage=0, material_sort=1),
    dict(primary_packets=0),
    dict(primary_packets=0, multi_frame=0),
    dict(bvh_width=4, bvh_leaf_size=1, ray_sort=1),  # packets over a sorted queue and a narrow tree
]


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


def render(ctx, scene, camera, cfg, frames, knobs):
    ctx.set_tuning(**{**DEFAULTS, **knobs})
    ctx.set_scene(scene)  # BVH shape knobs apply at scene upload
    ctx.set_config(cfg)
    ctx.set_camera(camera)
    ctx.render(frames)
    hdr, out = ctx.framebuffer()
    st = ctx.stats()
    assert st["error_flags"] == 0, st
    return hdr, out, st


def test_tuning_defaults_and_validation(ctx):
    ctx.set_tuning(**DEFAULTS)
    assert ctx.tuning() == DEFAULTS
    for bad in [dict(bvh_width=1), dict(bvh_width=9), dict(bvh_leaf_size=0), dict(bvh_leaf_size=4),
                dict(cuda_graph=2), dict(shade_blocks_per_sm=0), dict(extend_blocks_per_sm=33),
                dict(path_slots_per_pixel=0), dict(path_slots_per_pixel=65), dict(shadow_stage=2), dict(multi_frame=2),
                dict(primary_packets=2)]:
        with pytest.raises(native.SpkError):
            ctx.set_tuning(**bad)
        assert ctx.tuning() == DEFAULTS  # a rejected setting leaves the previous one


@pytest.mark.parametrize("kernel,spatial", [(abi.SPK_KERNEL_WAVEFRONT, False), (abi.SPK_KERNEL_WAVEFRONT, True),
                                            (abi.SPK_KERNEL_MEGAKERNEL, False)])
@pytest.mark.parametrize("nee", [False, True])
def test_knobs_render_identical_bits(ctx, small_terrain, kernel, spatial, nee):
    scene, cam_args = small_terrain
    W, H = 96, 64
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=4, bounce=6, enable_nee=nee, spatial_denoise=spatial, seed=5, kernel=kernel)
    # 70 frames: the multi-frame wavefront splits them into two passes (64 + 6), two chunk-graph keys
    base_hdr, base_out, _ = render(ctx, scene, camera, cfg, 70, {})
    for knobs in VARIANTS:
        hdr, out, _ = render(ctx, scene, camera, cfg, 70, knobs)
        assert np.array_equal(hdr.view(np.uint32), base_hdr.view(np.uint32)), knobs
        assert np.array_equal(out, base_out), knobs
    ctx.set_tuning(**DEFAULTS)


def test_graph_replays_keep_accumulating(ctx, cornell):
    """Split calls through the replayed chunk graph equal one call without graphs (bit-identical)."""
    scene, cam_args = cornell
    W, H = 64, 48
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=5, seed=11, kernel=abi.SPK_KERNEL_WAVEFRONT)
    ref, _, _ = render(ctx, scene, camera, cfg, 24, dict(cuda_graph=0))
    ctx.set_tuning(**DEFAULTS)
    ctx.set_scene(scene)
    ctx.set_config(cfg)
    ctx.set_camera(camera)
    for n in (5, 3, 8, 8):
        ctx.render(n)
    hdr, _ = ctx.framebuffer()
    st = ctx.stats()
    assert st["error_flags"] == 0 and st["trace_launches"] > 0 and st["trace_kernel_ms"] > 0, st
    assert st["graph_replays"] > 0, st
    assert np.array_equal(hdr.view(np.uint32), ref.view(np.uint32))
    ctx.set_tuning(**{**DEFAULTS, "cuda_graph": 0})
    ctx.render(2)
    assert ctx.stats()["graph_replays"] == 0
    ctx.set_tuning(**DEFAULTS)


@pytest.mark.parametrize("width,leaf,collapse,builder", [(2, 1, 1, 0), (4, 3, 1, 0), (8, 2, 1, 0), (8, 3, 0, 0),
                                                        (4, 2, 0, 0), (8, 3, 0, 1), (2, 1, 0, 1), (8, 1, 0, 1)])
def test_trace_hits_independent_of_bvh_shape(ctx, small_terrain, width, leaf, collapse, builder):
    scene, _ = small_terrain
    ctx.set_tuning(**DEFAULTS)
    ctx.set_scene(scene)
    rays = scenes.random_rays(*scene.world_bounds(), 50_000, seed=9)
    ref = ctx.trace(rays)
    nodes_default = ctx.stats()["bvh_nodes"]
    ctx.set_tuning(**{**DEFAULTS, "bvh_width": width, "bvh_leaf_size": leaf, "bvh_collapse": collapse,
                      "bvh_builder": builder})
    ctx.set_scene(scene)
    got = ctx.trace(rays)
    st = ctx.stats()
    assert st["error_flags"] == 0
    if width < 8 and not collapse and not builder:
        assert st["bvh_nodes"] > nodes_default
    for f in ("t", "u", "v", "prim", "face"):
        assert np.array_equal(got[f].view(np.uint32), ref[f].view(np.uint32)), f
    ctx.set_tuning(**DEFAULTS)


@pytest.mark.parametrize("frames", [1, 4, 8, 64])
def test_primary_packets_run_where_they_pay(ctx, small_terrain, frames):
    """The packet walk takes the primary rays of a pass whose pixels give it >= 8 samples in a row (the
    instrumented walk then counts each node once per packet, far fewer visits) and renders the same bits;
    with fewer samples per pixel per pass the persistent walk keeps them (the same count)."""
    scene, cam_args = small_terrain
    W, H = 128, 96
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=1, seed=3)  # one segment per path: the primary rays alone
    ctx.set_scene(scene)
    visits = {}
    for packets in (0, 1):
        ctx.set_tuning(**{**DEFAULTS, "primary_packets": packets})
        ctx.set_config(cfg)
        ctx.set_camera(camera)
        ctx.set_instrumentation(True)
        ctx.render(frames)
        ctx.set_instrumentation(False)
        st = ctx.stats()
        assert st["error_flags"] == 0 and st["extension_rays"] == W * H * frames
        visits[packets] = st["node_visits"]
        hdr, out = ctx.framebuffer()
        if packets == 0:
            base = (hdr, out)
    assert np.array_equal(hdr.view(np.uint32), base[0].view(np.uint32)) and np.array_equal(out, base[1])
    if frames >= 8:
        assert visits[1] * 4 < visits[0], visits
    else:
        assert visits[1] == visits[0], visits
    ctx.set_tuning(**DEFAULTS)


@pytest.mark.parametrize("frames", [9, 40])
def test_packets_with_ragged_ends(ctx, small_terrain, frames):
    """Odd image sizes: packets straddle pixels (40 frames: two rays per lane, 64 items across two pixels;
    9 frames: one ray per lane across four) and the last packet of the pass is partly empty (33 x 17 x 40 =
    22440 items, not a multiple of 64). Full depth, NEE on: the same bits with packets as without."""
    scene, cam_args = small_terrain
    W, H = 33, 17
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=6, enable_nee=True, seed=11)
    out = []
    for packets in (1, 0):
        hdr, img, st = render(ctx, scene, camera, cfg, frames, {"primary_packets": packets})
        out.append((hdr, img))
    assert np.array_equal(out[0][0].view(np.uint32), out[1][0].view(np.uint32))
    assert np.array_equal(out[0][1], out[1][1])
    ctx.set_tuning(**DEFAULTS)
