"""Batched requests (spk_set_scenes + spk_render_batch): each request of a batch over several resident
scenes renders bit-identically to the same request rendered alone through spk_set_scene / spk_set_config /
spk_render (frame buffer and tonemapped image), for both RNG policies, with and without NEE, in one group or
in several groups of requests (a small slot budget); and every request matches the CPU oracle's render of it
(parity tolerances of tests/parity.py)."""
import numpy as np
import pytest

import oracle
from sparkle_gb300 import abi, native, scenes

from parity import assert_image_parity, compare_images, oracle_image

pytestmark = pytest.mark.gpu

REQS = [  # scene, width, height, spp, bounce, seed
    (0, 48, 32, 1, 5, 1),
    (1, 64, 64, 8, 8, 2),
    (2, 17, 23, 3, 3, 3),
    (0, 96, 40, 70, 4, 4),  # more than one 64-frame pass when rendered alone
    (2, 40, 40, 16, 8, 5),
    (1, 33, 31, 2, 1, 6),
]


@pytest.fixture(scope="module")
def three_scenes(cornell, small_terrain):
    return [cornell, small_terrain, scenes.random_training_scene(5)]


# batch_slots 0: every request in one group; 20000: groups of whole requests of at most 20000 items, and the
# 268,800-item request alone in its group, regenerating its slots
@pytest.mark.parametrize("rng,nee,slots", [(abi.SPK_RNG_XOSHIRO256SS, False, 0), (abi.SPK_RNG_XOSHIRO256SS, True, 0),
                                           (abi.SPK_RNG_XOSHIRO128P, True, 0), (abi.SPK_RNG_XOSHIRO256SS, True, 20000)])
def test_batch_matches_single_renders(three_scenes, rng, nee, slots):
    batch = native.Context(0)
    batch.set_tuning(batch_slots=slots)
    batch.set_scenes([sc for sc, _ in three_scenes])
    requests = []
    for scene, w, h, spp, bounce, seed in REQS:
        cam = scenes.make_camera(three_scenes[scene][1], w, h)
        requests.append(dict(scene=scene, width=w, height=h, spp=spp, bounce=bounce, seed=seed, camera=cam))
    batch.render_batch(requests, rng=rng, enable_nee=nee)
    st = batch.stats()
    assert st["error_flags"] == 0
    assert st["paths"] == sum(w * h * spp for _, w, h, spp, _, _ in REQS)
    assert st["extension_rays"] > 0 and (st["shadow_rays"] > 0) == nee
    single = native.Context(0)
    osc = [oracle.OracleScene(sc) for sc, _ in three_scenes]
    for k, (scene, w, h, spp, bounce, seed) in enumerate(REQS):
        cfg = abi.make_config(w, h, spp=1, max_spp=4096, bounce=bounce, enable_nee=nee, rng=rng, seed=seed,
                              kernel=abi.SPK_KERNEL_WAVEFRONT)
        single.set_scene(three_scenes[scene][0])
        single.set_config(cfg)
        single.set_camera(requests[k]["camera"])
        single.render(spp)
        ref_hdr, ref_out = single.framebuffer()
        hdr, out = batch.read_batch(k)
        assert np.array_equal(hdr.view(np.uint32), ref_hdr.view(np.uint32)), k
        assert np.array_equal(out, ref_out), k
        assert np.isfinite(hdr).all()
        o_hdr, o_out = oracle_image(three_scenes[scene][0], requests[k]["camera"], cfg, spp, osc=osc[scene])
        # with more frames more pixels hold at least one diverged sample (each weighing 1/spp): the 70-spp
        # request keeps >= 98.5% of its pixels within 1e-4 relative
        assert_image_parity(compare_images(hdr, out, o_hdr, o_out), f"batch request {k} vs oracle",
                            min_close=0.995 if spp <= 16 else 0.985)
    single.close()
    batch.close()


def test_batch_validation(cornell):
    c = native.Context(0)
    c.set_scenes([cornell[0]])
    cam = scenes.make_camera(cornell[1], 16, 16)
    for bad in [dict(scene=1, width=16, height=16, spp=1, bounce=2, camera=cam),
                dict(scene=0, width=1, height=16, spp=1, bounce=2, camera=cam),
                dict(scene=0, width=16, height=16, spp=0, bounce=2, camera=cam)]:
        with pytest.raises(native.SpkError):
            c.render_batch([bad])
    assert c.L.spk_read_batch(c.h, 0, None, None) == 1  # no batch rendered yet
    c.close()


def test_scene_zero_is_the_default_scene(cornell, small_terrain):
    """spk_render on a multi-scene context renders scene 0, exactly as a single-scene context does."""
    a, b = native.Context(0), native.Context(0)
    a.set_scenes([small_terrain[0], cornell[0]])
    b.set_scene(small_terrain[0])
    cfg = abi.make_config(40, 30, spp=1, bounce=4, seed=3)
    cam = scenes.make_camera(small_terrain[1], 40, 30)
    for c in (a, b):
        c.set_config(cfg)
        c.set_camera(cam)
        c.render(3)
    assert np.array_equal(a.framebuffer()[0].view(np.uint32), b.framebuffer()[0].view(np.uint32))
    a.close()
    b.close()
