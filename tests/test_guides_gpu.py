"""Primary-hit guides (spk_render_guides) against the oracle's restatement of WritePrimaryHitGBuffer
(ray_trace.cs.slang:282-351): same hit/miss and emissive flags, same base colour, normal and linear depth
within 1e-5 relative, on pixels whose closest hit is not an exact tie between two faces (at most 1%)."""
import numpy as np
import pytest

import oracle
from sparkle_gb300 import abi, native, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = native.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("which", ["cornell", "terrain"])
def test_guides_match_oracle(ctx, cornell, small_terrain, which):
    scene, cam_args = cornell if which == "cornell" else small_terrain
    W, H = 96, 64
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=4)
    ctx.set_scene(scene)
    ctx.set_config(cfg)
    ctx.set_camera(camera)
    ctx.render_guides()
    nd, al = ctx.guides()
    assert ctx.stats()["error_flags"] == 0
    r = oracle.OracleRenderer(oracle.OracleScene(scene), cfg, camera)
    ond, oal = r.guides()
    same_flag = al[..., 3] == oal[..., 3]
    assert same_flag.mean() > 0.99
    ok = same_flag & np.all(al[..., :3] == oal[..., :3], axis=-1)
    ok &= np.all(np.abs(nd - ond) <= 1e-5 * (1 + np.abs(ond)), axis=-1)
    assert ok.mean() > 0.99, ok.mean()
    hit = oal[..., 3] > 0
    assert hit.mean() > 0.3
    assert np.allclose(np.linalg.norm(nd[hit][:, :3], axis=-1), 1.0, atol=1e-5)
    assert np.all(nd[hit][:, 3] > 0)  # in front of the camera
    assert np.all(nd[~hit] == 0) and np.all(al[~hit] == 0)
    if which == "cornell":
        assert (al[..., 3] == 2).any()  # the ceiling light is seen


def test_guides_need_a_scene():
    c = native.Context(0)
    with pytest.raises(native.SpkError):
        c.render_guides()
    c.close()
