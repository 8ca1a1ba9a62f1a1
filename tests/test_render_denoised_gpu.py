"""spk_render_denoised (one C-ABI call) against sparkle_gb300.denoise.render_denoised (the same steps driven
from Python): same frame, same fallback tiles, bit for bit."""
import numpy as np
import pytest

from sparkle_gb300 import abi, denoise, native, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("spp", [1, 4])
def test_one_call_denoised_frame_equals_the_python_pipeline(small_terrain, spp):
    scene, cam_args = small_terrain
    W, H = 96, 64
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=5, enable_nee=True, rng=abi.SPK_RNG_XOSHIRO256SS, seed=2,
                          max_spp=4096)
    dn = native.Denoiser(0, seed=0)
    denoise.load_weights(dn)
    out = []
    for path in ("python", "abi"):
        ctx = native.Context(0)
        ctx.set_scene(scene)
        ctx.set_config(cfg)
        ctx.set_camera(camera)
        if path == "python":
            fr = denoise.render_denoised(ctx, dn, camera, spp, tile=16, threshold=0.02)
            out.append((fr.image, fr.fallback_tiles))
        else:
            out.append(dn.render_denoised(ctx, spp, tile=16, threshold=0.02))
        ctx.close()
    (a, ta), (b, tb) = out
    assert ta == tb
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.isfinite(b).all() and b[..., :3].mean() > 0
    dn.close()
