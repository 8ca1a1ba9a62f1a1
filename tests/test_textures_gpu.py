"""Textured materials on the device against the oracle: an sRGB base-colour checker, a metallic-roughness
map, a normal map and a textured emitter (Image2D::Sample bilinear with wrap, MaterialRenderProxy's
texture x factor, MeshRenderProxy's normal mapping). Tolerance as the other image-parity tests: >= 90% of
pixels within 1e-4 relative and relMSE < 1e-3 (transcendental last bits may flip a coin)."""
import numpy as np
import pytest

import oracle
from sparkle_gb300 import abi, native, scenes

from parity import rel_mse

pytestmark = pytest.mark.gpu


def textured_scene():
    rng = np.random.default_rng(3)
    checker = np.zeros((16, 16, 4), np.float32)
    yy, xx = np.mgrid[0:16, 0:16]
    on = ((xx // 4 + yy // 4) % 2).astype(bool)
    checker[on] = [0.9, 0.2, 0.1, 1.0]
    checker[~on] = [0.1, 0.5, 0.9, 1.0]
    mr = np.concatenate([np.zeros((8, 8, 1)), rng.uniform(0.1, 1.0, (8, 8, 1)), rng.uniform(0, 1, (8, 8, 1)),
                         np.ones((8, 8, 1))], -1).astype(np.float32)
    nrm = np.zeros((32, 32, 4), np.float32)
    a = np.linspace(0, 4 * np.pi, 32)
    nrm[..., 0] = 0.5 + 0.3 * np.sin(a)[None, :]
    nrm[..., 1] = 0.5 + 0.3 * np.cos(a)[:, None]
    nrm[..., 2] = 0.9
    nrm[..., 3] = 1.0
    glow = np.zeros((4, 4, 4), np.float32)
    glow[..., :3] = rng.uniform(0.2, 1.0, (4, 4, 3))
    glow[..., 3] = 1.0
    textures = [abi.Texture(checker, srgb=True), abi.Texture(mr), abi.Texture(nrm), abi.Texture(glow, srgb=True)]
    floor = scenes._quad((-2, -2, 0), (2, -2, 0), (2, 2, 0), (-2, 2, 0), (0, 0, 1), (1, 0, 0))
    floor.uvs = floor.uvs * 3.0  # wrap the textures three times
    light = scenes._quad((-0.5, -0.5, 2), (0.5, -0.5, 2), (0.5, 0.5, 2), (-0.5, 0.5, 2), (0, 0, -1), (1, 0, 0))
    cube = scenes.unit_cube()
    mats = [abi.Material((1, 1, 1), (0, 0, 0), 0.5, 0.8, base_color_tex=0, metallic_roughness_tex=1, normal_tex=2),
            abi.Material((1, 1, 1), (6, 6, 6), 0.0, 1.0, emissive_tex=3),
            abi.Material.lambertian((0.7, 0.7, 0.7))]
    mats[2].base_color_tex = 0
    eye = np.eye(3)
    inst = [abi.Instance(0, 0, scenes._affine(eye, (0, 0, 0))), abi.Instance(1, 1, scenes._affine(eye, (0, 0, 0))),
            abi.Instance(2, 2, scenes._affine(eye * 0.8, (0.6, 0.4, 0.4)))]
    sky = abi.Sky(abi.SPK_SKY_GRADIENT, (0.4, 0.6, 1.0), None)
    scene = abi.Scene([floor, light, cube], inst, mats, sky, textures=textures)
    cam = dict(position=(0.0, -4.0, 2.5), target=(0.0, 0.0, 0.3), world_up=(0, 0, 1), vfov_rad=0.9,
               focus_distance=4.0, aperture_radius=0.0, exposure=1.0)
    return scene, cam


@pytest.mark.parametrize("kernel,nee", [(abi.SPK_KERNEL_WAVEFRONT, False), (abi.SPK_KERNEL_MEGAKERNEL, False),
                                        (abi.SPK_KERNEL_WAVEFRONT, True)])
def test_textured_scene_matches_oracle(kernel, nee):
    scene, cam_args = textured_scene()
    W, H = 64, 48
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=4, enable_nee=nee, rng=abi.SPK_RNG_XOSHIRO256SS, seed=2, kernel=kernel)
    ctx = native.Context(0)
    ctx.set_scene(scene)
    ctx.set_config(cfg)
    ctx.set_camera(camera)
    ctx.render(4)
    g, _ = ctx.framebuffer()
    assert ctx.stats()["error_flags"] == 0
    r = oracle.OracleRenderer(oracle.OracleScene(scene), cfg, camera)
    r.render(4, traversal=oracle.PRUNED)
    o, _ = r.framebuffer()
    close = np.all(np.abs(g[..., :3] - o[..., :3]) <= 1e-4 * (1 + np.abs(o[..., :3])), axis=-1).mean()
    assert close >= 0.9 and rel_mse(g, o) < 1e-3, (close, rel_mse(g, o))
    # the textures matter: the untextured scene renders differently
    plain = abi.Scene(scene.meshes, scene.instances, [abi.Material(m.base_color, m.emissive, m.metallic, m.roughness)
                                                      for m in scene.materials], scene.sky)
    ctx.set_scene(plain)
    ctx.set_camera(camera)
    ctx.render(4)
    assert rel_mse(ctx.framebuffer()[0], g) > 1e-2
    ctx.close()


def test_textured_guides_match_oracle():
    scene, cam_args = textured_scene()
    W, H = 64, 48
    camera = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=2)
    ctx = native.Context(0)
    ctx.set_scene(scene)
    ctx.set_config(cfg)
    ctx.set_camera(camera)
    ctx.render_guides()
    nd, al = ctx.guides()
    ond, oal = oracle.OracleRenderer(oracle.OracleScene(scene), cfg, camera).guides()
    ok = np.all(np.abs(al - oal) <= 1e-4 * (1 + np.abs(oal)), axis=-1) & \
        np.all(np.abs(nd - ond) <= 1e-4 * (1 + np.abs(ond)), axis=-1)
    assert ok.mean() > 0.99, ok.mean()
    assert len(np.unique(np.round(al[oal[..., 3] == 1][:, 0], 3))) > 4  # the checker shows in the albedo
    ctx.close()


def test_texture_validation():
    scene, _ = textured_scene()
    scene.materials[0].normal_tex = 7  # out of range
    ctx = native.Context(0)
    with pytest.raises(native.SpkError):
        ctx.set_scene(scene)
    ctx.close()
