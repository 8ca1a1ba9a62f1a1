"""Sky maps (sparkle_gb300/sky.py, spk_sky_from_equirect): Radiance files read as Image2D::LoadFromFile
holds them (RGBE -> float -> half), the cube cook of SkyLightCookJob::Execute (SkyLight.cpp:83-113)
against the oracle's restatement, and USD dome lights as the sky. The cook is floating point with atan2 /
asin, so device and oracle agree to one half ulp (relative 2^-10) per texel."""
import numpy as np
import pytest

import oracle
from sparkle_gb300 import abi, native, sky, usd

from image_decode import rgbe_encode


def equirect(h=32, w=64, seed=0):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    img = np.ones((h, w, 4), np.float32)
    img[..., 0] = (0.2 + xx / w).astype(np.float32)             # longitude ramp
    img[..., 1] = (0.1 + 2.0 * yy / h).astype(np.float32)       # latitude ramp
    img[..., 2] = rng.uniform(0, 3, (h, w)).astype(np.float32)  # noise
    img[h // 8, w // 3, :3] = 40.0                              # a sun texel
    return img


def test_hdr_files_read_as_half_texels(tmp_path):
    img = equirect(9, 37, 1)
    p = tmp_path / "sky.hdr"
    native.write_hdr(p, img)
    got = sky.load_sky_map(p)
    e = rgbe_encode(img[..., :3])
    ref = e[..., :3].astype(np.float32) * np.where(e[..., 3:] > 0, np.ldexp(np.float32(1), e[..., 3:].astype(np.int32) - 136), 0)
    assert got.shape == (9, 37, 4) and np.all(got[..., 3] == 1)
    np.testing.assert_array_equal(got[..., :3], ref.astype(np.float16).astype(np.float32))


def test_oracle_cook_maps_directions_as_the_reference():
    img = equirect()
    cube = oracle.sky_from_equirect(img, False, 8)
    assert cube.shape == (6, 8, 8, 4) and np.all(cube[..., 3] == 1)
    flat = np.ones((4, 8, 4), np.float32) * np.float32(0.7)
    np.testing.assert_array_equal(oracle.sky_from_equirect(flat, False, 4)[..., :3], np.float16(0.7).astype(np.float32))
    c = oracle.sky_from_equirect(img, False, 64)
    # +Z (face 4) centre looks at the map's top row (asin(-1) -> v = 0); +Y (face 2) at the equator
    assert c[4, 31:33, 31:33, 1].mean() < 0.2 and abs(c[2, 31:33, 31:33, 1].mean() - 1.1) < 0.1
    # +X (face 0) centre has longitude 0 -> u = 0.5 (red 0.7); -X centre u = 1, which wraps to column 0
    assert abs(c[0, 31:33, 31:33, 0].mean() - 0.7) < 0.05 and c[1, 31:33, 31:33, 0].mean() < 0.7


def test_usd_dome_light_colour_becomes_the_gradient_sky(tmp_path):
    text = '''#usda 1.0
(
    defaultPrim = "root"
)
def Xform "root"
{
    def DomeLight "sky"
    {
        color3f inputs:color = (0.5, 0.25, 1)
        float inputs:intensity = 2
        float inputs:exposure = 1
    }
}
'''
    p = tmp_path / "d.usda"
    p.write_text(text)
    sc = usd.load_usda(str(p))
    assert sc.sky.mode == abi.SPK_SKY_GRADIENT and sc.sky.color == pytest.approx((2.0, 1.0, 4.0))


@pytest.mark.gpu
@pytest.mark.parametrize("srgb,n", [(False, 16), (True, 16), (False, 61)])
def test_device_cook_matches_oracle(srgb, n):
    img = equirect(48, 96, 2)
    if srgb:
        img[..., :3] = np.clip(img[..., :3] / 4, 0, 1)
    got = sky.cube_from_equirect(img, srgb, n)
    ref = oracle.sky_from_equirect(img, srgb, n)
    tol = np.abs(ref) * 2.0 ** -10 + 1e-7
    assert np.all(np.abs(got - ref) <= tol)
    assert (got == ref).mean() > 0.99


@pytest.mark.gpu
def test_usd_textured_dome_light(tmp_path):
    img = equirect(16, 32, 3)
    native.write_hdr(tmp_path / "env.hdr", img)
    text = '''#usda 1.0
(
    defaultPrim = "root"
)
def Xform "root"
{
    def DomeLight "sky"
    {
        asset inputs:texture:file = @env.hdr@
    }
}
'''
    p = tmp_path / "t.usda"
    p.write_text(text)
    sc = usd.load_usda(str(p), sky_size=8)
    assert sc.sky.mode == abi.SPK_SKY_CUBE and sc.sky.cube.shape == (6, 8, 8, 4)
    np.testing.assert_array_equal(sc.sky.cube, sky.cube_from_equirect(sky.load_sky_map(tmp_path / "env.hdr"), False, 8))
