"""Image output: the screenshot conversion (ConvertPixelsToRGBA8 of RGBA16F, Image.cpp:54-67) against the
oracle for every half value, and the PNG / Radiance HDR / OpenEXR encoders read back by independent
decoders (tests/image_decode.py). The encoders and the host conversion need no GPU; the device path
(spk_read_rgba8, spk_save_image) is checked on the GPU against the same."""
import numpy as np
import pytest

import oracle
from sparkle_gb300 import abi, native, scenes

from image_decode import read_exr, read_hdr_rgbe, read_png, rgbe_encode


def all_halves():
    return np.arange(65536, dtype=np.uint32).astype(np.uint16).reshape(-1, 1, 4)


def test_conversion_matches_oracle_for_every_half():
    src = all_halves()
    got = native.convert_rgba8(src)
    ref = oracle.rgba16f_to_rgba8(src)
    assert np.array_equal(got, ref)
    # alpha channel of every half too (the last channel takes the alpha rule)
    rot = np.roll(src.reshape(-1), 3).reshape(-1, 1, 4)
    assert np.array_equal(native.convert_rgba8(rot), oracle.rgba16f_to_rgba8(rot))


def test_conversion_known_values():
    h = np.array([[[0.0, 1.0, 0.5, 0.5], [2.0, -1.0, 0.0031, 1.0]]], np.float16).view(np.uint16)
    out = native.convert_rgba8(h)
    # 0 -> 0; 1 -> 255; 0.5 -> round(255 * 0.5^0.45) = 187; alpha 0.5 -> lround(127.5) = 128; clamp above
    # and below; half(0.0031)^0.45 * 255 = 18.95 -> 19
    assert out.tolist() == [[[0, 255, 187, 128], [255, 0, 19, 255]]]


@pytest.mark.parametrize("w,h", [(1, 1), (7, 3), (64, 33), (200, 120)])
def test_png_round_trip(tmp_path, w, h):
    rng = np.random.default_rng(w * h)
    yy, xx = np.mgrid[0:h, 0:w]
    img = np.zeros((h, w, 4), np.uint8)
    img[..., 0] = (xx * 3) & 255               # gradients (Sub / Up / Paeth filters, long matches)
    img[..., 1] = (yy * 5 + xx) & 255
    img[..., 2] = rng.integers(0, 256, (h, w))  # noise (literals)
    img[..., 3] = 255
    img[h // 2:, : w // 2] = [10, 20, 30, 40]   # a flat block (runs)
    p = tmp_path / "a.png"
    native.write_png(p, img)
    assert np.array_equal(read_png(p.read_bytes()), img)


@pytest.mark.parametrize("w,h", [(1, 1), (5, 2), (64, 9), (300, 4)])
def test_hdr_round_trip(tmp_path, w, h):
    rng = np.random.default_rng(w + h)
    img = np.zeros((h, w, 4), np.float32)
    img[..., :3] = rng.lognormal(0, 2, (h, w, 3)).astype(np.float32)
    img[0, 0, :3] = 0.0
    if w > 3:
        img[:, 1:4, :3] = 7.25       # runs in every component
        img[-1, -1, :3] = [-1.0, 0.5, 0.25]  # negatives clamp to 0
    p = tmp_path / "a.hdr"
    native.write_hdr(p, img)
    got = read_hdr_rgbe(p.read_bytes())
    assert np.array_equal(got, rgbe_encode(img[..., :3]))
    # decoded values are within RGBE precision (8-bit mantissa of the largest channel)
    dec = got[..., :3].astype(np.float64) * np.ldexp(1.0, got[..., 3].astype(np.int32) - 136)[..., None]
    ref = np.maximum(img[..., :3], 0)
    assert np.all(np.abs(dec - ref) <= ref.max(axis=-1, keepdims=True) / 128 + 1e-30)


@pytest.mark.parametrize("w,h", [(1, 1), (6, 4), (97, 31)])
def test_exr_round_trip(tmp_path, w, h):
    rng = np.random.default_rng(w)
    img = rng.normal(0, 10, (h, w, 4)).astype(np.float16).view(np.uint16)
    p = tmp_path / "a.exr"
    native.write_exr(p, img)
    assert np.array_equal(read_exr(p.read_bytes()), img)


def test_write_errors(tmp_path):
    with pytest.raises(native.SpkError) as e:
        native.write_png(tmp_path / "no" / "such" / "dir.png", np.zeros((2, 2, 4), np.uint8))
    assert e.value.status == 7
    with pytest.raises(ValueError):
        native.write_png(tmp_path / "x.png", np.zeros((2, 2, 3), np.uint8))


@pytest.mark.gpu
def test_device_screenshot_and_files(tmp_path, cornell):
    scene, cam_args = cornell
    W, H = 80, 60
    ctx = native.Context(0)
    ctx.set_scene(scene)
    ctx.set_config(abi.make_config(W, H, spp=2, bounce=4, seed=1))
    ctx.set_camera(scenes.make_camera(cam_args, W, H))
    ctx.render(4)
    hdr, out = ctx.framebuffer()
    shot = ctx.read_rgba8()
    assert np.array_equal(shot, oracle.rgba16f_to_rgba8(out))
    assert len(np.unique(shot[..., 0])) > 20
    ctx.save_image(tmp_path / "s.png", abi.SPK_IMAGE_PNG)
    assert np.array_equal(read_png((tmp_path / "s.png").read_bytes()), shot)
    top = hdr[::-1]  # the frame buffer runs bottom up, files top down
    ctx.save_image(tmp_path / "s.exr", abi.SPK_IMAGE_EXR)
    assert np.array_equal(read_exr((tmp_path / "s.exr").read_bytes()), top.astype(np.float16).view(np.uint16))
    ctx.save_image(tmp_path / "s.hdr", abi.SPK_IMAGE_HDR)
    assert np.array_equal(read_hdr_rgbe((tmp_path / "s.hdr").read_bytes()), rgbe_encode(top[..., :3]))
    with pytest.raises(native.SpkError):
        ctx.save_image(tmp_path / "s.xyz", 9)
    ctx.close()
