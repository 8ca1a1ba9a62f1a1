"""Sky maps: reading them as the reference's Image2D::LoadFromFile holds them and cooking the cube the path
tracer samples on a miss (spk_sky_from_equirect, the restatement of SkyLightCookJob::Execute).

* Radiance .hdr files (Image.cpp:154-180 through stb_image's RGBE decode): each texel r8 * 2^(e - 136)
  (0 when e = 0), clamped to +-65504 and rounded to half (RGBAFloat16), alpha 1. Flat and new-style
  run-length scanlines are read.
* PNG files (Image.cpp:184-197): 8-bit RGBA / 255 as R8G8B8A8Unorm (linear: no sRGB decode on sampling).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi, native
from .gltf import decode_image

CUBE_SIZE = 1024  # SkyLight.cpp:24


def decode_hdr(data: bytes) -> np.ndarray:
    """(H, W, 4) float32 texels of a Radiance RGBE file, rounded to half as RGBAFloat16 stores them."""
    if not (data.startswith(b"#?RADIANCE") or data.startswith(b"#?RGBE")):
        raise ValueError("not a Radiance HDR file")
    end = data.index(b"\n\n") + 2
    header = data[:end].decode("ascii", "replace")
    if "FORMAT=32-bit_rle_rgbe" not in header and "FORMAT=" in header:
        raise ValueError("only 32-bit_rle_rgbe Radiance files are read")
    line_end = data.index(b"\n", end)
    parts = data[end:line_end].split()
    if len(parts) != 4 or parts[0] != b"-Y" or parts[2] != b"+X":
        raise ValueError("only -Y H +X W Radiance files are read")
    h, w = int(parts[1]), int(parts[3])
    pos = line_end + 1
    rgbe = np.zeros((h, w, 4), np.uint8)
    buf = np.frombuffer(data, np.uint8)
    for y in range(h):
        if w >= 8 and w < 32768 and data[pos] == 2 and data[pos + 1] == 2 and (data[pos + 2] & 0x80) == 0:
            if (data[pos + 2] << 8 | data[pos + 3]) != w:
                raise ValueError("run-length scanline of the wrong width")
            pos += 4
            for c in range(4):
                x = 0
                while x < w:
                    n = data[pos]
                    pos += 1
                    if n > 128:
                        n -= 128
                        rgbe[y, x:x + n, c] = data[pos]
                        pos += 1
                    else:
                        if n == 0:
                            raise ValueError("bad run-length scanline")
                        rgbe[y, x:x + n, c] = buf[pos:pos + n]
                        pos += n
                    x += n
        else:
            rgbe[y] = buf[pos:pos + 4 * w].reshape(w, 4)
            pos += 4 * w
    e = rgbe[..., 3].astype(np.int32)
    scale = np.where(e > 0, np.ldexp(np.float32(1.0), e - 136).astype(np.float32), np.float32(0.0))
    out = np.ones((h, w, 4), np.float32)
    out[..., :3] = rgbe[..., :3].astype(np.float32) * scale[..., None]
    out[..., :3] = np.clip(out[..., :3], -65504.0, 65504.0).astype(np.float16).astype(np.float32)
    return out


def load_sky_map(path) -> np.ndarray:
    """(H, W, 4) float32 texels of a .hdr, .png or .jpg sky map (Image2D::LoadFromFile)."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] == b"\x89PNG\r\n\x1a\n" or data[:2] == b"\xff\xd8":
        return decode_image(data)
    return decode_hdr(data)


def cube_from_equirect(rgba, srgb: bool = False, size: int = CUBE_SIZE, device: int = 0) -> np.ndarray:
    """(6, size, size, 4) cube faces (+X, -X, +Y, -Y, +Z, -Z) cooked from an equirectangular map on the GPU."""
    src = np.ascontiguousarray(rgba, np.float32)
    if src.ndim != 3 or src.shape[2] != 4:
        raise ValueError("sky map texels must be (H, W, 4)")
    out = np.zeros((6, size, size, 4), np.float32)
    st = native.lib().spk_sky_from_equirect(device, native._p(src), src.shape[1], src.shape[0], int(srgb), size,
                                           native._p(out))
    if st != 0:
        raise native.SpkError(st, "spk_sky_from_equirect failed")
    return out


def sky_from_file(path, size: int = CUBE_SIZE, device: int = 0) -> abi.Sky:
    """SkyLight::SetSkyMap(path) for the path tracer: the cooked cube as an SPK_SKY_CUBE sky."""
    return abi.Sky(abi.SPK_SKY_CUBE, (0.0, 0.0, 0.0), cube_from_equirect(load_sky_map(path), False, size, device))
