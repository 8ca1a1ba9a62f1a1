"""The PNG texture decoder (sparkle_gb300.gltf.decode_png) on files built here byte by byte from the PNG
specification: every row filter (None, Sub, Up, Average, Paeth), palette images with tRNS alpha, 16-bit
samples (high byte kept, as the reference's loader reduces 16-bit images), 1-bit grey, grey + alpha,
Adam7-interlaced files, and the library's own PNG writer."""
import struct
import time
import zlib

import numpy as np
import pytest

from sparkle_gb300.gltf import decode_png


def _chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def _paeth(a, b, c):
    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _filter_rows(rows, bpp, filters):
    """PNG filtering of raw scanlines (a list of bytes), filter type per row."""
    out, prev = [], bytes(len(rows[0]))
    for y, row in enumerate(rows):
        f = filters[y % len(filters)]
        enc = bytearray()
        for x, v in enumerate(row):
            a = row[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            pred = [0, a, b, (a + b) >> 1, _paeth(a, b, c)][f]
            enc.append((v - pred) & 0xFF)
        out.append(bytes([f]) + bytes(enc))
        prev = row
    return b"".join(out)


def make_png(w, h, ctype, depth, rows, bpp, filters=(0,), palette=None, trns=None, interlace=0):
    data = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, interlace))
    if palette is not None:
        data += _chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        data += _chunk(b"tRNS", bytes(np.asarray(trns, np.uint8)))
    data += _chunk(b"IDAT", zlib.compress(_filter_rows(rows, bpp, filters)))
    return data + _chunk(b"IEND", b"")


def test_rgba8_every_filter():
    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, (9, 13, 4), np.uint8)
    png = make_png(13, 9, 6, 8, [img[y].tobytes() for y in range(9)], 4, filters=(0, 1, 2, 3, 4))
    got = decode_png(png)
    np.testing.assert_array_equal(np.rint(got * 255).astype(np.uint8), img)


def test_rgb16_keeps_the_high_byte():
    rng = np.random.default_rng(2)
    img = rng.integers(0, 65536, (5, 7, 3), np.uint16)
    rows = [img[y].astype(">u2").tobytes() for y in range(5)]
    got = decode_png(make_png(7, 5, 2, 16, rows, 6, filters=(4, 3, 1)))
    np.testing.assert_array_equal(np.rint(got[..., :3] * 255).astype(np.uint8), (img >> 8).astype(np.uint8))
    assert np.all(got[..., 3] == 1)


def test_palette_4bit_with_alpha():
    palette = [[255, 0, 0], [0, 255, 0], [0, 0, 255], [10, 20, 30], [200, 100, 50]]
    trns = [0, 128]  # entries 0 and 1; the rest opaque
    rng = np.random.default_rng(3)
    idx = rng.integers(0, 5, (6, 11), np.uint8)
    rows = []
    for y in range(6):
        r = list(idx[y]) + [0]  # pad to whole bytes
        rows.append(bytes((r[2 * i] << 4) | r[2 * i + 1] for i in range(6)))
    got = decode_png(make_png(11, 6, 3, 4, rows, 1, filters=(2, 1), palette=palette, trns=trns))
    pal = np.array(palette, np.float32) / 255
    alpha = np.array([0, 128, 255, 255, 255], np.float32) / 255
    np.testing.assert_allclose(got[..., :3], pal[idx], atol=1e-7)
    np.testing.assert_allclose(got[..., 3], alpha[idx], atol=1e-7)


def test_grey_1bit_and_grey_alpha():
    bits = np.array([[1, 0, 1, 1, 0, 0, 1, 0, 1], [0, 1, 0, 0, 1, 1, 0, 1, 0]], np.uint8)
    rows = [bytes([int("".join(map(str, r[:8])), 2), r[8] << 7]) for r in bits]
    got = decode_png(make_png(9, 2, 0, 1, rows, 1))
    np.testing.assert_array_equal(got[..., 0], bits.astype(np.float32))
    ga = np.random.default_rng(4).integers(0, 256, (3, 4, 2), np.uint8)
    got = decode_png(make_png(4, 3, 4, 8, [ga[y].tobytes() for y in range(3)], 2, filters=(3,)))
    np.testing.assert_array_equal(np.rint(got[..., 0] * 255).astype(np.uint8), ga[..., 0])
    np.testing.assert_array_equal(np.rint(got[..., 3] * 255).astype(np.uint8), ga[..., 1])


def test_adam7_interlaced():
    """Seven passes of sub-images (x0, y0, dx, dy), each filtered on its own; empty passes carry no bytes."""
    adam7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))
    for h, w in ((9, 13), (3, 2), (1, 1), (16, 17)):
        img = np.random.default_rng(h * w).integers(0, 256, (h, w, 4), np.uint8)
        stream = b""
        for k, (x0, y0, dx, dy) in enumerate(adam7):
            sub = img[y0::dy, x0::dx]
            if sub.size == 0:
                continue
            stream += _filter_rows([sub[y].tobytes() for y in range(sub.shape[0])], 4, (k % 5, 4, 1))
        png = (b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 1)) +
               _chunk(b"IDAT", zlib.compress(stream)) + _chunk(b"IEND", b""))
        np.testing.assert_array_equal(np.rint(decode_png(png) * 255).astype(np.uint8), img, err_msg=f"{h}x{w}")


def test_truncated_data_is_refused():
    with pytest.raises(ValueError):
        decode_png(make_png(2, 2, 6, 8, [bytes(8), bytes(8)], 4, interlace=1)[:-40] + _chunk(b"IEND", b""))


def test_large_texture_decodes_in_seconds():
    rng = np.random.default_rng(5)
    img = rng.integers(0, 256, (256, 256, 4), np.uint8)
    png = make_png(256, 256, 6, 8, [img[y].tobytes() for y in range(256)], 4, filters=(1, 2, 0))
    t0 = time.perf_counter()
    got = decode_png(png)
    assert time.perf_counter() - t0 < 5.0
    np.testing.assert_array_equal(np.rint(got * 255).astype(np.uint8), img)


def test_decodes_the_library_png_writer(tmp_path):
    """spk_write_png picks a filter per row (least absolute residual): random and smooth images read back."""
    from sparkle_gb300 import native
    rng = np.random.default_rng(6)
    yy, xx = np.mgrid[0:40, 0:70]
    smooth = np.stack([(xx * 3) % 256, (yy * 5) % 256, ((xx + yy) * 2) % 256, np.full_like(xx, 200)],
                      -1).astype(np.uint8)
    for k, img in enumerate((rng.integers(0, 256, (40, 70, 4), np.uint8), smooth)):
        p = tmp_path / f"w{k}.png"
        native.write_png(p, img)
        got = decode_png(p.read_bytes())
        np.testing.assert_array_equal(np.rint(got * 255).astype(np.uint8), img)
