"""Independent readers for the image files the library writes (test infrastructure): PNG through Python's
zlib with the five PNG filters undone, Radiance RGBE (flat or new-style run-length scanlines) and
uncompressed scanline OpenEXR with half channels; plus Ward's RGBE encoding restated in numpy."""
import struct
import zlib

import numpy as np


def read_png(data: bytes) -> np.ndarray:
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w = 8, b"", None
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(kind + body) & 0xFFFFFFFF, kind
        if kind == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 6
        elif kind == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    stride = 4 * w
    out = np.zeros((h, stride), np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        row = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int32)
        up = out[y - 1] if y else np.zeros(stride, np.int32)
        cur = np.zeros(stride, np.int32)
        for x in range(stride):
            a = cur[x - 4] if x >= 4 else 0
            b = up[x]
            c = up[x - 4] if x >= 4 else 0
            if f == 0:
                p = 0
            elif f == 1:
                p = a
            elif f == 2:
                p = b
            elif f == 3:
                p = (a + b) >> 1
            else:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
            cur[x] = (row[x] + p) & 255
        out[y] = cur
    return out.astype(np.uint8).reshape(h, w, 4)


def rgbe_encode(rgb: np.ndarray) -> np.ndarray:
    """Ward's RGBE: e = frexp exponent of max(r, g, b); mantissas r * (m * 256 / max) truncated."""
    c = np.maximum(rgb.astype(np.float32), np.float32(0))
    v = c.max(axis=-1)
    m, e = np.frexp(v)
    ok = (v >= np.float32(1e-32)) & np.isfinite(v)
    scale = np.where(ok, m.astype(np.float32) * np.float32(256) / np.where(ok, v, 1), 0).astype(np.float32)
    out = np.zeros(rgb.shape[:-1] + (4,), np.uint8)
    out[..., :3] = np.where(ok[..., None], (c * scale[..., None]).astype(np.int32), 0)
    out[..., 3] = np.where(ok, e + 128, 0)
    return out


def read_hdr_rgbe(data: bytes) -> np.ndarray:
    """(H, W, 4) RGBE bytes of a Radiance file."""
    head_end = data.index(b"\n\n") + 2
    assert data.startswith(b"#?RADIANCE")
    line_end = data.index(b"\n", head_end)
    parts = data[head_end:line_end].split()
    assert parts[0] == b"-Y" and parts[2] == b"+X"
    h, w = int(parts[1]), int(parts[3])
    pos = line_end + 1
    out = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        if data[pos] == 2 and data[pos + 1] == 2 and (data[pos + 2] << 8 | data[pos + 3]) == w and w >= 8:
            pos += 4
            for c in range(4):
                x = 0
                while x < w:
                    n = data[pos]
                    pos += 1
                    if n > 128:
                        out[y, x:x + n - 128, c] = data[pos]
                        pos += 1
                        x += n - 128
                    else:
                        assert n > 0
                        out[y, x:x + n, c] = np.frombuffer(data, np.uint8, n, pos)
                        pos += n
                        x += n
                assert x == w
        else:
            out[y] = np.frombuffer(data, np.uint8, 4 * w, pos).reshape(w, 4)
            pos += 4 * w
    assert pos == len(data)
    return out


def read_exr(data: bytes) -> np.ndarray:
    """(H, W, 4) RGBA half bits (uint16) of an uncompressed scanline OpenEXR file with HALF channels."""
    assert data[:4] == b"\x76\x2f\x31\x01" and data[4] == 2
    pos, attrs = 8, {}
    while data[pos] != 0:
        name_end = data.index(b"\0", pos)
        name = data[pos:name_end].decode()
        type_end = data.index(b"\0", name_end + 1)
        kind = data[name_end + 1:type_end].decode()
        size, = struct.unpack("<i", data[type_end + 1:type_end + 5])
        attrs[name] = (kind, data[type_end + 5:type_end + 5 + size])
        pos = type_end + 5 + size
    pos += 1
    assert attrs["compression"][1] == b"\0"
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    chl, names, q = attrs["channels"][1], [], 0
    while chl[q] != 0:
        e = chl.index(b"\0", q)
        names.append(chl[q:e].decode())
        ptype, = struct.unpack("<i", chl[e + 1:e + 5])
        assert ptype == 1
        q = e + 17
    offsets = struct.unpack(f"<{h}Q", data[pos:pos + 8 * h])
    out = np.zeros((h, w, 4), np.uint16)
    order = {"R": 0, "G": 1, "B": 2, "A": 3}
    for off in offsets:
        y, size = struct.unpack("<ii", data[off:off + 8])
        assert size == 2 * w * len(names)
        line = np.frombuffer(data, "<u2", w * len(names), off + 8).reshape(len(names), w)
        for k, name in enumerate(names):
            out[y - y0, :, order[name]] = line[k]
    return out
