"""Baseline JPEG decoding for imported textures and sky maps (the reference's loaders decode JPEG files with
stb_image, a dependency absent from its tree).

Restates the sequential DCT-based process of ITU-T T.81 (JPEG, ISO/IEC 10918-1) as JFIF files use it:

* markers SOI, APPn (the Adobe APP14 transform flag is honoured), DQT (8- and 16-bit tables), SOF0 / SOF1
  (8-bit sample precision, Huffman coding), DHT, DRI, SOS, RSTn, EOI; progressive, lossless, arithmetic
  coded, 12-bit and four-component files are refused with a ValueError;
* Huffman decoding with the MINCODE / MAXCODE / VALPTR procedure of T.81 F.2.2.3, DC prediction per
  component (reset at each restart interval), run-length AC coefficients, interleaved and single-component
  scans;
* dequantisation, the 8 x 8 inverse DCT of T.81 A.3.3 in float64, level shift and rounding;
* chroma upsampling by the triangle (3/4, 1/4) filter along each subsampled axis, edges replicated, and the
  JFIF YCbCr -> RGB conversion (ITU-T T.871).

The inverse DCT and the upsampling are computed in floating point and rounded once, so decoded samples can
differ from stb_image's integer pipeline by a step or two; textures keep their shapes and levels.
"""
from __future__ import annotations

import struct

import numpy as np

# Zig-zag scan order of T.81 Figure A.6: position k of the coded sequence -> row-major index in the block.
ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27,
                   20, 13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58,
                   59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63], np.int64)


def _idct_basis() -> np.ndarray:
    """C[u, x] = c(u) / 2 * cos((2x + 1) u pi / 16), c(0) = 1 / sqrt(2): block = C^T F C (T.81 A.3.3)."""
    u = np.arange(8)[:, None]
    x = np.arange(8)[None, :]
    c = np.where(u == 0, 1.0 / np.sqrt(2.0), 1.0)
    return c / 2.0 * np.cos((2 * x + 1) * u * np.pi / 16.0)


_BASIS = _idct_basis()


class _Huffman:
    """Decoding tables of one DHT table (T.81 F.2.2.3)."""

    def __init__(self, counts, symbols):
        self.symbols = list(symbols)
        self.maxcode = [-1] * 17
        self.mincode = [0] * 17
        self.valptr = [0] * 17
        code = k = 0
        for length in range(1, 17):
            n = counts[length - 1]
            if n:
                self.valptr[length] = k
                self.mincode[length] = code
                code += n
                k += n
                self.maxcode[length] = code - 1
            code <<= 1


class _Bits:
    """MSB-first bit reader over one entropy-coded segment with the 0xFF00 stuffing already removed."""

    def __init__(self, data: bytes):
        self.data = data
        self.pos = 0
        self.acc = 0
        self.n = 0

    def bit(self) -> int:
        if self.n == 0:
            self.acc = self.data[self.pos] if self.pos < len(self.data) else 0  # past the end: zeros
            self.pos += 1
            self.n = 8
        self.n -= 1
        return (self.acc >> self.n) & 1

    def bits(self, count: int) -> int:
        v = 0
        for _ in range(count):
            v = (v << 1) | self.bit()
        return v

    def decode(self, table: _Huffman) -> int:
        code = self.bit()
        length = 1
        while code > table.maxcode[length]:
            code = (code << 1) | self.bit()
            length += 1
            if length > 16:
                raise ValueError("corrupt JPEG: bad Huffman code")
        return table.symbols[table.valptr[length] + code - table.mincode[length]]


def _extend(v: int, s: int) -> int:
    """T.81 F.2.2.1 EXTEND: the s-bit magnitude category value v as a signed difference."""
    return v - (1 << s) + 1 if s and v < (1 << (s - 1)) else v


def _segments(data: bytes, start: int):
    """Entropy-coded data of a scan from `start`: (segments split at RSTn markers, offset after the scan)."""
    segs, cur, i = [], bytearray(), start
    while i < len(data):
        b = data[i]
        if b != 0xFF:
            cur.append(b)
            i += 1
            continue
        nxt = data[i + 1] if i + 1 < len(data) else 0xD9
        if nxt == 0x00:
            cur.append(0xFF)
            i += 2
        elif 0xD0 <= nxt <= 0xD7:
            segs.append(bytes(cur))
            cur = bytearray()
            i += 2
        elif nxt == 0xFF:
            i += 1  # fill byte
        else:
            break  # a marker ends the scan
    segs.append(bytes(cur))
    return segs, i


def _upsample(plane: np.ndarray, fy: int, fx: int) -> np.ndarray:
    """Triangle-filter upsampling by integer factors (1 or 2 per axis; larger factors replicate)."""
    out = plane.astype(np.float64)
    for axis, f in ((0, fy), (1, fx)):
        if f == 1:
            continue
        if f != 2:
            out = np.repeat(out, f, axis=axis)
            continue
        lo = np.concatenate([np.take(out, [0], axis=axis), np.take(out, range(out.shape[axis] - 1), axis=axis)], axis)
        hi = np.concatenate([np.take(out, range(1, out.shape[axis]), axis=axis),
                             np.take(out, [out.shape[axis] - 1], axis=axis)], axis)
        even, odd = 0.75 * out + 0.25 * lo, 0.75 * out + 0.25 * hi
        out = np.stack([even, odd], axis=axis + 1).reshape(
            out.shape[:axis] + (2 * out.shape[axis],) + out.shape[axis + 1:])
    return out


def decode_jpeg(data: bytes) -> np.ndarray:
    """Baseline JPEG -> (H, W, 4) float32 in [0, 1] (grey replicated to RGB, alpha 1)."""
    if data[:2] != b"\xff\xd8":
        raise ValueError("not a JPEG file")
    qt = {}
    huff = {}
    frame = None
    comps = []
    restart = 0
    adobe_transform = None
    coefs = None
    i = 2
    while i < len(data):
        if data[i] != 0xFF:
            raise ValueError("corrupt JPEG: marker expected")
        marker = data[i + 1]
        i += 2
        if marker in (0xD8, 0x01) or 0xD0 <= marker <= 0xD7:
            continue
        if marker == 0xD9:
            break
        length, = struct.unpack(">H", data[i:i + 2])
        seg = data[i + 2:i + length]
        if marker == 0xDB:  # DQT
            k = 0
            while k < len(seg):
                pq, tq = seg[k] >> 4, seg[k] & 15
                if pq:
                    vals = np.frombuffer(seg[k + 1:k + 129], ">u2").astype(np.float64)
                    k += 129
                else:
                    vals = np.frombuffer(seg[k + 1:k + 65], np.uint8).astype(np.float64)
                    k += 65
                q = np.zeros(64)
                q[ZIGZAG] = vals
                qt[tq] = q.reshape(8, 8)
        elif marker in (0xC0, 0xC1):  # SOF0 / SOF1: Huffman, sequential
            precision, h, w, nc = struct.unpack(">BHHB", seg[:6])
            if precision != 8:
                raise ValueError(f"{precision}-bit JPEG samples are not decoded")
            if nc not in (1, 3):
                raise ValueError(f"JPEG with {nc} components is not decoded")
            if h == 0:
                raise ValueError("JPEG without a height in its frame header (DNL) is not decoded")
            for c in range(nc):
                cid, hv, tq = seg[6 + 3 * c:9 + 3 * c]
                comps.append({"id": cid, "h": hv >> 4, "v": hv & 15, "tq": tq})
            frame = (h, w)
            hmax = max(c["h"] for c in comps)
            vmax = max(c["v"] for c in comps)
            mcux, mcuy = -(-w // (8 * hmax)), -(-h // (8 * vmax))
            coefs = []
            for c in comps:
                c["bw"], c["bh"] = mcux * c["h"], mcuy * c["v"]  # blocks, padded to whole MCUs
                coefs.append(np.zeros((c["bh"], c["bw"], 64), np.float64))
        elif 0xC2 <= marker <= 0xCF and marker not in (0xC4, 0xC8, 0xCC):
            raise ValueError("progressive, lossless and arithmetic-coded JPEGs are not decoded")
        elif marker == 0xC4:  # DHT
            k = 0
            while k < len(seg):
                tc, th = seg[k] >> 4, seg[k] & 15
                counts = list(seg[k + 1:k + 17])
                n = sum(counts)
                huff[(tc, th)] = _Huffman(counts, seg[k + 17:k + 17 + n])
                k += 17 + n
        elif marker == 0xDD:  # DRI
            restart, = struct.unpack(">H", seg[:2])
        elif marker == 0xEE and seg[:5] == b"Adobe" and len(seg) >= 12:
            adobe_transform = seg[11]
        elif marker == 0xDA:  # SOS
            if frame is None:
                raise ValueError("corrupt JPEG: scan before frame header")
            ns = seg[0]
            scomps = []
            for c in range(ns):
                cid, tables = seg[1 + 2 * c:3 + 2 * c]
                idx = next(k for k, cc in enumerate(comps) if cc["id"] == cid)
                scomps.append((idx, huff[(0, tables >> 4)], huff[(1, tables & 15)]))
            segs, i = _segments(data, i + length)
            _decode_scan(segs, scomps, comps, coefs, restart, frame)
            continue
        i += length
    if frame is None:
        raise ValueError("JPEG without a frame header")
    h, w = frame
    hmax = max(c["h"] for c in comps)
    vmax = max(c["v"] for c in comps)
    planes = []
    for c, co in zip(comps, coefs):
        blocks = co.reshape(c["bh"], c["bw"], 8, 8) * qt[c["tq"]]
        spatial = np.einsum("ux,abuv,vy->abxy", _BASIS, blocks, _BASIS) + 128.0
        plane = spatial.transpose(0, 2, 1, 3).reshape(c["bh"] * 8, c["bw"] * 8)
        plane = np.clip(np.rint(plane), 0, 255)
        plane = _upsample(plane, vmax // c["v"], hmax // c["h"])[:h, :w]
        planes.append(plane)
    rgba = np.ones((h, w, 4), np.float32)
    if len(planes) == 1:
        rgba[..., :3] = (np.clip(np.rint(planes[0]), 0, 255) / 255.0)[..., None]
        return rgba
    y, cb, cr = planes
    if adobe_transform == 0:  # stored as RGB
        rgb = np.stack([y, cb, cr], -1)
    else:  # JFIF YCbCr (ITU-T T.871)
        rgb = np.stack([y + 1.402 * (cr - 128.0), y - 0.344136 * (cb - 128.0) - 0.714136 * (cr - 128.0),
                        y + 1.772 * (cb - 128.0)], -1)
    rgba[..., :3] = (np.clip(np.rint(rgb), 0, 255) / 255.0).astype(np.float32)
    return rgba


def _decode_scan(segs, scomps, comps, coefs, restart, frame):
    """Huffman-decodes one sequential scan into the components' coefficient arrays (zig-zag order)."""
    h, w = frame
    hmax = max(c["h"] for c in comps)
    vmax = max(c["v"] for c in comps)
    if len(scomps) == 1:  # non-interleaved: the component's own blocks in raster order
        idx = scomps[0][0]
        c = comps[idx]
        bw = -(-(-(-w * c["h"] // hmax)) // 8)
        bh = -(-(-(-h * c["v"] // vmax)) // 8)
        units = [[(idx, by, bx)] for by in range(bh) for bx in range(bw)]
    else:
        mcux, mcuy = -(-w // (8 * hmax)), -(-h // (8 * vmax))
        units = []
        for my in range(mcuy):
            for mx in range(mcux):
                u = []
                for idx, _, _ in scomps:
                    c = comps[idx]
                    for yy in range(c["v"]):
                        for xx in range(c["h"]):
                            u.append((idx, my * c["v"] + yy, mx * c["h"] + xx))
                units.append(u)
    tables = {idx: (dc, ac) for idx, dc, ac in scomps}
    per_segment = restart if restart else len(units)
    for s, start in enumerate(range(0, len(units), per_segment)):
        bits = _Bits(segs[s] if s < len(segs) else b"")
        pred = {idx: 0 for idx in tables}
        for unit in units[start:start + per_segment]:
            for idx, by, bx in unit:
                dc_t, ac_t = tables[idx]
                block = np.zeros(64)
                t = bits.decode(dc_t)
                pred[idx] += _extend(bits.bits(t), t)
                block[0] = pred[idx]
                k = 1
                while k < 64:
                    rs = bits.decode(ac_t)
                    r, size = rs >> 4, rs & 15
                    if size == 0:
                        if r == 15:
                            k += 16
                            continue
                        break  # end of block
                    k += r
                    if k > 63:
                        raise ValueError("corrupt JPEG: coefficient index past 63")
                    block[k] = _extend(bits.bits(size), size)
                    k += 1
                natural = np.zeros(64)
                natural[ZIGZAG] = block
                coefs[idx][by, bx] = natural
