"""The baseline JPEG decoder (sparkle_gb300.jpeg) on files written here by a small baseline encoder that
follows T.81 independently (forward DCT, quantisation, zig-zag, DC differences, run-length AC symbols,
canonical Huffman codes of fixed lengths, byte stuffing, restart markers): grey, 4:4:4 and 4:2:0 colour,
restart intervals, 16-bit quantisation tables, and the refusal of progressive files. The decoded image must
equal the encoder's input within the quantisation and rounding it went through (tolerances below)."""
import struct

import numpy as np
import pytest

from sparkle_gb300.jpeg import ZIGZAG, _BASIS, decode_jpeg


def _seg(marker, body):
    return bytes([0xFF, marker]) + struct.pack(">H", len(body) + 2) + body


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value, count):
        for k in range(count - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> k) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc = self.n = 0

    def flush(self):
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)  # pad with 1 bits


def _category(v):
    return 0 if v == 0 else int(abs(v)).bit_length()


def _bits_of(v, s):
    return v if v >= 0 else v + (1 << s) - 1


# Fixed-length canonical codes: 12 DC symbols of 4 bits, the 162 AC symbols of 8 bits.
DC_SYMS = list(range(12))
AC_SYMS = [0x00, 0xF0] + [(r << 4) | s for r in range(16) for s in range(1, 11)]


def _codes(syms, length):
    return {s: (i, length) for i, s in enumerate(syms)}


DC_CODE, AC_CODE = _codes(DC_SYMS, 4), _codes(AC_SYMS, 8)


def encode_jpeg(img, subsample=False, q=1, restart=0, q16=False):
    """Baseline JPEG of an (H, W) grey or (H, W, 3) RGB uint8 image."""
    img = np.asarray(img, np.float64)
    grey = img.ndim == 2
    h, w = img.shape[:2]
    if grey:
        planes = [img]
        samp = [(1, 1)]
    else:
        r, g, b = img[..., 0], img[..., 1], img[..., 2]
        y = 0.299 * r + 0.587 * g + 0.114 * b
        cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128
        cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128
        planes = [y, cb, cr]
        samp = [(2, 2), (1, 1), (1, 1)] if subsample else [(1, 1)] * 3
    hmax = max(s[0] for s in samp)
    vmax = max(s[1] for s in samp)
    mcux, mcuy = -(-w // (8 * hmax)), -(-h // (8 * vmax))
    qtab = np.full(64, q, np.float64)
    out = b"\xff\xd8"
    if q16:
        out += _seg(0xDB, bytes([0x10]) + qtab.astype(">u2").tobytes())
    else:
        out += _seg(0xDB, bytes([0x00]) + qtab.astype(np.uint8).tobytes())
    sof = struct.pack(">BHHB", 8, h, w, len(planes))
    for k, (hh, vv) in enumerate(samp):
        sof += bytes([k + 1, (hh << 4) | vv, 0])
    out += _seg(0xC0, sof)
    dht = bytes([0x00]) + bytes([0, 0, 0, 12] + [0] * 12) + bytes(DC_SYMS)
    dht += bytes([0x10]) + bytes([0] * 7 + [162] + [0] * 8) + bytes(AC_SYMS)
    out += _seg(0xC4, dht)
    if restart:
        out += _seg(0xDD, struct.pack(">H", restart))
    sos = bytes([len(planes)]) + b"".join(bytes([k + 1, 0x00]) for k in range(len(planes))) + bytes([0, 63, 0])
    out += _seg(0xDA, sos)
    # per component: padded plane (edge-replicated), subsampled by block averaging
    comp_planes = []
    for (hh, vv), p in zip(samp, planes):
        fy, fx = vmax // vv, hmax // hh
        ph, pw = mcuy * vmax * 8, mcux * hmax * 8
        padded = np.pad(p, ((0, ph - h), (0, pw - w)), mode="edge")
        sub = padded.reshape(ph // fy, fy, pw // fx, fx).mean(axis=(1, 3))
        comp_planes.append(sub - 128.0)
    bw = _BitWriter()
    pred = [0] * len(planes)
    mcu = 0
    rst = 0
    for my in range(mcuy):
        for mx in range(mcux):
            if restart and mcu and mcu % restart == 0:
                bw.flush()
                bw.out += bytes([0xFF, 0xD0 + rst])
                rst = (rst + 1) % 8
                pred = [0] * len(planes)
            for k, (hh, vv) in enumerate(samp):
                for yy in range(vv):
                    for xx in range(hh):
                        by, bx = my * vv + yy, mx * hh + xx
                        blk = comp_planes[k][by * 8:by * 8 + 8, bx * 8:bx * 8 + 8]
                        coef = _BASIS @ blk @ _BASIS.T
                        qc = np.rint(coef.reshape(-1) / qtab).astype(np.int64)[ZIGZAG]
                        diff = int(qc[0]) - pred[k]
                        pred[k] = int(qc[0])
                        s = _category(diff)
                        bw.put(*DC_CODE[s])
                        bw.put(_bits_of(diff, s), s)
                        run = 0
                        for i in range(1, 64):
                            v = int(qc[i])
                            if v == 0:
                                run += 1
                                continue
                            while run > 15:
                                bw.put(*AC_CODE[0xF0])
                                run -= 16
                            s = _category(v)
                            bw.put(*AC_CODE[(run << 4) | s])
                            bw.put(_bits_of(v, s), s)
                            run = 0
                        if run:
                            bw.put(*AC_CODE[0x00])
            mcu += 1
    bw.flush()
    return out + bytes(bw.out) + b"\xff\xd9"


def smooth_rgb(h, w, seed):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    img = np.stack([128 + 90 * np.sin(xx / 9.0 + seed), 128 + 90 * np.cos(yy / 7.0),
                    128 + 60 * np.sin((xx + yy) / 11.0)], -1)
    return np.clip(img + rng.normal(0, 2, img.shape), 0, 255).astype(np.uint8)


def test_grey_near_lossless():
    img = np.random.default_rng(1).integers(0, 256, (21, 35), np.uint8)
    got = decode_jpeg(encode_jpeg(img, q=1))
    assert got.shape == (21, 35, 4) and np.all(got[..., 3] == 1)
    err = np.abs(np.rint(got[..., 0] * 255) - img.astype(np.float64))
    assert err.max() <= 1.0
    assert np.array_equal(got[..., 0], got[..., 2])


@pytest.mark.parametrize("restart,q16", [(0, False), (3, True)])
def test_colour_444(restart, q16):
    img = smooth_rgb(40, 53, 2)
    got = decode_jpeg(encode_jpeg(img, q=1, restart=restart, q16=q16))
    err = np.abs(np.rint(got[..., :3] * 255) - img.astype(np.float64))
    assert err.max() <= 3.0  # YCbCr rounding both ways + coefficient rounding


def test_colour_420_with_restarts():
    img = smooth_rgb(48, 64, 3)
    got = decode_jpeg(encode_jpeg(img, subsample=True, q=2, restart=2))
    err = np.abs(np.rint(got[..., :3] * 255) - img.astype(np.float64))
    assert err.mean() <= 3.0 and err.max() <= 24.0  # chroma at quarter resolution


def test_quantisation_is_applied():
    img = smooth_rgb(16, 16, 4)
    coarse = decode_jpeg(encode_jpeg(img, q=40))
    fine = decode_jpeg(encode_jpeg(img, q=1))
    e_c = np.abs(coarse[..., :3] * 255 - img).mean()
    e_f = np.abs(fine[..., :3] * 255 - img).mean()
    assert e_f < e_c < 40


def test_refusals():
    with pytest.raises(ValueError):
        decode_jpeg(b"\x89PNG....")
    prog = b"\xff\xd8" + _seg(0xC2, struct.pack(">BHHB", 8, 8, 8, 1) + bytes([1, 0x11, 0])) + b"\xff\xd9"
    with pytest.raises(ValueError):
        decode_jpeg(prog)


def test_tables_against_independent_definitions():
    """The zig-zag order by walking the anti-diagonals, and the IDCT basis against scipy's orthonormal
    DCT-II (the encoder above shares both with the decoder, so they are pinned here on their own)."""
    order = []
    for d in range(15):
        cells = [(r, d - r) for r in range(8) if 0 <= d - r < 8]
        order += cells if d % 2 else cells[::-1]  # even diagonals run up-right, odd ones down-left
    assert list(ZIGZAG) == [r * 8 + c for r, c in order]
    scipy_fft = pytest.importorskip("scipy.fft")
    ref = scipy_fft.dct(np.eye(8), type=2, norm="ortho", axis=0)
    np.testing.assert_allclose(_BASIS, ref, atol=1e-12)
