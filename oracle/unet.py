"""TEST INFRASTRUCTURE ONLY -- numpy FP32 restatement of the learned denoiser (include/spk_denoise.h).

The checker for the tensor-core convolutions and the U-Net training step: 3x3 convolution forward, input
gradient and weight gradient; 2x2 average pooling and nearest upsampling with their backward passes; the
skip concatenations; the relMSE loss. With `bf16=True` every tensor the device stores in BF16 is rounded
to BF16 (round to nearest even) at the same point the device rounds it, so the comparison isolates the
FP32 accumulation order. Nothing here is used by the product path.

The reference has no learned denoiser (its cpu pipeline's only denoiser is the spatial fill of
CPURenderer::DenoisePass, CPURenderer.cpp:452-526), so this module restates the network the
specification describes, not reference code.
"""
from __future__ import annotations

import numpy as np

LEVELS = 5
WIDTHS = (32, 64, 96, 128, 128)
IN_PAD = 32
OUT_PAD = 32
FEATURES = 10
OUT_CLAMP = 16.0


def to_bf16(x: np.ndarray) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def _r(x, bf16):
    return to_bf16(x) if bf16 else x.astype(np.float32)


# --------------------------------------------------------------------------------------------------
# convolution (NHWC, weights [cout][3][3][cin], zero padding 1)
# --------------------------------------------------------------------------------------------------
def conv3x3(x: np.ndarray, w: np.ndarray, b: np.ndarray | None = None) -> np.ndarray:
    n, h, wd, cin = x.shape
    cout = w.shape[0]
    xp = np.zeros((n, h + 2, wd + 2, cin), np.float32)
    xp[:, 1:-1, 1:-1] = x
    y = np.zeros((n, h, wd, cout), np.float32)
    for dy in range(3):
        for dx in range(3):
            y += xp[:, dy:dy + h, dx:dx + wd, :] @ w[:, dy, dx, :].T.astype(np.float32)
    if b is not None:
        y += b.astype(np.float32)
    return y


def conv3x3_dgrad(gy: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Input gradient: gx[q] = sum_t gy[q - o_t] w_t, o_t = (dy - 1, dx - 1)."""
    n, h, wd, cout = gy.shape
    cin = w.shape[3]
    gp = np.zeros((n, h + 2, wd + 2, cout), np.float32)
    gp[:, 1:-1, 1:-1] = gy
    gx = np.zeros((n, h, wd, cin), np.float32)
    for dy in range(3):
        for dx in range(3):
            gx += gp[:, 2 - dy:2 - dy + h, 2 - dx:2 - dx + wd, :] @ w[:, dy, dx, :].astype(np.float32)
    return gx


def conv3x3_wgrad(x: np.ndarray, gy: np.ndarray) -> np.ndarray:
    """Weight gradient [cout][3][3][cin]: sum_p gy[p] (x) x[p + o_t]."""
    n, h, wd, cin = x.shape
    cout = gy.shape[3]
    xp = np.zeros((n, h + 2, wd + 2, cin), np.float32)
    xp[:, 1:-1, 1:-1] = x
    gw = np.zeros((cout, 3, 3, cin), np.float32)
    g2 = gy.reshape(-1, cout)
    for dy in range(3):
        for dx in range(3):
            gw[:, dy, dx, :] = g2.T @ xp[:, dy:dy + h, dx:dx + wd, :].reshape(-1, cin)
    return gw


def pool2(x):
    s = ((x[:, 0::2, 0::2] + x[:, 0::2, 1::2]) + x[:, 1::2, 0::2]) + x[:, 1::2, 1::2]
    return np.float32(0.25) * s


def upsample2(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def upsample2_bwd(g):
    return ((g[:, 0::2, 0::2] + g[:, 0::2, 1::2]) + g[:, 1::2, 0::2]) + g[:, 1::2, 1::2]


def pool2_bwd(g):
    return upsample2(np.float32(0.25) * g)


# --------------------------------------------------------------------------------------------------
# network
# --------------------------------------------------------------------------------------------------
def layer_shapes():
    """(cin, cout, relu) in the device's layer order: enc0a enc0b ... enc4b, dec3a dec3b ... dec0b, out."""
    L = []
    for l in range(LEVELS):
        L.append((IN_PAD if l == 0 else WIDTHS[l - 1], WIDTHS[l], True))
        L.append((WIDTHS[l], WIDTHS[l], True))
    for l in (3, 2, 1, 0):
        L.append((WIDTHS[l + 1] + WIDTHS[l], WIDTHS[l], True))
        L.append((WIDTHS[l], WIDTHS[l], True))
    L.append((WIDTHS[0], OUT_PAD, False))
    return L


def enc_a(l):
    return 2 * l


def enc_b(l):
    return 2 * l + 1


def dec_a(l):
    return 10 + 2 * (3 - l)


def dec_b(l):
    return 11 + 2 * (3 - l)


OUT_LAYER = 18


def unpack_params(flat: np.ndarray):
    """Flat device parameter vector -> [(w [cout][3][3][cin], b [cout])]."""
    out, off = [], 0
    for cin, cout, _ in layer_shapes():
        nw = cout * 9 * cin
        w = flat[off:off + nw].reshape(cout, 3, 3, cin)
        off += nw
        b = flat[off:off + cout]
        off += cout
        out.append((w, b))
    assert off == flat.size
    return out


def pack_params(layers) -> np.ndarray:
    return np.concatenate([np.concatenate([w.reshape(-1), b.reshape(-1)]) for w, b in layers]).astype(np.float32)


def input_tensor(features: np.ndarray, bf16: bool = True) -> np.ndarray:
    n, h, w, _ = features.shape
    x = np.zeros((n, h, w, IN_PAD), np.float32)
    x[..., :FEATURES] = features
    return _r(x, bf16)


def forward(params_flat, features, bf16: bool = True):
    """Returns the output tensor (n, h, w, OUT_PAD) and the saved activations."""
    P = unpack_params(params_flat)
    Pw = [(_r(w, bf16), b) for w, b in P]
    act = {}
    x = input_tensor(features, bf16)
    act["x0"] = x
    inp = x
    for l in range(LEVELS):
        w, b = Pw[enc_a(l)]
        ea = _r(np.maximum(conv3x3(inp, w, b), 0), bf16)
        w, b = Pw[enc_b(l)]
        eb = _r(np.maximum(conv3x3(ea, w, b), 0), bf16)
        act[f"ea{l}"], act[f"eb{l}"] = ea, eb
        if l < 4:
            inp = _r(pool2(eb), bf16)
            act[f"pool{l}"] = inp
    up = act["eb4"]
    for l in (3, 2, 1, 0):
        cat = np.concatenate([upsample2(up), act[f"eb{l}"]], axis=-1)
        w, b = Pw[dec_a(l)]
        da = _r(np.maximum(conv3x3(cat, w, b), 0), bf16)
        w, b = Pw[dec_b(l)]
        db = _r(np.maximum(conv3x3(da, w, b), 0), bf16)
        act[f"cat{l}"], act[f"da{l}"], act[f"db{l}"] = cat, da, db
        up = db
    w, b = Pw[OUT_LAYER]
    out = _r(conv3x3(act["db0"], w, b), bf16)
    return out, act, Pw


def loss_and_grad(out: np.ndarray, target: np.ndarray, bf16: bool = True):
    """relMSE = mean((expm1(o) - t)^2 / (t^2 + 0.01)) over pixels and the 3 colour channels."""
    o = out[..., :3].astype(np.float32)
    clamped = o > OUT_CLAMP
    o = np.minimum(o, np.float32(OUT_CLAMP))
    e = np.exp(o).astype(np.float32)
    d = e - np.float32(1.0)
    den = target * target + np.float32(0.01)
    diff = d - target
    loss = float(np.mean((diff * diff / den).astype(np.float64)))
    scale = np.float32(1.0 / (3.0 * o.shape[0] * o.shape[1] * o.shape[2]))
    g = np.zeros_like(out, dtype=np.float32)
    g[..., :3] = np.where(clamped, 0.0, np.float32(2.0) * diff / den * e * scale)
    return loss, _r(g, bf16)


def backward(act, Pw, gout, bf16: bool = True):
    """Gradients of every layer [(gw, gb)] from the output gradient, in the device's rounding points."""
    grads = [None] * len(Pw)

    def lg(li, x, gy):
        grads[li] = (conv3x3_wgrad(x, gy), gy.reshape(-1, gy.shape[-1]).sum(axis=0, dtype=np.float32))

    relu = lambda g, ref: g * (ref > 0)
    lg(OUT_LAYER, act["db0"], gout)
    gdb = _r(relu(conv3x3_dgrad(gout, Pw[OUT_LAYER][0]), act["db0"]), bf16)
    geb = {}
    gcat = {}
    for l in (0, 1, 2, 3):
        lg(dec_b(l), act[f"da{l}"], gdb)
        gda = _r(relu(conv3x3_dgrad(gdb, Pw[dec_b(l)][0]), act[f"da{l}"]), bf16)
        lg(dec_a(l), act[f"cat{l}"], gda)
        gc = _r(conv3x3_dgrad(gda, Pw[dec_a(l)][0]), bf16)
        gcat[l] = gc
        cu = WIDTHS[l + 1]
        ref = act[f"db{l + 1}"] if l < 3 else act["eb4"]
        g_up = _r(relu(upsample2_bwd(gc[..., :cu]), ref), bf16)
        if l < 3:
            gdb = g_up
        else:
            geb[4] = g_up
    for l in (4, 3, 2, 1, 0):
        lg(enc_b(l), act[f"ea{l}"], geb[l])
        gea = _r(relu(conv3x3_dgrad(geb[l], Pw[enc_b(l)][0]), act[f"ea{l}"]), bf16)
        inp = act["x0"] if l == 0 else act[f"pool{l - 1}"]
        lg(enc_a(l), inp, gea)
        if l == 0:
            break
        gpool = _r(conv3x3_dgrad(gea, Pw[enc_a(l)][0]), bf16)
        skip = gcat[l - 1][..., WIDTHS[l]:]
        g = (np.float32(0.25) * upsample2(gpool)) + skip
        geb[l - 1] = _r(relu(g, act[f"eb{l - 1}"]), bf16)
    return grads


def gradients(params_flat, features, target, bf16: bool = True):
    out, act, Pw = forward(params_flat, features, bf16)
    loss, gout = loss_and_grad(out, target, bf16)
    grads = backward(act, Pw, gout, bf16)
    return loss, pack_params(grads), out


def pack_features(hdr, normal_depth, albedo):
    """The device's feature packing: log1p(rgb), albedo, normal, log1p(depth) / 4."""
    f = np.empty(hdr.shape[:-1] + (FEATURES,), np.float32)
    f[..., 0:3] = np.log1p(np.maximum(hdr[..., :3], 0))
    f[..., 3:6] = albedo[..., :3]
    f[..., 6:9] = normal_depth[..., :3]
    f[..., 9] = 0.25 * np.log1p(np.maximum(normal_depth[..., 3], 0))
    return f


def decode(out):
    return np.maximum(np.expm1(np.minimum(out[..., :3], OUT_CLAMP)), 0)
