"""TEST INFRASTRUCTURE ONLY -- float64 numpy restatement of LDR-FLIP, the checker for the device evaluator.

The reference scores its rendering tests with the mean FLIP error of a screenshot against a ground-truth
PNG (tests/rendering/render_test_support.py:43-59: both images read as RGB / 255, then
flip_evaluator.nbflip.evaluate(reference, test, False, True, False, True, {}) -- LDR inputs in sRGB, default
parameters, mean returned). flip_evaluator (NVIDIA's FLIP package, 1.x) is not installed here, so this
module restates the published algorithm (Andersson et al., "FLIP: A Difference Evaluator for Alternating
Images", HPG 2020) and parity to the package is unpinned:

 colour: sRGB -> linear RGB -> XYZ -> YCxCz; each channel convolved with its contrast-sensitivity filter
   S(r) = a1 sqrt(pi/b1) exp(-pi^2 r^2/b1) + a2 sqrt(pi/b2) exp(-pi^2 r^2/b2) (r in degrees, kernel
   normalised to sum 1; A: 1, .0047, 0, 1e-5; RG: 1, .0053, 0, 1e-5; BY: 34.1, .04, 13.5, .025; radius
   ceil(3 sqrt(max b / (2 pi^2)) ppd)); back to linear RGB clamped to [0, 1]; CIELAB; Hunt adjustment
   (a, b scaled by L/100); HyAB distance |dL| + |(da, db)|; raised to 0.7 and mapped piecewise linearly
   with pc = 0.4, pt = 0.95 against cmax = HyAB(green, blue)^0.7.
 features: Y / Yn of each image filtered by the first (edges) and second (points) x / y derivatives of a
   Gaussian with sd = 0.5 * 0.082 ppd (radius ceil(3 sd); positive weights normalised to sum 1, negative to
   -1); dF = (max(|d|edge||, |d|point||) / sqrt 2)^0.5.
 FLIP = dEc^(1 - dF) per pixel; images are extended at the borders by replication. Default 67.02 pixels per
 degree (0.7 m from a 0.7 m wide 3840-pixel screen).
"""
from __future__ import annotations

import numpy as np

PPD = 0.7 * (3840 / 0.7) * np.pi / 180.0

RGB2XYZ = np.array([[0.4124564, 0.3575761, 0.1804375],
                    [0.2126729, 0.7151522, 0.0721750],
                    [0.0193339, 0.1191920, 0.9503041]])
XYZ2RGB = np.linalg.inv(RGB2XYZ)
WHITE = RGB2XYZ.sum(axis=1)  # XYZ of linear RGB (1, 1, 1)

CSF = {"A": (1.0, 0.0047, 0.0, 1e-5), "RG": (1.0, 0.0053, 0.0, 1e-5), "BY": (34.1, 0.04, 13.5, 0.025)}
QC, PC, PT, QF, FEATURE_WIDTH = 0.7, 0.4, 0.95, 0.5, 0.082


def srgb_to_linear(c):
    c = np.asarray(c, np.float64)
    return np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)


def linear_to_ycxcz(rgb):
    xyz = rgb @ RGB2XYZ.T / WHITE
    return np.stack([116.0 * xyz[..., 1] - 16.0, 500.0 * (xyz[..., 0] - xyz[..., 1]),
                     200.0 * (xyz[..., 1] - xyz[..., 2])], -1)


def ycxcz_to_linear(ycc):
    y = (ycc[..., 0] + 16.0) / 116.0
    xyz = np.stack([ycc[..., 1] / 500.0 + y, y, y - ycc[..., 2] / 200.0], -1) * WHITE
    return xyz @ XYZ2RGB.T


def linear_to_lab(rgb):
    t = rgb @ RGB2XYZ.T / WHITE
    d = 6.0 / 29.0
    f = np.where(t > d ** 3, np.cbrt(t), t / (3 * d * d) + 4.0 / 29.0)
    return np.stack([116.0 * f[..., 1] - 16.0, 500.0 * (f[..., 0] - f[..., 1]), 200.0 * (f[..., 1] - f[..., 2])], -1)


def hunt(lab):
    return np.stack([lab[..., 0], 0.01 * lab[..., 0] * lab[..., 1], 0.01 * lab[..., 0] * lab[..., 2]], -1)


def hyab(a, b):
    d = a - b
    return np.abs(d[..., 0]) + np.sqrt(d[..., 1] ** 2 + d[..., 2] ** 2)


def spatial_radius(ppd):
    bmax = max(max(p[1], p[3]) for p in CSF.values())
    return int(np.ceil(3.0 * np.sqrt(bmax / (2.0 * np.pi ** 2)) * ppd))


def spatial_kernel(channel, ppd):
    a1, b1, a2, b2 = CSF[channel]
    r = spatial_radius(ppd)
    x = np.arange(-r, r + 1) / ppd
    r2 = x[None, :] ** 2 + x[:, None] ** 2
    g = a1 * np.sqrt(np.pi / b1) * np.exp(-np.pi ** 2 * r2 / b1) + a2 * np.sqrt(np.pi / b2) * np.exp(-np.pi ** 2 * r2 / b2)
    return g / g.sum()


def feature_kernels(ppd):
    """(edge_x, point_x) kernels; the y kernels are their transposes."""
    sd = 0.5 * FEATURE_WIDTH * ppd
    r = int(np.ceil(3.0 * sd))
    x, y = np.meshgrid(np.arange(-r, r + 1), np.arange(-r, r + 1))
    g = np.exp(-(x ** 2 + y ** 2) / (2.0 * sd * sd))
    out = []
    for k in (-x * g, (x ** 2 / (sd * sd) - 1.0) * g):
        neg, pos = -k[k < 0].sum(), k[k > 0].sum()
        out.append(np.where(k < 0, k / neg, k / pos))
    return out


def convolve(img, k):
    """Same-size 2D correlation with border replication (kernels here are symmetric or transposed pairs)."""
    r = k.shape[0] // 2
    p = np.pad(img, ((r, r), (r, r)), mode="edge")
    h, w = img.shape
    out = np.zeros((h, w))
    for dy in range(k.shape[0]):
        for dx in range(k.shape[1]):
            out += k[dy, dx] * p[dy:dy + h, dx:dx + w]
    return out


def cmax():
    g = hunt(linear_to_lab(np.array([0.0, 1.0, 0.0])))
    b = hunt(linear_to_lab(np.array([0.0, 0.0, 1.0])))
    return hyab(g, b) ** QC


def flip_map(reference, test, ppd=PPD):
    """Per-pixel LDR-FLIP of two (H, W, 3) sRGB images in [0, 1]."""
    ref_lin, test_lin = srgb_to_linear(reference), srgb_to_linear(test)
    filtered = []
    for img in (ref_lin, test_lin):
        ycc = linear_to_ycxcz(img)
        f = np.stack([convolve(ycc[..., c], spatial_kernel(ch, ppd)) for c, ch in enumerate(("A", "RG", "BY"))], -1)
        filtered.append(hunt(linear_to_lab(np.clip(ycxcz_to_linear(f), 0.0, 1.0))))
    de = hyab(filtered[0], filtered[1]) ** QC
    cm = cmax()
    dec = np.where(de < PC * cm, PT / (PC * cm) * de, PT + (de - PC * cm) / (cm - PC * cm) * (1.0 - PT))
    ex, px = feature_kernels(ppd)
    feats = []
    for img in (ref_lin, test_lin):
        y = (img @ RGB2XYZ.T / WHITE)[..., 1]
        e = np.hypot(convolve(y, ex), convolve(y, ex.T))
        p = np.hypot(convolve(y, px), convolve(y, px.T))
        feats.append((e, p))
    df = np.maximum(np.abs(feats[0][0] - feats[1][0]), np.abs(feats[0][1] - feats[1][1]))
    df = (df / np.sqrt(2.0)) ** QF
    return dec ** (1.0 - df)


def flip_mean(reference, test, ppd=PPD):
    return float(flip_map(reference, test, ppd).mean())


def rel_mse(x, ref, eps=0.01):
    """relMSE = mean over pixels and channels of (x - ref)^2 / (ref^2 + eps)."""
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.mean((x - ref) ** 2 / (ref * ref + eps)))
