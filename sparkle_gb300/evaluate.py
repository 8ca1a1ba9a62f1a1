"""Image evaluators on the GPU: LDR-FLIP and relMSE (spk_flip, spk_relmse), and the reference's
screenshot comparison flow (tests/rendering/render_test_support.py:43-59: both PNGs read as RGB / 255,
mean FLIP of the screenshot against the ground truth)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native
from .gltf import decode_image

PIXELS_PER_DEGREE = 0.7 * (3840 / 0.7) * np.pi / 180.0  # FLIP's default viewing condition


def flip(reference, test, pixels_per_degree: float = PIXELS_PER_DEGREE, device: int = 0, return_map: bool = False):
    """Mean LDR-FLIP of `test` against `reference`, (H, W, 3) sRGB images in [0, 1]; with return_map also
    the (H, W) per-pixel error."""
    ref = np.ascontiguousarray(reference, np.float32)
    tst = np.ascontiguousarray(test, np.float32)
    if ref.shape != tst.shape or ref.ndim != 3 or ref.shape[2] != 3:
        raise ValueError(f"image size mismatch or not RGB: {ref.shape} vs {tst.shape}")
    h, w, _ = ref.shape
    emap = np.zeros((h, w), np.float32) if return_map else None
    mean = C.c_double()
    st = native.lib().spk_flip(device, native._p(ref), native._p(tst), w, h, pixels_per_degree,
                               None if emap is None else native._p(emap), C.byref(mean))
    if st != 0:
        raise native.SpkError(st, "spk_flip failed")
    return (mean.value, emap) if return_map else mean.value


def rel_mse(x, reference, eps: float = 0.01, device: int = 0) -> float:
    """mean((x - ref)^2 / (ref^2 + eps)) over every value."""
    a = np.ascontiguousarray(x, np.float32)
    b = np.ascontiguousarray(reference, np.float32)
    if a.shape != b.shape:
        raise ValueError(f"shape mismatch: {a.shape} vs {b.shape}")
    out = C.c_double()
    st = native.lib().spk_relmse(device, native._p(a), native._p(b), a.size, eps, C.byref(out))
    if st != 0:
        raise native.SpkError(st, "spk_relmse failed")
    return out.value


def load_image(path) -> np.ndarray:
    """A PNG (or baseline JPEG) as (H, W, 3) float32 RGB / 255 (render_test_support.load_image)."""
    with open(path, "rb") as f:
        return decode_image(f.read())[..., :3]


def compare_images(ground_truth, screenshot, device: int = 0) -> float:
    """Mean FLIP of a screenshot PNG against a ground-truth PNG (render_test_support.compare_images)."""
    gt = load_image(ground_truth)
    sc = load_image(screenshot)
    if gt.shape != sc.shape:
        raise ValueError(f"Image size mismatch: {gt.shape} vs {sc.shape}")
    return flip(gt, sc, device=device)
