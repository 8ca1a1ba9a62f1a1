"""TEST INFRASTRUCTURE ONLY -- comparisons of device results with the oracle's (hit records and images).

Used by tests/ and __graft_entry__.smoke(); never by the product path.
"""
from __future__ import annotations

import numpy as np

INVALID = 0xFFFFFFFF


def axis_parallel(rays: np.ndarray) -> np.ndarray:
    """Rays with a direction component |d| <= FLT_EPSILON: the reference's slab test (bvh v2 safe_inverse
    = +-FLT_MAX, inv_org = -inv * org) overflows for them and culls whole levels once |org| > 1, so they
    are checked against the tree-independent brute-force oracle instead of the oracle's BVH walk."""
    return np.any(np.abs(rays[:, 3:]) <= np.finfo(np.float32).eps, axis=1)


def oracle_hits(osc, rays: np.ndarray, pruned: int):
    """Closest hits of the oracle scene `osc` (axis-parallel rays by brute force); (hits, axis-parallel mask)."""
    ref, ovf = osc.trace(rays, traversal=pruned)
    assert ovf == 0, "oracle walk stack overflow"
    quirk = axis_parallel(rays)
    if quirk.any():
        ref[quirk] = osc.trace_brute(rays[quirk])
    return ref, quirk


def classify_hits(gpu: np.ndarray, ref: np.ndarray) -> dict:
    """Compares two hit-record arrays (HIT_DTYPE). A ray counts as `exact` when primitive, face, t, u and v
    are bit-identical; `tie` when both hit at bit-identical t but different (prim, face) (which of two
    hits at exactly equal t wins depends on the visit order); `gpu_closer` / `ref_closer` when one side
    reports a strictly smaller t or the other misses (a triangle one walk culled on a grazing box test)."""
    g_hit = gpu["prim"] != INVALID
    r_hit = ref["prim"] != INVALID
    same_id = (gpu["prim"] == ref["prim"]) & (gpu["face"] == ref["face"])
    same_t = gpu["t"].view(np.uint32) == ref["t"].view(np.uint32)
    same_uv = (gpu["u"].view(np.uint32) == ref["u"].view(np.uint32)) & (gpu["v"].view(np.uint32) == ref["v"].view(np.uint32))
    both_miss = ~g_hit & ~r_hit
    exact = both_miss | (g_hit & r_hit & same_id & same_t & same_uv)
    mism = ~exact
    tie = mism & g_hit & r_hit & same_t & ~same_id
    gpu_closer = mism & g_hit & (~r_hit | (gpu["t"] < ref["t"]))
    ref_closer = mism & r_hit & (~g_hit | (ref["t"] < gpu["t"]))
    other = mism & ~tie & ~gpu_closer & ~ref_closer
    n = len(gpu)
    return {"n": n, "exact": int(exact.sum()), "tie": int(tie.sum()), "gpu_closer": int(gpu_closer.sum()),
            "ref_closer": int(ref_closer.sum()), "other": int(other.sum()), "hits": int(r_hit.sum()),
            "mismatch_idx": np.nonzero(mism)[0]}


def rel_mse(x: np.ndarray, ref: np.ndarray) -> float:
    """mean over pixels and channels of (x - ref)^2 / (ref^2 + 0.01)."""
    x = x[..., :3].astype(np.float64)
    ref = ref[..., :3].astype(np.float64)
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + 0.01)))


def close_fraction(a: np.ndarray, b: np.ndarray, rel: float = 1e-4) -> float:
    """Fraction of pixels whose three colour channels agree to `rel` relative (1e-4 * (1 + |ref|))."""
    d = np.abs(a[..., :3] - b[..., :3])
    ok = np.all(d <= rel * (1.0 + np.abs(b[..., :3])), axis=-1)
    return float(ok.mean())


def compare_images(g_hdr: np.ndarray, g_out, o_hdr: np.ndarray, o_out) -> dict:
    """Per-pixel comparison of a device render with the oracle's on the same seeds. `*_hdr` are the frame
    buffers (rows bottom-up, float4), `*_out` the tonemapped RGBA16F images (rows top-down, the vertical
    flip of ToneMappingPass) or None. Reports the pixel count, the pixels whose frame-buffer value is
    bit-identical in all four channels, the pixels that differ, the fraction within 1e-4 relative, the
    relMSE, and -- over the bit-identical pixels -- how many tonemapped pixels differ in any bit (the
    tonemap is a pure function of the frame-buffer pixel, so that count must be 0)."""
    same = np.all(g_hdr.view(np.uint32) == o_hdr.view(np.uint32), axis=-1)
    res = {"pixels": int(same.size), "identical": int(same.sum()), "differing": int((~same).sum()),
           "close": close_fraction(g_hdr, o_hdr), "relmse": rel_mse(g_hdr, o_hdr)}
    if g_out is not None and o_out is not None:
        same_top = same[::-1]  # output row H-1-j holds frame-buffer row j
        out_eq = np.all(g_out.view(np.uint16) == o_out.view(np.uint16), axis=-1)
        res["tonemap_checked"] = int(same_top.sum())
        res["tonemap_mismatch"] = int((same_top & ~out_eq).sum())
    return res
