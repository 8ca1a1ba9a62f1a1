"""Shared comparison helpers of the parity tests (hit records and images)."""
from __future__ import annotations

import numpy as np

INVALID = 0xFFFFFFFF


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
