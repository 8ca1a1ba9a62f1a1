"""Replicas: the path shards by sample, so N GPUs render independent sample streams of the same view and the
only exchange is one sample-weighted reduction of the HDR frame buffers (no collective on the data path).

The reference renders on one host thread pool and has no multi-device path; this is the host-side merge that
makes N replicas equivalent to one renderer with N times the samples.
"""
from __future__ import annotations

import numpy as np


def replica_seed(base_seed: int, rank: int) -> int:
    """Per-replica seed of the xoshiro256** policy, so replicas draw disjoint sample streams."""
    return (base_seed + 0x9E3779B9 * rank) & 0xFFFFFFFF


def merge_framebuffers(hdr: np.ndarray, samples: int, group=None) -> np.ndarray:
    """Sample-weighted mean of every rank's accumulated HDR frame buffer (float4 per pixel), computed in
    float64 with torch.distributed all_reduce (gloo for host tensors). Returns the merged buffer."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(hdr, dtype=np.float64) * float(samples))
    n = torch.tensor([float(samples)], dtype=torch.float64)
    dist.all_reduce(t, group=group)
    dist.all_reduce(n, group=group)
    if n.item() <= 0:
        raise ValueError("no samples on any rank")
    return (t / n).numpy().astype(np.float32)
