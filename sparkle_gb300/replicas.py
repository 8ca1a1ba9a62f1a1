"""Replicas: the path shards by sample, so N GPUs render disjoint samples of the same view and the only
exchange is one sample-weighted reduction of the HDR frame buffers (no collective on the data path).

The reference renders on one host thread pool and has no multi-device path; this is the host-side split
and merge that make N replicas equivalent to one renderer with N times the samples. Each replica keeps
the view's seed and starts its frames where the previous replicas' end (`spk_config.sample_offset`): the
per-pixel seeds of frame f are built from the dispatched sample count (j*W + i + frame_seed*W*H for the
reference's Xoshiro128+, CPURenderer.cpp:436-444; (seed, frame, pixel) for xoshiro256**), so replica r
rendering F frames from offset r*F*spp draws exactly frames r*F .. (r+1)*F-1 of the single renderer.

The merge is the sample-weighted mean of the replicas' running means, which equals the single renderer's
running mean up to rounding while every replica's accumulation stays below `max_spp`. Past that cap the
reference's lerp turns into an exponential moving average (CameraRenderProxy.cpp:66-75) that weights
recent frames more, and no merge of independent replicas reproduces it: keep frames per replica <= max_spp.
"""
from __future__ import annotations

import numpy as np


def replica_sample_offset(rank: int, frames_per_replica: int, spp_eff: int = 1, base: int = 0) -> int:
    """spk_config.sample_offset of replica `rank` when every replica renders `frames_per_replica` frames of
    `spp_eff` samples (the config's round(sqrt(spp))^2) after `base` samples of the view."""
    return (base + rank * frames_per_replica * spp_eff) & 0xFFFFFFFF


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
