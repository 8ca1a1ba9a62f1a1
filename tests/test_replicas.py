"""Multi-rank host logic on CPU (gloo, world size 2): two replicas render disjoint sample streams with the
oracle and merge their frame buffers; the merge equals the sample-weighted mean of the two renders."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from sparkle_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _render(rank, frames):
    import oracle
    from sparkle_gb300 import abi, scenes
    scene, cam_args = scenes.cornell_box(0)
    cam = scenes.make_camera(cam_args, 16, 12)
    cfg = abi.make_config(16, 12, spp=1, bounce=4, rng=abi.SPK_RNG_XOSHIRO256SS, seed=replicas.replica_seed(5, rank))
    r = oracle.OracleRenderer(oracle.OracleScene(scene), cfg, cam)
    r.render(frames)
    return r.framebuffer()[0]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    frames = 3 + rank  # uneven sample counts per replica
    hdr = _render(rank, frames)
    merged = replicas.merge_framebuffers(hdr, frames)
    np.save(os.path.join(out_dir, f"merged{rank}.npy"), merged)
    np.save(os.path.join(out_dir, f"local{rank}.npy"), hdr)
    dist.destroy_process_group()


def test_two_rank_merge(tmp_path):
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    m0 = np.load(tmp_path / "merged0.npy")
    m1 = np.load(tmp_path / "merged1.npy")
    l0 = np.load(tmp_path / "local0.npy").astype(np.float64)
    l1 = np.load(tmp_path / "local1.npy").astype(np.float64)
    assert np.array_equal(m0, m1)
    exp = ((3 * l0 + 4 * l1) / 7).astype(np.float32)
    np.testing.assert_allclose(m0, exp, rtol=1e-6, atol=1e-7)
    assert not np.array_equal(l0, l1)  # disjoint sample streams


def test_replica_seeds_are_distinct():
    seeds = {replicas.replica_seed(0, r) for r in range(64)}
    assert len(seeds) == 64
