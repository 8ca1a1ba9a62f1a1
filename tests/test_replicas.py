"""Multi-rank host logic on CPU (gloo, world size 2): two replicas render consecutive frames of one view
with the oracle (each from its own sample offset, uneven frame counts) and merge their frame buffers. Under
both generators the merge must equal the sample-weighted mean of the two renders exactly, and one renderer
drawing all the frames up to float rounding; the replicas' samples must be disjoint."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from sparkle_gb300 import abi, replicas

FRAMES = (3, 4)  # uneven frames per replica


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _render(rng, frames, offset):
    import oracle
    from sparkle_gb300 import scenes
    scene, cam_args = scenes.cornell_box(0)
    cam = scenes.make_camera(cam_args, 16, 12)
    cfg = abi.make_config(16, 12, spp=1, bounce=4, rng=rng, seed=5, sample_offset=offset)
    r = oracle.OracleRenderer(oracle.OracleScene(scene), cfg, cam)
    r.render(frames)
    return r.framebuffer()[0]


def _worker(rank, world, port, out_dir, rng):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    frames = FRAMES[rank]
    offset = sum(FRAMES[:rank])  # frames before this replica's (uneven counts: no common frames per replica)
    hdr = _render(rng, frames, offset)
    merged = replicas.merge_framebuffers(hdr, frames)
    np.save(os.path.join(out_dir, f"merged{rank}.npy"), merged)
    np.save(os.path.join(out_dir, f"local{rank}.npy"), hdr)
    dist.destroy_process_group()


@pytest.mark.parametrize("rng", [abi.SPK_RNG_XOSHIRO128P, abi.SPK_RNG_XOSHIRO256SS])
def test_two_rank_merge_equals_one_renderer(tmp_path, rng):
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path), rng), nprocs=2, join=True, start_method="spawn")
    m0 = np.load(tmp_path / "merged0.npy")
    m1 = np.load(tmp_path / "merged1.npy")
    l0 = np.load(tmp_path / "local0.npy").astype(np.float64)
    l1 = np.load(tmp_path / "local1.npy").astype(np.float64)
    assert np.array_equal(m0, m1)
    exp = ((FRAMES[0] * l0 + FRAMES[1] * l1) / sum(FRAMES)).astype(np.float32)
    np.testing.assert_allclose(m0, exp, rtol=1e-6, atol=1e-7)
    assert not np.array_equal(l0, l1)  # disjoint samples
    single = _render(rng, sum(FRAMES), 0)  # one renderer drawing all 7 frames
    np.testing.assert_allclose(m0, single, rtol=2e-5, atol=1e-6)


def test_sample_offsets_tile_the_frames():
    offs = [replicas.replica_sample_offset(r, 64, 4) for r in range(8)]
    assert offs == [r * 256 for r in range(8)]
    assert replicas.replica_sample_offset(1, 10, base=100) == 110
