"""The multi-rank bench path on CPU: two gloo ranks shard the work as
replicas (each traces its own seeded rays over the same scene with the CPU
oracle), exchange nothing on the data path, and reduce only the slowest
rank's time; the whole-job rate counts every rank's rays."""
import os
import socket

import numpy as np
import pytest

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from libyafaray_gb300 import scenes
        from oracle import orc
        verts, faces = scenes.random_triangles(512, seed=1)
        rays = bench.rank_rays(256, rank)
        hits = orc.OracleScene(verts, faces).trace(rays, mode=0, threads=1)[0]
        local_s = 0.01 * (rank + 1)
        slowest = bench.max_over_ranks(local_s, dist)
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), rays=rays, hits=hits, slowest=slowest,
                 rate=bench.whole_job_rate(len(rays), world, slowest))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_as_replicas(tmp_path):
    import torch.multiprocessing as mp
    pytest.importorskip("torch.distributed")
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    r0, r1 = (np.load(tmp_path / f"rank{k}.npz") for k in (0, 1))
    # distinct rays per rank, each answered on its own
    assert not np.array_equal(r0["rays"], r1["rays"])
    assert len(r0["hits"]) == len(r0["rays"]) and len(r1["hits"]) == len(r1["rays"])
    # one scalar exchange: both ranks see the slowest rank's time
    assert float(r0["slowest"]) == float(r1["slowest"]) == pytest.approx(0.02)
    # whole-job throughput over both ranks' rays at the slowest time
    assert float(r0["rate"]) == pytest.approx(2 * 256 / 0.02 / 1e6)


def test_single_rank_helpers_need_no_process_group():
    assert bench.max_over_ranks(1.5, None) == 1.5
    assert bench.whole_job_rate(1_000_000, 1, 0.5) == pytest.approx(2.0)
    a, b = bench.rank_rays(8, 0), bench.rank_rays(8, 1)
    assert a.shape == b.shape and not np.array_equal(a, b)
