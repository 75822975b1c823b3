"""World-size-2 checks of the multi-GPU bookkeeping on CPU (gloo): batch
sharding covers every slice exactly once, per-rank CPU-oracle projections of
the shards gathered back equal the single-process result, and the timing
reduction takes the max over ranks."""

import os

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from ctlib_gb300.distributed import shard_range


def test_shard_range_partition():
    for n in (0, 1, 5, 16, 19):
        for world in (1, 2, 3, 4, 8):
            got = [shard_range(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(got[i][1] == got[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def _worker(rank, world, port, result_dir):
    import math
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from ctlib_gb300.distributed import gather_shards, max_over_ranks, shard
    from ctlib_gb300.workloads import para_options
    opts = para_options(20, 30, 16, 16, 1.0, 1.1, 0.0, math.pi / 20, 0.0)
    rng = np.random.default_rng(0)
    x = torch.from_numpy(rng.random((5, 1, 16, 16)))
    mine = shard(x, rank, world)
    y = torch.from_numpy(oracle.run("projection", mine.numpy(), opts, oracle.MODE_F64)) if mine.shape[0] \
        else torch.zeros((0, 1, 20, 30), dtype=torch.float64)
    full = gather_shards(y, 5)
    t = max_over_ranks(1.0 + rank)
    if rank == 0:
        np.save(os.path.join(result_dir, "full.npy"), full.numpy())
        with open(os.path.join(result_dir, "t.txt"), "w") as f:
            f.write(str(t))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_shard_and_gather(tmp_path, oracle_mod):
    import math
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_worker, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    from ctlib_gb300.workloads import para_options
    opts = para_options(20, 30, 16, 16, 1.0, 1.1, 0.0, math.pi / 20, 0.0)
    x = np.random.default_rng(0).random((5, 1, 16, 16))
    want = oracle_mod.run("projection", x, opts, oracle_mod.MODE_F64)
    got = np.load(tmp_path / "full.npy")
    assert np.array_equal(got, want)
    assert float((tmp_path / "t.txt").read_text()) == 2.0
