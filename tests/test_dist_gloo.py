"""Multi-process (world size 2, gloo on 127.0.0.1) coverage of what
bench.py --gpus N does across ranks: split the batch's independent scenes
across ranks (scenes.shard_batch, the arguments of each rank's batched
handle) without any exchange on the data path, then take the max of the
ranks' times.  Runs on CPU: each rank steps its shard with the oracle."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        from pbf_gb300 import scenes
        scs = scenes.batch_scenes(8, seed=2, iterations=2, nmin=200, nmax=1200, box_min=12,
                                  box_max=16)
        # the rank's batched-handle arguments, as bench.py's sharded leg builds them
        mine, params, counts, x4, v4 = scenes.shard_batch(scs, rank, world)
        sums = np.zeros(len(scs))
        off = 0
        for k, p, c in zip(mine, params, counts):
            o = oracle.Oracle(p, c, threads=1)
            o.set_state(x4[off:off + c], v4[off:off + c])
            off += c
            o.step(1)
            sums[k] = float(np.sum(o.get_state()[0][:, :3], dtype=np.float64))
        assert off == x4.shape[0]
        t = torch.tensor([float(rank + 1)])
        dist.all_reduce(t, op=dist.ReduceOp.MAX)  # the bench's max over ranks
        owned = torch.zeros(len(scs))
        owned[mine] = 1.0
        dist.all_reduce(owned)  # every scene exactly once
        cs = torch.from_numpy(sums)
        dist.all_reduce(cs)
        if rank == 0:
            out.put((float(t.item()), owned.tolist(), cs.tolist()))
    finally:
        dist.destroy_process_group()


def test_scene_sharding_and_max_timing_over_two_gloo_ranks(product_lib, oracle_mod):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    tmax, owned, sums = q.get(timeout=10)
    assert tmax == 2.0
    assert owned == [1.0] * 8
    # the sharded result equals stepping every scene in one process
    from pbf_gb300 import scenes
    scs = scenes.batch_scenes(8, seed=2, iterations=2, nmin=200, nmax=1200, box_min=12, box_max=16)
    for k, s in enumerate(scs):
        o = oracle_mod.Oracle(s.params, s.n, threads=1)
        o.set_state(s.x4, s.v4)
        o.step(1)
        assert sums[k] == pytest.approx(float(np.sum(o.get_state()[0][:, :3], dtype=np.float64)),
                                        rel=0, abs=0)
