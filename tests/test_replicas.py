"""Multi-rank host logic on CPU (gloo, world size 2): the path shards partition a
batch, every rank renders its own shard with the oracle, and the job totals come
from reductions — the same code bench.py runs with NCCL on GPUs."""
import os
import socket

import numpy as np
import pytest

from footile_gb300 import replicas


def test_shard_partition():
    for n in (0, 1, 7, 64, 65536):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in replicas.shard(n, r, world)]
            assert got == list(range(n))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    from footile_gb300 import _abi, workloads
    ops, paths, nbytes = workloads.glyphs(64, seed=9)
    mine = paths[list(replicas.shard(len(paths), rank, world))]
    r = np.zeros(nbytes, np.uint8)
    st = oracle.fill_batch(0, _abi.NONZERO, ops, mine, _abi.MATTE8, r)
    px = int((mine["width"].astype(np.int64) * mine["height"]).sum())
    total_px = replicas.reduce_sum(px)
    slowest = replicas.reduce_max(float(rank + 1))
    replicas.barrier()
    out.put((rank, int(st.max()), px, total_px, slowest, int(r.sum())))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from footile_gb300 import workloads
    _, paths, _ = workloads.glyphs(64, seed=9)
    want_px = int((paths["width"].astype(np.int64) * paths["height"]).sum())
    assert res[0][2] + res[1][2] == want_px
    assert res[0][3] == res[1][3] == want_px
    assert res[0][4] == res[1][4] == 2.0
    assert all(r[1] == 0 and r[5] > 0 for r in res)
