"""Host-side logic of multi-GPU runs (replicas / sharded ensemble members),
exercised with two gloo ranks on CPU."""
import os
import socket

import pytest

from nextsimdg_gb300.replicas import shard


def test_shard_covers_members_once():
    for n in (1, 5, 32, 33):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in shard(n, r, world)]
            assert got == list(range(n))
            sizes = [len(shard(n, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    from nextsimdg_gb300 import replicas
    w, r, _ = replicas.init_from_env()
    members = list(replicas.shard(32, r, w))
    seconds = 1.0 + r  # rank 1 is the slowest
    thr = replicas.throughput(len(members) * 100.0, seconds, w)
    replicas.barrier(w)
    q.put((r, members[0], members[-1], thr))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][1:3] == (0, 15) and out[1][1:3] == (16, 31)
    # 32 members x 100 units over the slowest rank's 2 s
    assert out[0][3] == pytest.approx(1600.0) and out[1][3] == pytest.approx(1600.0)
