"""Multi-process bookkeeping of the replica benchmark on CPU (gloo, 2 ranks)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from code_tohoku_gb300 import replicas
    replicas.init("gloo")
    # rank r processed 100 units in 1 + r seconds
    v = replicas.job_throughput(100.0, 1.0 + rank)
    m = replicas.max_over_ranks(3.0 * (rank + 1))
    replicas.barrier()
    q.put((rank, v, m))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_throughput_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, v, m in out:
        assert v == pytest.approx(200.0 / 2.0)   # all units over the slowest rank
        assert m == 6.0


def test_single_process_is_identity():
    from code_tohoku_gb300 import replicas
    assert replicas.job_throughput(50.0, 2.0) == 25.0
