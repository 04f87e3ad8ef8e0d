"""The N>1 path of bench.py on CPU: ranks are independent replicas; the only
cross-rank step is the max-over-ranks of the timed region and a barrier
(gloo, world size 2)."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, lr = bench.dist_env()
    bench.barrier(w)
    t = bench.max_over_ranks(1.0 + rank, w)
    q.put((r, w, lr, t))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
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
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(o[3] == 2.0 for o in out)  # max over ranks


@pytest.mark.parametrize("world", [1])
def test_single_rank_is_identity(world):
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.5, world) == 3.5
