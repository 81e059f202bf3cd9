"""Two-rank gloo run of the multi-GPU layout on CPU.

The frame path does not shard: N GPUs render N independent replicas and the
only collectives are a barrier and a max over ranks of the timed duration.
This runs that protocol with two CPU ranks, each rendering the frame with the
oracle, and checks that the replicas agree and the reduction is a max."""
import hashlib
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import oracle
    from tests.golden_scenes import heightfield_small
    dist.barrier()
    rgba, z, tpf, st = oracle.draw_scene(heightfield_small(), nthreads=1)
    elapsed = torch.tensor([float(rank + 1)], dtype=torch.float64)  # stand-in durations 1, 2
    dist.all_reduce(elapsed, op=dist.ReduceOp.MAX)
    h = hashlib.sha256(rgba.tobytes() + z.tobytes()).hexdigest()
    q.put((rank, st, tpf, h, float(elapsed.item())))
    dist.destroy_process_group()


def test_two_rank_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert all(r[1] == 0 for r in res)
    assert res[0][2:4] == res[1][2:4]           # identical replicas
    assert res[0][4] == res[1][4] == 2.0         # max over ranks
