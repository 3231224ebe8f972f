"""The N > 1 rank logic of bench.py on the CPU: two gloo processes, each on
its own images (replicas, no data-path collective); timings reduce to the
slowest rank, votes to the whole job."""
import os
import socket
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, ws, port, q):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    imgs = bench.make_images(rank, 2)
    sig = [int(im.sum()) for im in imgs]
    out = bench.reduce_over_ranks([1.0 + rank, 10.0 - rank], 100.0 * (rank + 1), ws,
                                  torch.device("cpu"))
    q.put((rank, sig, out))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_shard_images_and_reduce():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, sig0, out0), (r1, sig1, out1) = res
    assert sig0 != sig1                       # each rank votes its own images
    assert out0 == out1 == (2.0, 10.0, 300.0)  # max of timings, sum of votes
