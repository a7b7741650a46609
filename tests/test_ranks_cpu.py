"""The multi-GPU host logic (tramonto_gb300/ranks.py) with two gloo ranks on the CPU: problems dealt out to the
ranks cover the sweep exactly once, and the whole-job throughput is the sum of the ranks' units over the
slowest rank's time."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from tramonto_gb300 import ranks
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    w, r, lr = ranks.env()
    mine = ranks.shard(range(64), r, w)
    gathered = [None] * w
    dist.all_gather_object(gathered, mine)
    units = 10.0 * (r + 1)            # rank r processed 10 (r + 1) units
    ms = 100.0 * (r + 1)              # in 100 (r + 1) ms
    total, ms_max, rate = ranks.whole_job_rate(units, ms)
    out.put((r, w, lr, gathered, total, ms_max, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_aggregate():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, w, lr, gathered, total, ms_max, rate in res:
        assert w == 2 and lr == r
        flat = sorted(i for part in gathered for i in part)
        assert flat == list(range(64))                       # every problem exactly once
        assert total == 30.0 and ms_max == 200.0              # 10 + 20 units, slowest rank 200 ms
        assert abs(rate - 150.0) < 1e-12                      # 30 units / 0.2 s
