"""Multi-process host logic of bench.py on CPU (gloo, world size 2): each process of a torchrun
launch reads its rank from the environment, the job's time is the maximum over ranks, and the
reference arm runs on rank 0 only. Genes are independent, so N GPUs run N replicas of the DE
call with no collective on the data path; only these host-side steps involve other ranks."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    r, w, l = bench.dist_env()
    dist.init_process_group("gloo", rank=r, world_size=w)
    dist.barrier()
    m = bench.max_over_ranks([1.0 + rank, 5.0 - rank], dist)
    dist.destroy_process_group()
    q.put((rank, (r, w, l), m))


def test_two_ranks_take_the_maximum_over_ranks():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, env, m in out:
        assert env == (rank, 2, rank)
        assert m == [2.0, 5.0]


def test_reference_arm_runs_on_rank_zero_only():
    sys.path.insert(0, ROOT)
    import bench

    class Args:  # rank 1 must return before building the workload or timing anything
        pass
    assert bench.run_reference(Args(), 1, 2) == 0
