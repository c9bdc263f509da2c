"""World-size-2 gloo test of the replica bookkeeping used by bench.py for N > 1."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from smaiso_wcomp_gb300 import replicas  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = replicas.rank_env()
    times = [1.0 + rank, 10.0 - rank]        # rank-dependent timings
    mx = replicas.max_over_ranks(times, dist)
    thr = replicas.job_throughput(100, mx[0], w)
    out.put((r, w, lr, mx, thr, replicas.replica_seed(1002, r)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, w, lr, mx, thr, seed) in enumerate(res):
        assert (rank, w, lr) == (r, 2, r)
        assert mx == [2.0, 10.0]              # max over ranks, element-wise
        assert thr == pytest.approx(2 * 100 / 2.0)
        assert seed == 1002


def test_single_process_identity():
    assert replicas.max_over_ranks([3.0, 4.0]) == [3.0, 4.0]
    assert replicas.job_throughput(10, 2.0, 1) == 5.0
