"""The multi-GPU path of bench.py on CPU: two gloo ranks on 127.0.0.1.

bench.py --gpus N runs N independent replicas (the operator does not shard
here: no data-path collective).  Its cross-rank logic is the barrier, the
job time as the largest rank time (max_over_ranks) and the whole-job rate
over all replicas (job_rate).  The reference arm runs on rank 0 only.
Both ranks here are host processes; no GPU is touched.
"""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        dist.barrier()
        t = bench.max_over_ranks(dist, 1.0 + 0.5 * r, "cpu")
        rate = bench.job_rate(2 * 1000 * 1000, 4, w, t)
        # the reference arm: ranks other than 0 return at once without work
        ref = bench.run_reference(None, r, w) if r != 0 else None
        q.put((r, w, local, t, rate, ref))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_time_and_job_rate():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 and o[2] == o[0] for o in out)
    for r, w, local, t, rate, ref in out:
        assert t == 1.5  # the slower rank's time
        assert rate == pytest.approx(2 * 1000 * 1000 * 4 * 2 / 1.5 / 1e9)
    assert out[1][5] == 0
