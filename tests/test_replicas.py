"""bench.py's multi-GPU mode runs independent replicas (weak scaling, no data-path collective): each
rank times its own replica, the ranks meet at barriers around the timed region and the reported
time is the maximum over the ranks. Checked here with two gloo ranks on the CPU."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist

    import bench

    r, w, local = bench._dist()
    dist.init_process_group("gloo", rank=r, world_size=w)
    bench._barrier(w)
    worst = bench._allreduce_max(1.0 + r, w)  # rank r "took" 1 + r seconds
    dof_stage = 1000.0
    value = w * dof_stage / worst  # whole-job rate from the slowest replica
    bench._barrier(w)
    dist.destroy_process_group()
    out.put((r, local, worst, value))


def test_two_gloo_replicas_report_the_slowest_rank():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _, _ in results] == [0, 1]
    assert all(worst == 2.0 for _, _, worst, _ in results)
    assert all(value == pytest.approx(1000.0) for _, _, _, value in results)
