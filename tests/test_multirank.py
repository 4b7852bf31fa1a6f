"""The bench's multi-rank path on the host: replicas time their steps, the job
takes the slowest rank's time and counts every rank's cell updates
(weak scaling, no collective on the data path).  Two gloo ranks on CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, results):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        elapsed = [12.5, 20.0][rank]  # the second replica is the slower one
        dist.barrier()
        slowest = bench.reduce_max(elapsed, dist)
        results[rank] = (slowest, bench.replica_mlups(1_000_000, 100, slowest, world))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_whole_job():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    results = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, results)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert results[0] == results[1]
    slowest, mlups = results[0]
    assert slowest == 20.0
    # 2 replicas x 1e6 cells x 100 steps in 20 ms
    assert mlups == pytest.approx(2 * 1e6 * 100 / 0.020 / 1e6)


def test_reference_arm_runs_on_rank_zero_only(capsys):
    """Under torchrun the reference arm's other ranks exit without work."""
    import argparse
    import bench
    args = argparse.Namespace(steps=1, warmup=3, gpus=2, impl="reference")
    bench.run_reference(args, rank=1, world=2)
    assert capsys.readouterr().out == ""
