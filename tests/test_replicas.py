"""Multi-GPU runs of the step are independent replicas (one process per GPU,
no collective on the data path).  The host logic of that path runs here as
two gloo ranks on the CPU: the timing reduction (the slowest rank's time),
and the reference arm, which only rank 0 runs."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(torch, 10.0 + 5.0 * rank, "cpu")
        dist.barrier()
        ref = bench.run_reference(type("A", (), {"steps": 1})())
        out.put((rank, ms, ref))
    finally:
        dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks_and_reference_runs_on_rank0_only():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(1, world)]
    for p in procs:
        p.start()
    # rank 0 (this process) takes part in the timing reduction only: its
    # run_reference would time the full-size CPU sample
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK="0", WORLD_SIZE=str(world))
    import bench
    dist.init_process_group("gloo", rank=0, world_size=world)
    try:
        ms0 = bench.max_over_ranks(torch, 10.0, "cpu")
        dist.barrier()
    finally:
        dist.destroy_process_group()
        for k in ("RANK", "WORLD_SIZE", "MASTER_PORT"):
            os.environ.pop(k, None)
    rank, ms1, ref1 = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert ms0 == ms1 == 15.0
    assert rank == 1 and ref1 is None
