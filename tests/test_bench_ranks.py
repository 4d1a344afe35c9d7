"""bench.py's multi-replica host logic on CPU: two gloo ranks on 127.0.0.1
agree on the slowest rank's time, and the aggregate counts every rank's work."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(dist, 10.0 + 5.0 * rank)
        dist.barrier()
        q.put((rank, ms))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 15.0, 1: 15.0}


def test_both_arms_name_the_same_workload(capsys):
    """`bench.py --impl reference` prints the workload string of the GPU arm
    (the driver pairs the two lines by it); the CPU path is described beside."""
    import json
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.arm_workload("c2").startswith("view-heavy fused op: x[64,128,56,56]")
    assert "split-BF16" not in bench.arm_workload("c3")
    sys_argv = sys.argv
    try:
        sys.argv = ["bench.py", "--workload", "c3s", "--impl", "reference", "--steps", "1", "--warmup", "3"]
        bench.main()
    finally:
        sys.argv = sys_argv
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["config"]["workload"] == bench.arm_workload("c3s")
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
