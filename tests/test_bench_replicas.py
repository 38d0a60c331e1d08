"""The multi-GPU path of bench.py is replicas only (one independent simulation per rank, no
collective on the data path).  Its host logic -- the max over ranks of the timed region and the
whole-job value -- runs here on two gloo ranks on the CPU; the reference arm prints only on
rank 0."""
import io
import os
import socket
from contextlib import redirect_stdout

import pytest
import torch.multiprocessing as tmp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [12.5, 17.25][rank]                     # rank 1 is the slower replica
    dist.barrier()
    slowest = bench.max_over_ranks(ms, dist, "cpu")
    q.put((rank, slowest, bench.whole_job_mcells(1.0e6, 100, slowest, world)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_value_on_two_gloo_ranks():
    ctx = tmp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    tmp.start_processes(_rank_main, args=(2, port, q), nprocs=2, join=True, start_method="spawn")
    got = sorted(q.get() for _ in range(2))
    for rank, slowest, value in got:
        assert slowest == 17.25                      # every rank sees the slowest rank's time
        assert value == pytest.approx(2 * 1.0e6 * 100 / 17.25e-3 / 1e6)


def test_single_rank_values():
    import bench
    assert bench.max_over_ranks(3.0) == 3.0
    assert bench.whole_job_mcells(2.0e6, 10, 4.0, 1) == pytest.approx(2.0e6 * 10 / 4.0e-3 / 1e6)


def test_reference_arm_prints_on_rank_zero_only():
    import bench
    buf = io.StringIO()
    with redirect_stdout(buf):
        assert bench.run_reference(None, None, "", 1) is None
    assert buf.getvalue() == ""
