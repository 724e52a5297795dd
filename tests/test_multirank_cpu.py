"""The N>1 host logic of bench.py on CPU: world_size-2 gloo ranks reduce their
step times to the slowest rank's, the whole-job value counts every rank's
work (independent replicas, no data-path collective), and under a launcher
only rank 0 of the reference arm does work."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.reduce_over_ranks([10.0 + 5 * rank, 3.0 - rank], world, "cpu")
    out[rank] = (ms, bench.job_value(1e8, world, ms[0]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_reduction_and_value():
    import torch.multiprocessing as mp

    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
    for r in (0, 1):
        ms, value = out[r]
        assert ms == [15.0, 3.0]  # each entry: the slowest rank's time
        assert value == pytest.approx(2 * 1e8 / 15e-3)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
