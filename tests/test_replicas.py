"""The multi-GPU path of bench.py is replicas only: independent chains, one
per rank, and the only communication is the max over ranks of the step
times.  Checked here with two gloo ranks on the CPU."""
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
    times = bench.replica_max([1.0 + rank, 10.0 - rank], dist, "cpu")
    out.put((rank, times, bench.replica_rate(world, times[0] / 1000.0, 1.25)))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_max_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, times, rate in res:
        assert times == [2.0, 10.0], (rank, times)
        assert rate == pytest.approx(2 / 0.002 / 1.25)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun every rank but 0 exits 0 without work or output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
