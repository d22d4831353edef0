"""The multi-GPU path runs replicas (the path does not shard): the host logic
is checked here with world_size-2 gloo process groups on the CPU.

- job_rate: every rank gets the whole-job rate over the slowest replica's
  time and the same slowest time.
- bench.py --impl reference under a launcher: ranks other than 0 exit 0
  without work."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, seconds, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    from cubedsphere_sbp_swm_gb300 import replicas
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        assert replicas.world() == (world, rank)
        rate, slow = replicas.job_rate(10.0, seconds[rank])
        out.put((rank, rate, slow))
    finally:
        dist.destroy_process_group()


def test_job_rate_uses_the_slowest_replica():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    seconds = [1.0, 2.5]
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, seconds, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(out.get(timeout=5) for _ in range(2))
    for rank, rate, slow in res:
        assert slow == 2.5
        assert rate == pytest.approx(2 * 10.0 / 2.5)


def test_job_rate_single_process():
    sys.path.insert(0, ROOT)
    from cubedsphere_sbp_swm_gb300 import replicas
    assert replicas.world() == (1, 0)
    assert replicas.job_rate(50, 2.0) == (25.0, 2.0)
    with pytest.raises(ValueError):
        replicas.job_rate(1, 0.0)


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(_free_port()))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
