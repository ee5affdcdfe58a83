"""The multi-GPU launch path's host logic on CPU (gloo, world size 2).

bench.py runs one replica of the workload per rank (weak scaling, no
collective on the data path); the process group carries only the timing
barrier and the max over ranks. Here two CPU processes take that path with
gloo: the barrier, the max-reduction of the step time, and the reference
arm's rule (rank 0 alone works and prints, the others exit 0 silently).
"""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        impl = "ours"

    w, r, _ = bench.dist_init(Args(), backend="gloo")
    bench.barrier(w)
    # each rank's own step time; the job's time is the slowest rank's
    t = bench.max_over_ranks(w, 10.0 + 5.0 * r)
    import torch.distributed as dist
    dist.destroy_process_group()
    out.put((r, w, t))


def test_barrier_and_max_over_ranks():
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
    assert res == [(0, 2, 15.0), (1, 2, 15.0)]


def test_reference_arm_other_ranks_exit_silently():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
               MASTER_PORT=str(_free_port()))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""
