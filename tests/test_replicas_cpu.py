"""The multi-GPU form of the bench is independent replicas, one per rank:
its only communication is a barrier and a max-over-ranks of the timed
interval.  Checked here with two gloo ranks on the CPU (127.0.0.1)."""
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


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    ws, r, local = bench.dist_env()
    dist = bench.init_pg(ws)
    bench.barrier(dist)
    t = bench.allmax(dist, 1.0 + r)          # each rank's own "timed interval"
    v = bench.replica_throughput(ws, 1000, 10, t)
    q.put((r, local, ws, t, v))
    dist.destroy_process_group()


def test_two_gloo_ranks_time_by_the_slowest_rank():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the max (2.0 s) and the whole-job rate of both replicas
    assert [o[:3] for o in out] == [(0, 0, 2), (1, 1, 2)]
    assert all(o[3] == 2.0 for o in out)
    assert all(o[4] == 2 * 1000 * 10 / 2.0 for o in out)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the reference arm's other ranks exit 0 without output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""
