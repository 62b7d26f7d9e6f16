"""The N>1 path of bench.py on the CPU: two ranks over gloo (127.0.0.1).
The path shards by frame (replicas): each rank develops frames of its own
seeds, nothing but a barrier and the max of the timings crosses ranks, and
the whole-job rate is all ranks' frames over the slowest rank's time. The
reference arm runs on rank 0 alone."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank: int, ws: int, port: int, out):
    os.environ.update(WORLD_SIZE=str(ws), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    import torch.distributed as dist
    r, w, local = bench.dist_init("gloo")
    seeds = [bench.replica_seed(2002, r, i) for i in range(4)]
    bench.barrier(w)
    # Rank 1 is the slow one: the job is as fast as it.
    rate = bench.whole_job_rate(10, w, 1.0 + r)
    out.put((r, w, local, seeds, rate, dist.get_backend()))
    bench.barrier(w)
    dist.destroy_process_group()


def test_two_rank_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, l0, s0, rate0, be0), (r1, w1, l1, s1, rate1, be1) = res
    assert (r0, r1) == (0, 1) and w0 == w1 == 2 and be0 == be1 == "gloo"
    # Replicas develop different frames.
    assert not set(s0) & set(s1)
    # 2 ranks x 10 frames over the slowest rank's 2 s, the same on both ranks.
    assert rate0 == rate1 == pytest.approx(10.0)


def test_reference_arm_rank_nonzero_exits_without_work():
    """Under torchrun the reference arm's other ranks exit 0 at once."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
