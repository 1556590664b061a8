"""The multi-GPU path of bench.py is replicas only: every rank advances its
own copy of the lattice, the slowest rank's time counts and the value is the
whole job's.  Its host side (rendezvous, max over ranks, the aggregate, the
reference arm's rank-0-only rule) runs here as two gloo ranks on the CPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    ws, r, local, dist = bench.dist_setup("gloo")
    seconds = 0.5 + r  # the slower rank sets the job's time
    t = bench.max_over_ranks(dist, seconds)
    value = bench.aggregate_mlups(ws, 1_000_000, 10, t)
    with open(os.path.join(out, f"r{r}.json"), "w") as f:
        json.dump({"ws": ws, "rank": r, "max": t, "value": value}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_max_and_aggregate(tmp_path):
    ctx = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in range(2)]
    for d in res:
        assert d["ws"] == 2 and d["max"] == 1.5
        # two replicas of 1e6 nodes x 10 steps in 1.5 s
        assert abs(d["value"] - 2 * 1e6 * 10 / 1.5 / 1e6) < 1e-9


def test_reference_arm_other_ranks_exit_quietly(tmp_path):
    """Under torchrun only rank 0 of the reference arm works and prints; the
    other ranks leave at once with status 0 and print nothing.  Rank 0 here
    only joins the group and leaves, so rank 1's rendezvous completes."""
    port = _free_port()
    env = dict(os.environ, WORLD_SIZE="2", MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    r0 = subprocess.Popen([sys.executable, "-c",
                           "import os, sys; sys.path.insert(0, %r); os.environ.update(RANK='0', LOCAL_RANK='0');"
                           "import bench; ws, r, l, d = bench.dist_setup('gloo'); d.destroy_process_group()" % ROOT],
                          env=env)
    r1 = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                         "--warmup", "3"], env=dict(env, RANK="1", LOCAL_RANK="1"), capture_output=True, text=True,
                        timeout=120)
    r0.wait(120)
    assert r1.returncode == 0, r1.stderr
    assert r1.stdout.strip() == ""
    assert r0.returncode == 0
