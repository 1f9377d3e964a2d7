"""The replicas path of bench.py: one process per GPU and no collective on
the data path.  Its rank helpers run here over a world of two gloo ranks on
the CPU: the barrier, the slowest rank's time taken by every rank, and the
reference arm, which rank 0 alone runs."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import io, json, sys, contextlib
sys.path.insert(0, {root!r})
sys.argv = ["bench.py", "--impl", "reference", "--gpus", "2"]
import bench
rank, world, local, pg = bench.dist_init()
bench.barrier(pg)
slowest = bench.allreduce_max(pg, 1.5 + rank)
out = io.StringIO()
if rank != 0:
    # rank 1 of the reference arm exits without work or output
    with contextlib.redirect_stdout(out):
        bench.run_reference_arm(bench.parse(), rank, world, pg)
bench.barrier(pg)
print(json.dumps({{"rank": rank, "world": world, "local": local, "slowest": slowest, "printed": out.getvalue()}}))
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks():
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), WORLD_SIZE="2", LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            outs.append(p.communicate(timeout=180))
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e[-2000:]
    res = sorted((json.loads(o.strip().splitlines()[-1]) for o, _ in outs), key=lambda r: r["rank"])
    assert [r["rank"] for r in res] == [0, 1]
    assert all(r["world"] == 2 for r in res)
    assert [r["local"] for r in res] == [0, 1]
    # every rank reports the slowest rank's time
    assert all(r["slowest"] == 2.5 for r in res)
    assert res[1]["printed"] == ""
