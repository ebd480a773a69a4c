"""Multi-GPU runs are replicas (no data exchange): every rank runs its own
workload and bench.py only coordinates the ranks on the host over gloo --
a barrier around the timed region, the maximum of the ranks' times and the
sum of their cell counts.  This runs that coordination with two CPU
processes (world size 2, rendezvous on 127.0.0.1), no GPU."""
import json
import os
import socket
import subprocess
import sys

from conftest import ROOT

CHILD = r"""
import json, os, sys, time
sys.path.insert(0, os.environ["ROOT"])
import bench
ws, rank, local = bench.dist_env()
g = bench.Group(ws)
t = 10.0 + rank          # this rank's time
cells = 1000.0 * (rank + 1)
g.barrier()
out = {"rank": rank, "ws": ws, "max": g.reduce(t, "max"), "sum": g.reduce(cells, "sum")}
g.barrier()
g.close()
print(json.dumps(out))
"""


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_rank_replica_coordination():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, ROOT=ROOT, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=120)
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    for o in outs:
        assert o["ws"] == 2
        assert o["max"] == 11.0  # the slower rank's time
        assert o["sum"] == 3000.0  # all ranks' cells


def test_single_process_needs_no_rendezvous():
    env = dict(os.environ, ROOT=ROOT)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    r = subprocess.run([sys.executable, "-c", CHILD], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    o = json.loads(r.stdout.strip().splitlines()[-1])
    assert o["ws"] == 1 and o["max"] == 10.0 and o["sum"] == 1000.0
