"""The multi-GPU story is replicas only: bench.py's Dist gives a barrier and the max of the
timed region over ranks, with no collective on the data path.  World size 2 on gloo, CPU."""
import os
import socket
import subprocess
import sys

from conftest import ROOT

SCRIPT = r"""
import os, sys, json
sys.path.insert(0, os.environ["TDDA_ROOT"])
import bench
d = bench.Dist()
d.barrier()
v = d.max(10.0 + d.rank)
print(json.dumps({"rank": d.rank, "world": d.world, "max": v}))
d.close()
"""


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_rank_max_and_barrier():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), TDDA_ROOT=ROOT)
        procs.append(subprocess.Popen([sys.executable, "-c", SCRIPT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    import json
    res = sorted((json.loads(o[0].strip().splitlines()[-1]) for o in outs), key=lambda r: r["rank"])
    assert [r["rank"] for r in res] == [0, 1]
    assert all(r["world"] == 2 and r["max"] == 11.0 for r in res)
