"""bench.py's replica path (--gpus N under torch.distributed.run): every rank
renders its own replica, the ranks meet at barriers and the throughput is all
ranks' units over the slowest rank's time.  Two gloo ranks on the CPU."""
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys, time
sys.path.insert(0, %r)
import bench
assert bench.WORLD == 2 and bench.RANK == int(os.environ["RANK"])
bench.init_dist()
bench.barrier()
secs = 0.5 if bench.RANK == 0 else 2.0          # rank 1 is the slow one
v = bench.aggregate(10, secs)
assert abs(v - 2 * 10 / 2.0) < 1e-9, v            # 20 units over the slowest 2 s
assert bench.allreduce_max(bench.RANK + 0.25) == 1.25
bench.barrier()
print("ok", bench.RANK, v)
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_replicas():
    port = str(_free_port())
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=port)
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD % ROOT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.STDOUT, text=True))
    outs = []
    for p in procs:
        try:
            out, _ = p.communicate(timeout=120)
        except subprocess.TimeoutExpired:
            p.kill()
            out, _ = p.communicate()
        outs.append(out)
        assert p.returncode == 0, out
    assert all("ok" in o for o in outs)
