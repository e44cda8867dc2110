"""bench.py's multi-rank path on CPU (two gloo ranks on 127.0.0.1).

The path does not shard: under torchrun every rank runs a replica of the
step, and the reported time is the slowest rank's (max over ranks).  The
reference arm runs on rank 0 only; the other ranks exit at once without
output.
"""
import os
import socket
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

_RANK_CODE = """
import sys
sys.path.insert(0, {repo!r})
import torch.distributed as dist
dist.init_process_group("gloo")
import bench
print(bench.max_over_ranks(1.5 + dist.get_rank(), dist, "cpu"))
print(bench.max_over_ranks(7.0, None, "cpu"))
dist.destroy_process_group()
"""


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_with_two_gloo_ranks():
    port = _free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", _RANK_CODE.format(repo=REPO)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=180)
        assert p.returncode == 0, err
        outs.append(out.split())
    # both ranks see the slowest rank's value; no process group: the value itself
    assert outs == [["2.5", "7.0"], ["2.5", "7.0"]]


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference"], cwd=REPO, env=env,
                       capture_output=True, text=True, timeout=180)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
