"""The multi-GPU path is replicas (every rank its own window, no data-path
collective): its host logic on two gloo ranks on the CPU — the launcher's
environment, distinct stimulus seeds, the maximum time over ranks and the
whole-job rate."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent
CHILD = r"""
import json, sys
sys.path[:0] = [sys.argv[1], sys.argv[1] + "/gate-level-simulator_gb300"]
import torch.distributed as dist
from gls.replicas import max_over_ranks, rank_seed, whole_job_rate, world_rank
world, rank, local = world_rank()
dist.init_process_group("gloo", rank=rank, world_size=world)
t = max_over_ranks(0.5 + rank, "cpu")
print(json.dumps({"world": world, "rank": rank, "local": local, "t": t, "seed": rank_seed(2024, rank),
                  "rate": whole_job_rate(1000.0, world, t)}))
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replicas_on_two_gloo_ranks():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                   LOCAL_RANK=str(rank))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD, str(REPO)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, e = p.communicate(timeout=240)
        assert p.returncode == 0, e
        outs.append(json.loads(o.strip().splitlines()[-1]))
    outs.sort(key=lambda d: d["rank"])
    assert [d["world"] for d in outs] == [2, 2] and [d["local"] for d in outs] == [0, 1]
    assert [d["t"] for d in outs] == [1.5, 1.5]                 # the slowest rank's time on every rank
    assert outs[0]["seed"] != outs[1]["seed"]                   # every rank simulates its own window
    assert [d["rate"] for d in outs] == [2000.0 / 1.5] * 2      # both ranks' work over the slowest time


def test_replicas_single_process():
    sys.path[:0] = [str(REPO / "gate-level-simulator_gb300")]
    from gls.replicas import max_over_ranks, whole_job_rate
    assert max_over_ranks(3.25) == 3.25                          # no process group: the value itself
    assert whole_job_rate(10.0, 1, 2.0) == 5.0
