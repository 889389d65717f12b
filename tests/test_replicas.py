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
from gls.replicas import max_over_ranks, partition_windows, rank_seed, whole_job_rate, world_rank
world, rank, local = world_rank()
dist.init_process_group("gloo", rank=rank, world_size=world)
t = max_over_ranks(0.5 + rank, "cpu")
work = [((k * 7919) % 97 + 1) * 1000 for k in range(40)]   # uneven windows
mine = partition_windows(work, world)[rank]
print(json.dumps({"world": world, "rank": rank, "local": local, "t": t, "seed": rank_seed(2024, rank),
                  "rate": whole_job_rate(1000.0, world, t), "windows": mine,
                  "load": sum(work[k] for k in mine)}))
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
    # the uneven windows split by predicted work: every window on exactly one
    # rank, loads within one window of each other
    w0, w1 = outs[0]["windows"], outs[1]["windows"]
    assert sorted(w0 + w1) == list(range(40)) and not set(w0) & set(w1)
    assert abs(outs[0]["load"] - outs[1]["load"]) <= 97 * 1000


def test_partition_windows_balances_predicted_work():
    sys.path[:0] = [str(REPO / "gate-level-simulator_gb300")]
    import numpy as np
    from gls.replicas import partition_windows
    rng = np.random.default_rng(0)
    work = rng.integers(1_000, 50_000, size=256).astype(float)
    for world in (1, 2, 4, 8):
        parts = partition_windows(work, world)
        assert sorted(k for p in parts for k in p) == list(range(256))
        loads = [work[p].sum() for p in parts]
        assert max(loads) - min(loads) <= work.max()        # the greedy bound
        assert max(loads) <= work.sum() / world + work.max()


def test_replicas_single_process():
    sys.path[:0] = [str(REPO / "gate-level-simulator_gb300")]
    from gls.replicas import max_over_ranks, whole_job_rate
    assert max_over_ranks(3.25) == 3.25                          # no process group: the value itself
    assert whole_job_rate(10.0, 1, 2.0) == 5.0
