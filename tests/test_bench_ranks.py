"""The replica arithmetic of bench.py on CPU: two gloo ranks (one process
each, rendezvous on 127.0.0.1) agree on the slowest rank's step time, and the
whole-job value spreads it over the states of every replica (weak scaling, no
collective on the data path)."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

CHILD = r"""
import json, os
import torch.distributed as dist
import bench
rank, ws = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"])
dist.init_process_group("gloo", rank=rank, world_size=ws)
ms = bench.max_over_ranks(100.0 + 50.0 * rank, ws, "cpu")
print(json.dumps({"rank": rank, "ms": ms, "value": bench.per_state(ms, 4, ws)}), flush=True)
dist.destroy_process_group()
"""


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_replicas_report_the_slowest_rank():
    pytest.importorskip("torch")
    ws, port = 2, _free_port()
    procs = []
    for r in range(ws):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(r), WORLD_SIZE=str(ws),
                   PYTHONPATH=str(ROOT) + os.pathsep + os.environ.get("PYTHONPATH", ""))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD], cwd=str(ROOT), env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=300)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert sorted(o["ms"] for o in outs) == [150.0, 150.0]
    for o in outs:
        assert o["value"] == pytest.approx(150.0 / 1e3 / (4 * ws))


def test_one_rank_is_the_identity():
    import bench
    assert bench.max_over_ranks(12.5, 1, "cpu") == 12.5
    assert bench.per_state(6000.0, 4, 1) == pytest.approx(1.5)
