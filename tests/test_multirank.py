"""The replica harness of bench.py on 2 CPU ranks (gloo): barrier, max-over-ranks timing, rank-0-only output.

The simulation step does not shard (a single fire would need halo exchanges every stencil and every
multigrid colour sweep), so `bench.py --gpus N` runs N independent replicas; these host-side pieces are
what multi-GPU runs add, and they are exercised here without a GPU.
"""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

WORKER = r"""
import os, sys, time, json
sys.path.insert(0, sys.argv[1])
import bench
rank, world = bench.dist_init("gloo")
assert (rank, world) == (int(os.environ["RANK"]), 2)
t = 0.01 * (rank + 1)                         # rank 1 is the slow one
time.sleep(t)
bench.barrier()
m = bench.max_over_ranks(t)
print(json.dumps({"rank": rank, "max": m}), flush=True)
bench.barrier()
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_rank_barrier_and_max(tmp_path):
    pytest.importorskip("torch.distributed")
    port = _free_port()
    script = tmp_path / "w.py"
    script.write_text(WORKER)
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(script), str(ROOT)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    res = [json.loads(o.strip().splitlines()[-1]) for o, _ in outs]
    assert {r["rank"] for r in res} == {0, 1}
    for r in res:
        assert r["max"] == pytest.approx(0.02)


def test_reference_arm_other_ranks_exit_quietly():
    """Under torchrun, ranks other than 0 do no work in the reference arm and print nothing."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
