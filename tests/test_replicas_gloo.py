"""The multi-rank path of bench.py (replicas, one process per GPU) on CPU: two gloo
ranks rendezvous the way torchrun launches them, the timing reduction is a max over
ranks, and the reference arm runs on rank 0 only."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

CHILD = r"""
import json, os, sys
sys.path.insert(0, {root!r})
import bench
ws, rank, local, pg = bench.dist_setup()
bench.barrier(pg)
t = bench.max_over_ranks(pg, 1.0 + rank)
print(json.dumps({{"rank": rank, "ws": ws, "max": t}}), flush=True)
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _launch(code, nranks=2):
    port = _free_port()
    procs = []
    for r in range(nranks):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(nranks),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, cwd=str(ROOT),
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(out)
    return outs


def test_two_gloo_ranks_take_the_max_time():
    outs = _launch(CHILD.format(root=str(ROOT)))
    rows = [json.loads(o.strip().splitlines()[-1]) for o in outs]
    assert sorted(r["rank"] for r in rows) == [0, 1]
    assert all(r["ws"] == 2 and r["max"] == 2.0 for r in rows)


def test_reference_arm_prints_on_rank_zero_only():
    """Ranks other than 0 exit without work; rank 0 would run the oracle (skipped here by
    checking the early return with a tiny workload)."""
    code = (
        "import sys; sys.path.insert(0, %r); sys.argv = ['bench.py', '--impl', 'reference', "
        "'--side', '16', '--steps', '1', '--warmup', '1']; import bench; bench.main()"
        % str(ROOT))
    outs = _launch(code)
    lines = [[json.loads(x) for x in o.splitlines() if x.startswith("{")] for o in outs]
    assert sum(len(x) for x in lines) == 1
    line = [x for x in lines if x][0][0]
    assert line["impl"] == "reference" and line["value"] > 0
