"""The multi-process (replica) path of bench.py on CPU, world size 2 over gloo:
the max-over-ranks timing helper, and the reference arm under torchrun (rank 0
alone runs and prints; the other rank exits 0 without work).

Run as a script (under torch.distributed.run) this file is the rank worker of
the first test."""
import json
import os
import re
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=600):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
    env = dict(os.environ, OMP_NUM_THREADS="1")
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)


def _worker():
    sys.path.insert(0, str(ROOT))
    import bench
    rank, world, _ = bench.dist_env()
    d = bench.Dist(world, "gloo")
    d.barrier()
    got = d.max(1.5 + rank)           # ranks time 1.5 and 2.5: the job takes 2.5
    d.barrier()
    print("RANK_RESULT " + json.dumps({"rank": rank, "world": world, "max": got}), flush=True)
    d.close()


def test_max_over_ranks_gloo():
    res = _torchrun([str(Path(__file__).resolve())], timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    # the ranks write concurrently, so their lines may run together
    lines = [json.loads(m) for m in re.findall(r"RANK_RESULT (\{[^}]*\})", res.stdout)]
    assert sorted(x["rank"] for x in lines) == [0, 1]
    assert all(x["world"] == 2 and x["max"] == 2.5 for x in lines)


def test_reference_arm_rank0_only():
    pytest.importorskip("torch")
    res = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
                     "--sessions", "100000", "--queries", "5000", "--cpu-sample", "20000"])
    assert res.returncode == 0, res.stdout + res.stderr
    lines = [json.loads(l) for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


if __name__ == "__main__":
    _worker()
