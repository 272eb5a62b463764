"""The host thread pool (massiveclicks_gb300/csrc/host/pool.cpp) under many
jobs of random sizes, most smaller than the number of workers: every index of
every job runs exactly once, and no worker runs a job that has returned
(tests/host_api/pool_stress.cpp, compiled with g++ against the pool's
sources)."""
import re
import subprocess
import tempfile
from pathlib import Path

from conftest import ROOT

SRC = ROOT / "tests" / "host_api" / "pool_stress.cpp"
HOST = ROOT / "massiveclicks_gb300" / "csrc" / "host"


def test_pool_runs_every_index_once():
    with tempfile.TemporaryDirectory() as tmp:
        exe = Path(tmp) / "pool_stress"
        cmd = ["g++", "-std=c++17", "-O2", "-pthread", "-Wall", "-Werror", f"-I{HOST}", str(SRC),
               str(HOST / "pool.cpp"), "-o", str(exe)]
        res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert res.returncode == 0, res.stdout
        res = subprocess.run([str(exe), "20000"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                             timeout=300)
        assert res.returncode == 0, res.stdout
        m = re.search(r"JOBS (\d+) BAD (\d+)", res.stdout)
        assert m and m.group(1) == "20000" and m.group(2) == "0", res.stdout
