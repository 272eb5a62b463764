"""The C++ host API (include/mclicks_host.hpp) as code written against the
reference's host classes uses it: two programs under tests/host_api are
compiled with g++ against the header and linked with libmclicks.so.

  * caller_main.cpp is shaped like the reference's driver (main.cpp:149-448)
    without MPI: ProcessingConfig filled field by field, ClusterProperties,
    LocalPartitions sized by the node's workers, the three-argument
    Dataset::parse_dataset, then em_parallel.
  * virtuals_check.cpp evaluates a test set through LogLikelihood and
    Perplexity, which reach a model subclass only through its virtuals
    (evaluation.cpp:25-66), with parameter values from the oracle.

The CPU tests parse and evaluate on the host; the GPU test runs em_parallel.
"""
import os
import re
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from conftest import CASES, ROOT, case_models, load_case
from massiveclicks_gb300 import build

SRC = ROOT / "tests" / "host_api"


def _compile(name: str, out_dir: Path) -> Path:
    build.build_library()
    exe = out_dir / name
    cuda = build._cuda_home()
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-ffp-contract=off", f"-I{ROOT / 'include'}",
           str(SRC / f"{name}.cpp"), "-o", str(exe), f"-L{build.BUILD}", "-lmclicks", f"-Wl,-rpath,{build.BUILD}",
           f"-L{cuda / 'lib64'}", "-lcudart", "-lpthread"]
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert res.returncode == 0, res.stdout
    return exe


@pytest.fixture(scope="module")
def programs():
    with tempfile.TemporaryDirectory() as tmp:
        d = Path(tmp)
        yield {"caller": _compile("caller_main", d), "virtuals": _compile("virtuals_check", d), "dir": d}


def _log(case, d: Path) -> Path:
    p = d / "log.txt"
    p.write_bytes(case["log"].tobytes())
    return p


@pytest.mark.parametrize("name", CASES)
def test_caller_parses_like_the_reference(programs, name):
    """The three-argument parse_dataset fills partition 0 with the reference's
    own partition sizes."""
    case = load_case(name)
    log = _log(case, programs["dir"])
    res = subprocess.run([str(programs["caller"]), "--raw-path", str(log), "--max-sessions",
                          str(int(case["max_sessions"])), "--test-share", str(float(case["test_share"])),
                          "--parse-only", "1"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert res.returncode == 0, res.stdout
    parts = re.findall(r"^PARTITION (\d+) (\d+) (\d+) (\d+)$", res.stdout, re.M)
    assert parts and parts[0] == ("0", str(len(case["train_query"])), str(len(case["test_query"])),
                                  str(int(case["n_qd"])))
    assert all(p[1:] == ("0", "0", "0") for p in parts[1:])


def test_caller_rejects_several_nodes(programs):
    case = load_case("edge")
    log = _log(case, programs["dir"])
    res = subprocess.run([str(programs["caller"]), "--raw-path", str(log), "--nodes", "2", "--parse-only", "1"],
                         stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert res.returncode == 1
    assert "one node" in res.stdout


@pytest.mark.parametrize("name", CASES)
def test_virtuals_match_oracle_evaluation(programs, name, oracle_lib):
    """LogLikelihood and Perplexity through the per-session virtuals, against
    the oracle's FP32 evaluation (the reference's expressions and summation
    order) on the same parameter values."""
    from oracle import bindings
    case = load_case(name)
    log = _log(case, programs["dir"])
    for model in case_models(case):
        f = bindings.OracleFit("f32", model, 0, case["train_query"], case["train_pidx"], case["train_click"],
                               int(case["n_qd"]))
        f.run(3)
        _, _, val = f.flat()
        pfile = programs["dir"] / "params.f32"
        val.astype(np.float32).tofile(pfile)
        res = subprocess.run([str(programs["virtuals"]), str(log), str(int(case["max_sessions"])),
                              str(float(case["test_share"])), str(model), str(pfile)],
                             stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        assert res.returncode == 0, res.stdout
        out = dict(re.findall(r"^(LLH|TASK|CALLS|SERP_DEV|FOOTPRINT|MEMORY) (\S+)$", res.stdout, re.M))
        l2 = np.array([float(v) for _, v in sorted(re.findall(r"^L2 (\d) (\S+)$", res.stdout, re.M),
                                                     key=lambda t: int(t[0]))])
        ref = f.evaluate(case["test_pidx"], case["test_click"])
        n = ref["n"]
        assert int(out["CALLS"]) == n
        assert float(out["TASK"]) == n
        assert float(out["LLH"]) == pytest.approx(ref["llh_sum"], rel=1e-6, abs=1e-6)
        np.testing.assert_allclose(l2, ref["log2_sums"], rtol=1e-6, atol=1e-6)
        assert float(out["SERP_DEV"]) <= 1e-6
        assert int(out["FOOTPRINT"]) > 0 and int(out["MEMORY"]) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("name,model", [("dbn_dbnclicks", 2), ("ubm_dbnclicks", 3)])
def test_caller_em_parallel(programs, name, model, oracle_lib):
    """The main.cpp-shaped caller runs em_parallel on the GPU; its printed test
    log-likelihood and perplexity agree with the FP64 oracle within 1e-5."""
    from oracle import bindings
    case = load_case(name)
    log = _log(case, programs["dir"])
    iters = 10
    res = subprocess.run([str(programs["caller"]), "--raw-path", str(log), "--max-sessions",
                          str(int(case["max_sessions"])), "--test-share", str(float(case["test_share"])),
                          "--itr", str(iters), "--model-type", str(model)],
                         stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert res.returncode == 0, res.stdout
    llh = float(re.search(r"Total Log likelihood is: (\S+)", res.stdout).group(1))
    ppl = float(re.search(r"^Perplexity is: (\S+)", res.stdout, re.M).group(1))
    f = bindings.OracleFit("f64", model, 0, case["train_query"], case["train_pidx"], case["train_click"],
                           int(case["n_qd"]))
    f.run(iters)
    ref = f.evaluate(case["test_pidx"], case["test_click"])
    assert llh == pytest.approx(ref["llh"], rel=1e-5)
    assert ppl == pytest.approx(ref["ppl"], rel=1e-5)
