"""The mclicks command-line tool and the C++ host API behind it
(include/mclicks_host.hpp), against the reference's own output on the same
log: the result lines and the parameter CSV files (communicator.cpp:423-516)."""
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from conftest import load_case
from massiveclicks_gb300 import build
from oracle import bindings

pytestmark = pytest.mark.gpu


def _csv_rows(text: str):
    """(header or None, rows).  The reference's private-parameter files have no
    header: its data write at offset 0 overwrites the header line."""
    lines = text.strip().splitlines()
    head = lines[0] if not lines[0][:1].isdigit() and not lines[0].startswith("-") else None
    body = lines[1:] if head is not None else lines
    return head, [tuple(x.strip() for x in l.split(",")) for l in body]


@pytest.mark.parametrize("name,model", [("dbn_dbnclicks", 2), ("pbm_pbmclicks", 0), ("ccm_ccmclicks", 1),
                                        ("ubm_dbnclicks", 3)])
def test_cli_matches_reference_output(name, model):
    build.build_library()
    case = load_case(name)
    iters = int(case["iterations"])
    with tempfile.TemporaryDirectory() as tmp:
        tmp = Path(tmp)
        log = tmp / "log.txt"
        log.write_bytes(case["log"].tobytes())
        res = subprocess.run([str(build.CLI), "--raw-path", str(log), "--max-sessions", str(int(case["max_sessions"])),
                              "--itr", str(iters), "--model-type", str(model), "--test-share", "0.2",
                              "--output", str(tmp / "out")], capture_output=True, text=True, timeout=300)
        assert res.returncode == 0, res.stderr
        out = res.stdout
        ll = float([l for l in out.splitlines() if l.startswith("Total Log likelihood is: ")][0].split(": ")[1])
        ppl = float([l for l in out.splitlines() if l.startswith("Perplexity is: ")][0].split(": ")[1])
        assert "Average time per iteration: " in out
        f = bindings.OracleFit("f64", model, 0, case["train_query"], case["train_pidx"], case["train_click"],
                               int(case["n_qd"]))
        f.run(iters)
        ev = f.evaluate(case["test_pidx"], case["test_click"])
        assert ll == pytest.approx(ev["llh"], rel=1e-5)
        assert ll == pytest.approx(float(case[f"m{model}_llh"]), rel=1e-4)      # the FP32 reference
        assert ppl == pytest.approx(float(case[f"m{model}_ppl"]), rel=1e-4)
        for key in case:
            if not key.startswith(f"m{model}_csv_"):
                continue
            pname = key[len(f"m{model}_csv_"):]
            ref_head, ref_rows = _csv_rows(case[key].tobytes().decode())
            got_head, got_rows = _csv_rows((tmp / f"out_{pname}.csv").read_text())
            assert got_head == ref_head
            assert len(got_rows) == len(ref_rows)
            if len(ref_rows[0]) == 3:  # query, document, value
                assert [r[:2] for r in got_rows] == [r[:2] for r in ref_rows]
                vg = np.array([float(r[2]) for r in got_rows])
                vr = np.array([float(r[2]) for r in ref_rows])
            else:                      # rank, value
                assert [r[0] for r in got_rows] == [r[0] for r in ref_rows]
                vg = np.array([float(r[1]) for r in got_rows])
                vr = np.array([float(r[1]) for r in ref_rows])
            np.testing.assert_allclose(vg, vr, rtol=1e-4, atol=2e-6)


def test_cli_help_and_bad_flag():
    build.build_library()
    res = subprocess.run([str(build.CLI), "--help"], capture_output=True, text=True, timeout=60)
    assert res.returncode == 0 and "--model-type" in res.stdout
    res = subprocess.run([str(build.CLI), "--no-such-flag", "1"], capture_output=True, text=True, timeout=60)
    assert "Did not recognize flag" in res.stderr


def test_cli_missing_file_fails():
    build.build_library()
    res = subprocess.run([str(build.CLI), "--raw-path", "/nonexistent/log.txt"], capture_output=True, text=True,
                         timeout=60)
    assert res.returncode != 0 and "Unable to open the raw dataset" in res.stderr
