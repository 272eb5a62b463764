"""The oracle against the golden vectors produced by the compiled reference.

The FP32 oracle must reproduce every parameter (numerator and denominator) of
the reference bit for bit after every dumped iteration, for all four models,
and its test-set evaluation within 2e-6 relative (the reference compiles its
evaluation with -ffast-math).  The oracle's own ingest must reproduce the
reference's partition exactly.
"""
import tempfile
from pathlib import Path

import numpy as np
import pytest

from conftest import CASES, case_models, dumped_iters, load_case
from oracle import bindings


@pytest.mark.parametrize("name", CASES)
def test_oracle_f32_bit_exact(name, oracle_lib):
    case = load_case(name)
    for model in case_models(case):
        fit = bindings.OracleFit("f32", model, 0, case["train_query"], case["train_pidx"], case["train_click"],
                                 int(case["n_qd"]))
        done = 0
        for it in dumped_iters(case, model):
            fit.run(it - done)
            done = it
            num, den, _ = fit.flat()
            ref = case[f"m{model}_params_{it:04d}"]
            assert np.array_equal(num.astype(np.float32), ref[:, 0]), (name, model, it, "numerator")
            assert np.array_equal(den.astype(np.float32), ref[:, 1]), (name, model, it, "denominator")
        ev = fit.evaluate(case["test_pidx"], case["test_click"])
        if ev["n"]:
            assert ev["llh_sum"] == pytest.approx(float(case[f"m{model}_llh_sum"]), rel=2e-6)
            assert ev["llh"] == pytest.approx(float(case[f"m{model}_llh"]), rel=2e-6)
            assert ev["ppl"] == pytest.approx(float(case[f"m{model}_ppl"]), rel=2e-6)
            np.testing.assert_allclose(ev["log2_sums"], case[f"m{model}_log2_sums"], rtol=2e-6)


@pytest.mark.parametrize("name", CASES)
def test_oracle_ingest_matches_reference(name, oracle_lib):
    case = load_case(name)
    with tempfile.TemporaryDirectory() as tmp:
        log = Path(tmp) / "log.txt"
        log.write_bytes(case["log"].tobytes())
        part = bindings.parse(str(log), int(case["max_sessions"]), float(case["test_share"]))
    assert part["n_qd"] == int(case["n_qd"])
    for s in ("train", "test"):
        for k in ("query", "docs", "pidx", "click"):
            assert np.array_equal(part[s][k], case[f"{s}_{k}"]), (name, s, k)


@pytest.mark.parametrize("name", ["dbn_dbnclicks", "ubm_dbnclicks"])
def test_oracle_f64_close_to_f32(name, oracle_lib):
    """The FP64 run differs from the FP32 reference only by rounding."""
    case = load_case(name)
    model = case_models(case)[0]
    a = bindings.OracleFit("f32", model, 0, case["train_query"], case["train_pidx"], case["train_click"], int(case["n_qd"]))
    b = bindings.OracleFit("f64", model, 0, case["train_query"], case["train_pidx"], case["train_click"], int(case["n_qd"]))
    a.run(20)
    b.run(20)
    va, vb = a.flat()[2], b.flat()[2]
    np.testing.assert_allclose(va, vb, rtol=1e-3, atol=1e-5)


def test_oracle_threads_only_reorder(oracle_lib):
    """Several threads change only the order of FP32 additions."""
    case = load_case("dbn_dbnclicks")
    a = bindings.OracleFit("f32", 2, 0, case["train_query"], case["train_pidx"], case["train_click"], int(case["n_qd"]))
    b = bindings.OracleFit("f32", 2, 0, case["train_query"], case["train_pidx"], case["train_click"], int(case["n_qd"]))
    a.run(5, threads=1)
    b.run(5, threads=4)
    np.testing.assert_allclose(a.flat()[2], b.flat()[2], rtol=1e-4, atol=1e-6)


def test_oracle_clean_mode_differs_only_where_unwritten(oracle_lib):
    """PBM and CCM write every statistic slot, so clean mode equals parity mode."""
    case = load_case("pbm_pbmclicks")
    a = bindings.OracleFit("f64", 0, 0, case["train_query"], case["train_pidx"], case["train_click"], int(case["n_qd"]))
    b = bindings.OracleFit("f64", 0, 1, case["train_query"], case["train_pidx"], case["train_click"], int(case["n_qd"]))
    a.run(3)
    b.run(3)
    assert np.array_equal(a.flat()[2], b.flat()[2])
