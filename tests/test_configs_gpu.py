"""The two small benchmark configurations, run as stated, against the FP64
oracle (the reference's CPU training path restated in double precision):

  * 40,000 sessions, 1,000 queries Zipf(1.1), 20-doc pools, top-10 shown,
    ground-truth PBM clicks (attractiveness ~ Beta(1, 3), examination
    0.9 / sqrt(r + 1)); PBM fitted for 50 iterations, test share 0.2;
  * 2,000,000 sessions, 100,000 queries Zipf(1.0), 30-doc pools, ground-truth
    DBN clicks (attractiveness ~ Beta(1, 3), satisfaction ~ Beta(1, 4),
    continuation 0.9); UBM (examination starting at 1/2) and DBN fitted for
    50 iterations, test share 0.2; the plain FP32 GPU EM beside the fused one.

Bars (the fused product path): every parameter within 1e-5 relative (+1e-6
absolute, for values near the 1 - 1e-6 clamp) of the oracle, test
log-likelihood and perplexity within 1e-5 relative.  The plain all-FP32 GPU
EM is held to 1e-5 on test log-likelihood and perplexity only; its parameter
errors are reported.  One JSON line per fit is printed (prefix CONFIG) and
appended to the file MC_CONFIG_OUT names, if set."""
import json
import os
import time

import numpy as np
import pytest

from massiveclicks_gb300 import api
from massiveclicks_gb300._capi import IMPL_FUSED, IMPL_PLAIN, MODEL_NAMES
from oracle import bindings

pytestmark = pytest.mark.gpu

ITERATIONS = 50
PARAM_RTOL = 1e-5
PARAM_ATOL = 1e-6
EVAL_RTOL = 1e-5


def _dataset(preset: int):
    cfg = api.synth_config(preset)
    q, d, m = api.synth_sessions(cfg)
    return cfg, api.Dataset.from_sessions(q, d, m, 0.2)


@pytest.fixture(scope="module")
def config1():
    return _dataset(0)


@pytest.fixture(scope="module")
def config2():
    return _dataset(1)


def _param_errors(got: dict, ref: dict) -> dict:
    out = {}
    for k, r in ref.items():
        g = got[k].astype(np.float64)
        err = np.abs(g - r)
        excess = err - (PARAM_RTOL * np.abs(r) + PARAM_ATOL)
        out[k] = {"max_abs": float(err.max()), "max_rel": float((err / np.maximum(np.abs(r), 1e-30)).max()),
                  "within_bar": bool(np.all(excess <= 0))}
    return out


def _fit_and_compare(cfg, ds, model: int, impls) -> dict:
    f = bindings.OracleFit("f64", model, 0, ds.train.query, ds.train.pidx, ds.train.click, ds.n_qd)
    t0 = time.perf_counter()
    f.run(ITERATIONS, threads=os.cpu_count() or 1, copy_sessions=False)
    t_oracle = time.perf_counter() - t0
    ref = f.values()
    ref_ev = f.evaluate(ds.test.pidx, ds.test.click)
    line = {"model": MODEL_NAMES[model], "sessions": int(cfg.n_sessions), "queries": int(cfg.n_queries),
            "pool": int(cfg.pool), "zipf_s": float(cfg.zipf_s), "seed": int(cfg.seed),
            "train_sessions": len(ds.train), "test_sessions": len(ds.test), "n_qd": ds.n_qd,
            "iterations": ITERATIONS,
            "oracle": {"test_llh": ref_ev["llh"], "perplexity": ref_ev["ppl"], "seconds": round(t_oracle, 2),
                       "threads": os.cpu_count()}}
    for name, impl in impls:
        cm = api.ClickModel.create(model)
        cm.init_parameters(ds)
        cm.em(ITERATIONS, impl)
        ev = cm.evaluate(1)
        params = cm.get_parameters()
        cm.destroy_parameters()
        line[name] = {"params": _param_errors(params, ref), "test_llh": ev.llh,
                      "test_llh_rel_err": abs(ev.llh - ref_ev["llh"]) / abs(ref_ev["llh"]),
                      "perplexity": ev.perplexity,
                      "perplexity_rel_err": abs(ev.perplexity - ref_ev["ppl"]) / ref_ev["ppl"],
                      "test_sessions_evaluated": ev.n_sessions}
        assert ev.n_sessions == ref_ev["n"]
    print("CONFIG " + json.dumps(line))
    out = os.environ.get("MC_CONFIG_OUT")
    if out:
        with open(out, "a") as fh:
            fh.write(json.dumps(line) + "\n")
    return line


def _assert_bars(line: dict, name: str, params: bool):
    r = line[name]
    if params:
        for k, e in r["params"].items():
            assert e["within_bar"], f"{line['model']} {name} {k}: max abs {e['max_abs']:.3g}, rel {e['max_rel']:.3g}"
    assert r["test_llh_rel_err"] <= EVAL_RTOL, (line["model"], name, r["test_llh_rel_err"])
    assert r["perplexity_rel_err"] <= EVAL_RTOL, (line["model"], name, r["perplexity_rel_err"])


def test_config1_pbm(config1):
    cfg, ds = config1
    assert cfg.n_sessions == 40_000 and cfg.n_queries == 1_000 and cfg.pool == 20
    assert len(ds.train) == 32_000
    line = _fit_and_compare(cfg, ds, api.PBM, [("fused", IMPL_FUSED)])
    _assert_bars(line, "fused", params=True)


@pytest.mark.parametrize("model", [api.UBM, api.DBN])
def test_config2(config2, model):
    cfg, ds = config2
    assert cfg.n_sessions == 2_000_000 and cfg.n_queries == 100_000 and cfg.pool == 30
    assert len(ds.train) == 1_600_000
    line = _fit_and_compare(cfg, ds, model, [("fused", IMPL_FUSED), ("plain", IMPL_PLAIN)])
    _assert_bars(line, "fused", params=True)
    _assert_bars(line, "plain", params=False)
