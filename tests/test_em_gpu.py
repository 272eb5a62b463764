"""GPU EM against the FP64 oracle, through the C-ABI.

Tolerances (FP32 GPU arithmetic against an FP64 run of the reference's
expressions, after the stated number of iterations):
  * parameters:  |gpu - f64| <= PARAM_RTOL * |f64| + PARAM_ATOL
  * test-set log-likelihood and perplexity: relative LL_RTOL
The FP32 reference itself differs from its FP64 run by more than this on the
same inputs (see test_reference_f32_error_budget), so these bounds are tighter
than the reference's own rounding.
"""
import numpy as np
import pytest

from conftest import CASES, case_models, load_case
from massiveclicks_gb300 import api
from massiveclicks_gb300._capi import IMPL_FUSED, IMPL_PLAIN, MODE_CLEAN, MODE_PARITY
from oracle import bindings

pytestmark = pytest.mark.gpu

PARAM_RTOL = 1e-5
PARAM_ATOL = 1e-6
LL_RTOL = 1e-5


def sset(case, which):
    return api.SessionSet(case[f"{which}_query"], case[f"{which}_docs"], case[f"{which}_pidx"], case[f"{which}_click"])


def gpu_fit(case, model, iters, impl=IMPL_FUSED, mode=MODE_PARITY, config=None):
    cm = api.ClickModel.create(model, mode=mode)
    cm.upload(sset(case, "train"), int(case["n_qd"]))
    cm.upload_test(sset(case, "test"))
    if config:
        cm.configure(*config)
    cm.em(iters, impl)
    return cm


def oracle_fit(case, model, iters, mode=MODE_PARITY):
    f = bindings.OracleFit("f64", model, mode, case["train_query"], case["train_pidx"], case["train_click"],
                           int(case["n_qd"]))
    f.run(iters)
    return f


def assert_params_close(gpu: dict, ref: dict, rtol=PARAM_RTOL, atol=PARAM_ATOL, what=""):
    for name, v in ref.items():
        g = gpu[name].astype(np.float64)
        err = np.abs(g - v)
        bound = rtol * np.abs(v) + atol
        worst = int(np.argmax(err - bound)) if err.size else 0
        assert np.all(err <= bound), f"{what} {name}: worst index {worst} gpu {g[worst]!r} f64 {v[worst]!r}"


def assert_eval_close(cm, f, case, rtol=LL_RTOL):
    ev = cm.evaluate(1)
    ref = f.evaluate(case["test_pidx"], case["test_click"])
    if ref["n"] == 0:
        assert ev.n_sessions == 0
        return
    assert ev.n_sessions == ref["n"]
    assert ev.llh == pytest.approx(ref["llh_sum"] / ref["n"], rel=rtol)
    np.testing.assert_allclose(ev.log2_sums, ref["log2_sums"], rtol=rtol)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("impl", [IMPL_FUSED, IMPL_PLAIN])
def test_em_matches_f64_oracle(name, impl):
    case = load_case(name)
    iters = int(case["iterations"])
    for model in case_models(case):
        cm = gpu_fit(case, model, iters, impl)
        f = oracle_fit(case, model, iters)
        rtol = PARAM_RTOL if impl == IMPL_FUSED else 5 * PARAM_RTOL
        assert_params_close(cm.get_parameters(), f.values(), rtol=rtol, what=f"{name} m{model} impl{impl}")
        assert_eval_close(cm, f, case, rtol=LL_RTOL if impl == IMPL_FUSED else 10 * LL_RTOL)


@pytest.mark.parametrize("name", ["ubm_dbnclicks", "dbn_dbnclicks", "dbn_ccmclicks"])
def test_clean_mode_matches_f64_oracle(name):
    case = load_case(name)
    model = case_models(case)[0]
    cm = gpu_fit(case, model, 10, mode=MODE_CLEAN)
    f = oracle_fit(case, model, 10, mode=MODE_CLEAN)
    assert_params_close(cm.get_parameters(), f.values(), what=f"clean {name}")


@pytest.mark.parametrize("config", [(7, 16, 64), (32, 64, 128), (100, 5000, 64), (1024, 4096, 256), (4096, 1024, 256)])
def test_tiling_does_not_change_results(config):
    """Tiny tiles force queries split over many tiles and windows too wide for
    shared memory; results must not depend on the tile shape."""
    case = load_case("dbn_dbnclicks")
    a = gpu_fit(case, 2, 5, config=config).get_parameters()
    f = oracle_fit(case, 2, 5)
    assert_params_close(a, f.values(), what=f"config {config}")


@pytest.mark.parametrize("model", [0, 1, 2, 3])
def test_tiling_all_models(model):
    case = load_case({0: "pbm_pbmclicks", 1: "ccm_ccmclicks", 2: "dbn_ccmclicks", 3: "ubm_dbnclicks"}[model])
    f = oracle_fit(case, model, 4)
    for config in [(5, 12, 64), (64, 256, 96)]:
        g = gpu_fit(case, model, 4, config=config).get_parameters()
        assert_params_close(g, f.values(), what=f"m{model} config {config}")


def test_ubm_every_click_pattern():
    """All 1024 click patterns, including the two in which a later rank
    overwrites an earlier rank's examination slot."""
    rng = np.random.default_rng(7)
    n = 1024 * 4
    masks = np.tile(np.arange(1024, dtype=np.uint16), 4)
    query = np.sort(rng.integers(0, 64, n)).astype(np.int32)
    docs = np.stack([qq * 100 + rng.permutation(30)[:10] for qq in query]).astype(np.int32)
    ds = api.Dataset.from_sessions(query, docs, masks, 0.0)
    for model in (3, 0, 2, 1):
        cm = api.ClickModel.create(model)
        cm.upload(ds.train, ds.n_qd)
        cm.em(6)
        f = bindings.OracleFit("f64", model, 0, ds.train.query, ds.train.pidx, ds.train.click, ds.n_qd)
        f.run(6)
        assert_params_close(cm.get_parameters(), f.values(), what=f"patterns m{model}")


@pytest.mark.parametrize("model", [0, 1, 2, 3])
def test_medium_synthetic(model):
    """A few hundred thousand sessions in the benchmark's shape."""
    cfg = api.synth_config(2 if model in (1, 2) else 1, n_sessions=250000, n_queries=20000)
    q, d, m = api.synth_sessions(cfg)
    ds = api.Dataset.from_sessions(q, d, m, 0.2)
    cm = api.ClickModel.create(model)
    cm.init_parameters(ds)
    cm.em(10)
    f = bindings.OracleFit("f64", model, 0, ds.train.query, ds.train.pidx, ds.train.click, ds.n_qd)
    f.run(10)
    assert_params_close(cm.get_parameters(), f.values(), what=f"medium m{model}")
    ev = cm.evaluate(1)
    ref = f.evaluate(ds.test.pidx, ds.test.click)
    assert ev.llh == pytest.approx(ref["llh"], rel=LL_RTOL)
    assert ev.perplexity == pytest.approx(sum(2.0 ** (-ref["log2_sums"] / ref["n"])) / 10, rel=LL_RTOL)


def test_eval_matches_oracle_on_same_parameters():
    """Evaluation alone: the oracle is given the GPU's parameters."""
    for name in ("pbm_pbmclicks", "ubm_dbnclicks", "dbn_dbnclicks", "ccm_ccmclicks"):
        case = load_case(name)
        model = case_models(case)[0]
        cm = gpu_fit(case, model, 7)
        f = oracle_fit(case, model, 0)
        f.set_values({k: v.astype(np.float64) for k, v in cm.get_parameters().items()})
        assert_eval_close(cm, f, case, rtol=2e-6)
        # training-set evaluation too
        ev = cm.evaluate(0)
        ref = f.evaluate(case["train_pidx"], case["train_click"])
        assert ev.llh == pytest.approx(ref["llh_sum"] / ref["n"], rel=2e-6)


def test_fused_and_plain_agree():
    case = load_case("dbn_ccmclicks")
    a = gpu_fit(case, 2, 20, IMPL_FUSED)
    b = gpu_fit(case, 2, 20, IMPL_PLAIN)
    assert a.evaluate(1).llh == pytest.approx(b.evaluate(1).llh, rel=1e-5)


def test_graph_replay_and_split_calls_equal_one_call():
    case = load_case("ccm_ccmclicks")
    a = gpu_fit(case, 1, 6)
    b = gpu_fit(case, 1, 2)
    b.em(2)
    b.em(2)
    assert_params_close(b.get_parameters(), {k: v.astype(np.float64) for k, v in a.get_parameters().items()},
                        rtol=1e-6, atol=1e-7)


def test_process_and_update_equal_plain_iteration():
    case = load_case("pbm_pbmclicks")
    a = gpu_fit(case, 0, 3, IMPL_PLAIN)
    b = gpu_fit(case, 0, 0)
    for _ in range(3):
        b.process_session()
        b.update_parameters()
    assert_params_close(b.get_parameters(), {k: v.astype(np.float64) for k, v in a.get_parameters().items()},
                        rtol=1e-5, atol=1e-6)


def test_reset_to_prior_and_set_get_roundtrip():
    case = load_case("dbn_dbnclicks")
    cm = gpu_fit(case, 2, 3)
    p = cm.get_parameters()
    cm.reset_to_prior()
    assert all(np.all(v == 0.5) for v in cm.get_parameters().values())
    cm.set_parameters(p)
    q = cm.get_parameters()
    assert all(np.array_equal(p[k], q[k]) for k in p)


def test_empty_and_single_session():
    cm = api.ClickModel.create(2)
    cm.upload(api.SessionSet(np.zeros(0, np.int32), np.zeros((0, 10), np.int32), np.zeros((0, 10), np.int32),
                             np.zeros(0, np.uint16)), 0)
    cm.em(3)
    assert cm.evaluate(0).n_sessions == 0
    one = api.SessionSet(np.array([5], np.int32), np.arange(10, dtype=np.int32)[None],
                         np.arange(10, dtype=np.int32)[None], np.array([0b101], np.uint16))
    for model in range(4):
        cm = api.ClickModel.create(model)
        cm.upload(one, 10)
        cm.em(4)
        f = bindings.OracleFit("f64", model, 0, one.query, one.pidx, one.click, 10)
        f.run(4)
        assert_params_close(cm.get_parameters(), f.values(), what=f"single m{model}")


def test_configure_rejects_shapes_that_do_not_fit():
    case = load_case("dbn_dbnclicks")
    cm = gpu_fit(case, 2, 0)
    with pytest.raises(api._capi.MCError):
        cm.configure(4096, 16384, 256)
    with pytest.raises(api._capi.MCError):
        cm.configure(0, 0, 1024)


def test_bad_indices_rejected():
    bad = api.SessionSet(np.array([1], np.int32), np.zeros((1, 10), np.int32), np.full((1, 10), 11, np.int32),
                         np.zeros(1, np.uint16))
    cm = api.ClickModel.create(0)
    with pytest.raises(api._capi.MCError):
        cm.upload(bad, 10)


def test_autotune_keeps_parameters():
    case = load_case("dbn_ccmclicks")
    cm = gpu_fit(case, 2, 3)
    before = cm.get_parameters()
    cm.autotune()
    after = cm.get_parameters()
    assert all(np.array_equal(before[k], after[k]) for k in before)
    cm.em(2)
    f = oracle_fit(case, 2, 5)
    assert_params_close(cm.get_parameters(), f.values(), what="after autotune")


def test_reference_f32_error_budget():
    """How far the FP32 reference (golden vectors) sits from the FP64 oracle:
    the GPU must do at least as well."""
    case = load_case("dbn_dbnclicks")
    f = oracle_fit(case, 2, 20)
    ref = case["m2_params_0020"]
    ref_val = np.minimum(ref[:, 0] / ref[:, 1], np.float32(1.0 - 0.000001))
    f64 = np.concatenate(list(f.values().values()))
    ref_err = np.max(np.abs(ref_val - f64) / np.abs(f64))
    cm = gpu_fit(case, 2, 20)
    gpu_err = np.max(np.abs(cm.flat_parameters().astype(np.float64) - f64) / np.abs(f64))
    assert gpu_err <= max(ref_err, PARAM_RTOL)


def test_float_bins_when_fixed_point_lacks_bits():
    """Tiles accumulate in 32-bit fixed point when the tile's largest
    occurrence count leaves at least 20 fraction bits, else in FP32.  A query
    with 3,000 sessions over 12 documents in one 4,096-session tile (a
    document shown about 2,500 times) takes the FP32 bins; both kinds of tile
    must match the oracle."""
    rng = np.random.default_rng(5)
    n = 3000
    query = np.zeros(n, np.int32)
    docs = np.stack([rng.permutation(12)[:10] for _ in range(n)]).astype(np.int32)
    masks = rng.integers(0, 1024, n).astype(np.uint16)
    ds = api.Dataset.from_sessions(query, docs, masks, 0.0)
    for model in (2, 1):
        f = bindings.OracleFit("f64", model, 0, ds.train.query, ds.train.pidx, ds.train.click, ds.n_qd)
        f.run(5)
        for config in ((4096, 1024, 256), (256, 1024, 256)):
            cm = api.ClickModel.create(model)
            cm.upload(ds.train, ds.n_qd)
            cm.configure(*config)
            cm.em(5)
            assert_params_close(cm.get_parameters(), f.values(), what=f"m{model} {config}")


def test_ccm_large_continuation_bounds_the_scale():
    """The CCM term of a clicked last rank grows as 1 / (1 - max(t2, t3));
    with t2 near the clamp the fixed-point scale drops and the tiles fall back
    to FP32 bins.  One iteration from the same parameters as the oracle."""
    case = load_case("ccm_ccmclicks")
    rng = np.random.default_rng(9)
    n_qd = int(case["n_qd"])
    values = {"attractiveness": rng.uniform(0.05, 0.95, n_qd).astype(np.float32),
              "continuation": np.array([0.6, 0.999999, 0.2], np.float32)}
    cm = api.ClickModel.create(1)
    cm.upload(sset(case, "train"), n_qd)
    cm.set_parameters(values)
    cm.em(1)
    f = bindings.OracleFit("f64", 1, 0, case["train_query"], case["train_pidx"], case["train_click"], n_qd)
    f.set_values({k: v.astype(np.float64) for k, v in values.items()})
    f.run(1)
    assert_params_close(cm.get_parameters(), f.values(), what="ccm t2 near 1")
