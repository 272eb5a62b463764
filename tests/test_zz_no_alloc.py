"""mc_evaluate_static, the allocation-free evaluation entry point.

It serves callers that cannot allocate device memory when they evaluate: a
serving process whose device memory already belongs to its own pool, a job
under a memory budget that forbids new allocations, or a host thread that must
not enter the allocator (and its implicit synchronisation) while other streams
run.  Checked here through the C-ABI:

  * against the FP64 oracle and against mc_model_evaluate on the same
    parameters and test sessions, on two calls in a row (the second call
    reuses the scratch array the first one left behind);
  * on several thousand blocks: a call near the 16,777,216-session limit and
    then a smaller one (sizes not multiples of the 2048-session block), each
    against mc_model_evaluate, so stale rows of the larger call are not read;
  * that a call after the set-up changes neither the driver's free device
    memory nor torch's reserved memory;
  * that an index that is neither -1 nor a pair index is an error.

The caller's device buffers come from torch; the entry point itself allocates
nothing.  This file is collected last, so a stop at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_case
from massiveclicks_gb300 import api, _capi
from massiveclicks_gb300._capi import CCM, DBN, PBM, UBM
from oracle import bindings

pytestmark = pytest.mark.gpu

RTOL_MODEL = 2e-6    # against mc_model_evaluate: the same FP32 terms, another summation order
RTOL_ORACLE = 1e-5   # against the FP64 oracle: the evaluation bar of the other GPU tests
MAX_SESSIONS = 16_777_216
PUBLIC = {PBM: "examination", UBM: "examination", CCM: "continuation", DBN: "continuation"}


def _fit(case, model, iters):
    cm = api.ClickModel.create(model)
    cm.upload(api.SessionSet(case["train_query"], case["train_docs"], case["train_pidx"], case["train_click"]),
              int(case["n_qd"]))
    cm.upload_test(api.SessionSet(case["test_query"], case["test_docs"], case["test_pidx"], case["test_click"]))
    cm.em(iters)
    return cm


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class DeviceParams:
    """The model's parameter values in torch device tensors (the caller's buffers)."""

    def __init__(self, torch, model, params):
        dev = torch.device("cuda", 0)
        self.atr = torch.from_numpy(params["attractiveness"]).to(dev)
        self.sat = torch.from_numpy(params["satisfaction"]).to(dev) if model == DBN else None
        self.pub = torch.from_numpy(params[PUBLIC[model]]).to(dev)


def _static(lib, model, n, pidx, click, n_qd, p: DeviceParams):
    ll = C.c_double()
    l2 = np.zeros(10, np.float64)
    rc = lib.mc_evaluate_static(model, n, _ptr(pidx), _ptr(click), n_qd, _ptr(p.atr), _ptr(p.sat), _ptr(p.pub),
                                C.byref(ll), l2.ctypes.data_as(C.c_void_p), None)
    return rc, ll.value, l2


def _dev_sessions(torch, pidx, click):
    dev = torch.device("cuda", 0)
    p = torch.from_numpy(np.ascontiguousarray(pidx, np.int32).reshape(-1)).to(dev)
    m = torch.from_numpy(np.ascontiguousarray(click, np.uint16).view(np.int16)).to(dev)
    return p, m


@pytest.mark.parametrize("name,model", [("pbm_pbmclicks", PBM), ("ccm_ccmclicks", CCM), ("dbn_ccmclicks", DBN),
                                        ("ubm_dbnclicks", UBM)])
def test_static_evaluation_matches_oracle_and_model_evaluate(name, model):
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    case = load_case(name)
    cm = _fit(case, model, 6)
    ref = cm.evaluate(1)
    params = cm.get_parameters()
    f = bindings.OracleFit("f64", model, 0, case["train_query"], case["train_pidx"], case["train_click"],
                           int(case["n_qd"]))
    f.set_values(params)
    oracle = f.evaluate(case["test_pidx"], case["test_click"])
    dp = DeviceParams(torch, model, params)
    pidx, click = _dev_sessions(torch, case["test_pidx"], case["test_click"])
    n = int(case["test_query"].shape[0])
    torch.cuda.synchronize()
    for _ in range(2):
        rc, ll, l2 = _static(lib, model, n, pidx, click, int(case["n_qd"]), dp)
        _capi.check(rc)
        assert ll == pytest.approx(ref.llh_sum, rel=RTOL_MODEL)
        np.testing.assert_allclose(l2, ref.log2_sums, rtol=RTOL_MODEL)
        assert ll == pytest.approx(oracle["llh_sum"], rel=RTOL_ORACLE)
        np.testing.assert_allclose(l2, oracle["log2_sums"], rtol=RTOL_ORACLE)


@pytest.mark.parametrize("model", [DBN, UBM])
def test_static_evaluation_many_blocks_then_fewer(model):
    """8192 blocks (3 sessions short of the limit), then 2442 blocks on a
    prefix of the same buffers: each call against mc_model_evaluate of the
    same sessions."""
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    case = load_case("dbn_ccmclicks" if model == DBN else "ubm_dbnclicks")
    cm = _fit(case, model, 4)
    params = cm.get_parameters()
    n_qd = int(case["n_qd"])
    rng = np.random.default_rng(11)
    n_big, n_small = MAX_SESSIONS - 3, 5_000_001
    pidx = rng.integers(-1, n_qd, size=(n_big, 10), dtype=np.int32)
    click = rng.integers(0, 1024, size=n_big, dtype=np.uint16)
    dp = DeviceParams(torch, model, params)
    d_pidx, d_click = _dev_sessions(torch, pidx, click)
    torch.cuda.synchronize()
    for n in (n_big, n_small):
        rc, ll, l2 = _static(lib, model, n, d_pidx, d_click, n_qd, dp)
        _capi.check(rc)
        cm.upload_test(api.SessionSet(None, None, pidx[:n], click[:n]))
        ref = cm.evaluate(1)
        assert ref.n_sessions == n
        assert ll == pytest.approx(ref.llh_sum, rel=RTOL_MODEL)
        np.testing.assert_allclose(l2, ref.log2_sums, rtol=RTOL_MODEL)


def test_static_evaluation_allocates_nothing():
    """After the set-up call (n_sessions = 0), a call leaves the driver's free
    device memory and torch's reserved memory as they were."""
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    case = load_case("dbn_ccmclicks")
    cm = _fit(case, DBN, 3)
    dp = DeviceParams(torch, DBN, cm.get_parameters())
    pidx, click = _dev_sessions(torch, case["test_pidx"], case["test_click"])
    n = int(case["test_query"].shape[0])
    rc, ll, l2 = _static(lib, DBN, 0, None, None, int(case["n_qd"]), dp)
    _capi.check(rc)
    assert ll == 0.0 and not l2.any()
    _capi.check(_static(lib, DBN, n, pidx, click, int(case["n_qd"]), dp)[0])
    torch.cuda.synchronize()
    free0, reserved0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_reserved()
    for _ in range(3):
        _capi.check(_static(lib, DBN, n, pidx, click, int(case["n_qd"]), dp)[0])
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_reserved() == reserved0


@pytest.mark.parametrize("bad", [-2, "n_qd"])
def test_static_evaluation_rejects_bad_indices(bad):
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    case = load_case("dbn_ccmclicks")
    cm = _fit(case, DBN, 2)
    ref = cm.evaluate(1)
    dp = DeviceParams(torch, DBN, cm.get_parameters())
    n_qd = int(case["n_qd"])
    tp = np.array(case["test_pidx"], np.int32)
    tp[len(tp) // 2, 3] = n_qd if bad == "n_qd" else bad
    pidx, click = _dev_sessions(torch, tp, case["test_click"])
    n = len(tp)
    rc, _, _ = _static(lib, DBN, n, pidx, click, n_qd, dp)
    assert rc == 1
    buf = C.create_string_buffer(512)
    lib.mc_last_error(buf, 512)
    assert b"neither -1 nor in [0, n_qd)" in buf.value
    good, gclick = _dev_sessions(torch, case["test_pidx"], case["test_click"])
    rc, ll, _ = _static(lib, DBN, n, good, gclick, n_qd, dp)
    _capi.check(rc)
    assert ll == pytest.approx(ref.llh_sum, rel=RTOL_MODEL)


def test_static_evaluation_rejects_sizes_beyond_its_scratch():
    lib = _capi.load()
    ll = C.c_double()
    l2 = np.zeros(10, np.float64)
    rc = lib.mc_evaluate_static(DBN, MAX_SESSIONS + 1, None, None, 1, None, None, None, C.byref(ll),
                                l2.ctypes.data_as(C.c_void_p), None)
    assert rc == 1
    buf = C.create_string_buffer(512)
    lib.mc_last_error(buf, 512)
    assert b"exceed the maximum" in buf.value
