"""mc_evaluate_static, the allocation-free evaluation entry point.

It serves callers that cannot allocate device memory when they evaluate (their
device memory belongs to their own pool, or they must not enter the allocator
while other streams run).  Checked here against mc_model_evaluate on the same
parameters and test sessions, through the C-ABI, on two calls in a row (the
second call reuses the scratch array the first one left behind).  The caller's
device buffers come from torch; the entry point itself allocates nothing.

This file is collected last, so a stop at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_case
from massiveclicks_gb300 import api, _capi

pytestmark = pytest.mark.gpu

RTOL = 2e-6          # the evaluation tolerance of the other GPU tests
MAX_SESSIONS = 16_777_216


def _fit(case, model, iters):
    cm = api.ClickModel.create(model)
    cm.upload(api.SessionSet(case["train_query"], case["train_docs"], case["train_pidx"], case["train_click"]),
              int(case["n_qd"]))
    cm.upload_test(api.SessionSet(case["test_query"], case["test_docs"], case["test_pidx"], case["test_click"]))
    cm.em(iters)
    return cm


def _dev_ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


@pytest.mark.parametrize("name,model", [("pbm_pbmclicks", 0), ("ccm_ccmclicks", 1), ("dbn_ccmclicks", 2),
                                        ("ubm_dbnclicks", 3)])
def test_static_evaluation_matches_model_evaluate(name, model):
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    case = load_case(name)
    cm = _fit(case, model, 6)
    ref = cm.evaluate(1)
    params = cm.get_parameters()
    dev = torch.device("cuda", 0)
    n = int(case["test_query"].shape[0])
    n_qd = int(case["n_qd"])
    pidx = torch.from_numpy(np.ascontiguousarray(case["test_pidx"], np.int32).reshape(-1)).to(dev)
    click = torch.from_numpy(np.ascontiguousarray(case["test_click"], np.uint16).view(np.int16)).to(dev)
    atr = torch.from_numpy(params["attractiveness"]).to(dev)
    sat = torch.from_numpy(params["satisfaction"]).to(dev) if model == 2 else None
    pub_name = "continuation" if model in (1, 2) else "examination"
    pub = torch.from_numpy(params[pub_name]).to(dev)
    torch.cuda.synchronize()
    for _ in range(2):
        ll = C.c_double()
        l2 = np.zeros(10, np.float64)
        rc = lib.mc_evaluate_static(model, n, _dev_ptr(pidx), _dev_ptr(click), n_qd, _dev_ptr(atr), _dev_ptr(sat),
                                    _dev_ptr(pub), C.byref(ll), l2.ctypes.data_as(C.c_void_p), None)
        _capi.check(rc)
        assert ll.value == pytest.approx(ref.llh_sum, rel=RTOL)
        np.testing.assert_allclose(l2, ref.log2_sums, rtol=RTOL)


def test_static_evaluation_rejects_sizes_beyond_its_scratch():
    lib = _capi.load()
    ll = C.c_double()
    l2 = np.zeros(10, np.float64)
    rc = lib.mc_evaluate_static(2, MAX_SESSIONS + 1, None, None, 1, None, None, None, C.byref(ll),
                                l2.ctypes.data_as(C.c_void_p), None)
    assert rc == 1
    buf = C.create_string_buffer(512)
    lib.mc_last_error(buf, 512)
    assert b"exceed the maximum" in buf.value
