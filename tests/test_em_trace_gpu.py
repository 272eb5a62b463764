"""Training log-likelihood per iteration (mc_model_em_trace): each value is the
evaluation of the training sessions under the parameters one fused iteration
produced; checked against the evaluation entry point on the same model and
against the FP64 oracle after the same number of iterations."""
import numpy as np
import pytest

from conftest import load_case
from massiveclicks_gb300 import api
from oracle import bindings

pytestmark = pytest.mark.gpu

LL_RTOL = 1e-5


@pytest.mark.parametrize("name,model", [("dbn_dbnclicks", api.DBN), ("ccm_ccmclicks", api.CCM),
                                        ("ubm_dbnclicks", api.UBM), ("pbm_pbmclicks", api.PBM)])
def test_trace_matches_evaluation_and_oracle(name, model):
    case = load_case(name)
    n_qd = int(case["n_qd"])
    train = api.SessionSet(case["train_query"], case["train_docs"], case["train_pidx"], case["train_click"])
    cm = api.ClickModel.create(model)
    cm.upload(train, n_qd)
    lls = cm.em_trace(5)
    assert lls.shape == (5,) and np.all(np.isfinite(lls))
    # the last value evaluates the parameters the model now holds
    assert lls[-1] == pytest.approx(cm.evaluate(0).llh, rel=1e-12)
    more = cm.em_trace(2)  # continues from where the first trace stopped
    f = bindings.OracleFit("f64", model, 0, train.query, train.pidx, train.click, n_qd)
    for i, got in enumerate(np.concatenate([lls, more])):
        f.run(1)
        ref = f.evaluate(train.pidx, train.click)["llh"]
        assert got == pytest.approx(ref, rel=LL_RTOL), f"iteration {i + 1}"


def test_trace_rejects_bad_arguments():
    case = load_case("dbn_dbnclicks")
    cm = api.DBNModel()
    with pytest.raises(api._capi.MCError):
        cm.em_trace(1)  # nothing uploaded
    cm.upload(api.SessionSet(case["train_query"], case["train_docs"], case["train_pidx"], case["train_click"]),
              int(case["n_qd"]))
    with pytest.raises(api._capi.MCError):
        cm.em_trace(-1)
    assert cm.em_trace(0).shape == (0,)
