"""Device-block cache and page-locked host pool (csrc/host/devmem.cpp): a
model created, fitted and destroyed again with the same sizes reuses the freed
device blocks and the page-locked buffers its upload reads back into (segment
ranges, has-a-click bits), both still holding the previous fit's data, and
gets the same results; mc_empty_cache(-1) returns both to the driver."""
import numpy as np
import pytest

from conftest import load_case
from massiveclicks_gb300 import api

pytestmark = pytest.mark.gpu


def _fit(model, train, n_qd, test):
    cm = api.ClickModel.create(model)
    cm.upload(train, n_qd)
    cm.upload_test(test)
    cm.em(6)
    out = cm.get_parameters(), cm.evaluate(1).llh
    cm.destroy_parameters()
    return out


@pytest.mark.parametrize("name,model", [("dbn_dbnclicks", api.DBN), ("ubm_dbnclicks", api.UBM),
                                        ("pbm_pbmclicks", api.PBM), ("ccm_ccmclicks", api.CCM)])
def test_reused_blocks_give_identical_fits(name, model):
    case = load_case(name)
    train = api.SessionSet(case["train_query"], case["train_docs"], case["train_pidx"], case["train_click"])
    test = api.SessionSet(case["test_query"], case["test_docs"], case["test_pidx"], case["test_click"])
    api.empty_cache()
    assert api.cache_bytes() == 0
    p1, ll1 = _fit(model, train, int(case["n_qd"]), test)
    cached = api.cache_bytes()
    assert cached > 0
    # Dirty the cached blocks through another fit of a different model first.
    _fit(api.DBN if model != api.DBN else api.PBM, train, int(case["n_qd"]), test)
    p2, ll2 = _fit(model, train, int(case["n_qd"]), test)
    # Shared-memory FP32 bins sum in a run-dependent order, so two runs of a
    # fit differ by a few ulp per iteration; state left over in a reused
    # block would show as errors of 1e-3 and more.
    for k in p1:
        err = np.abs(p1[k].astype(np.float64) - p2[k])
        assert np.all(err <= 5e-6 * np.abs(p1[k]) + 1e-6), k
    assert ll2 == pytest.approx(ll1, rel=1e-6)
    assert api.empty_cache() >= cached
    assert api.cache_bytes() == 0
