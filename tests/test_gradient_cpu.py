"""Host-side layout of the gradient trainer's sessions (no GPU needed)."""
import numpy as np

from conftest import load_case
from massiveclicks_gb300 import api, gradient


def test_query_order_renumbers_consistently():
    """Adam's session layout: whole queries in a random order, pairs
    renumbered, and a map back to the original numbering."""
    case = load_case("dbn_ccmclicks")
    train = api.SessionSet(case["train_query"], case["train_docs"], case["train_pidx"], case["train_click"])
    t, n_qd, to_orig = gradient.query_order(train, seed=4)
    assert n_qd == int(case["n_qd"]) and len(t) == len(train)
    # grouped by query, not in ascending query order
    starts = np.flatnonzero(np.r_[True, t.query[1:] != t.query[:-1]])
    assert len(starts) == len(np.unique(t.query))
    assert sorted(to_orig.tolist()) == list(range(n_qd))
    # every (query, doc) maps to the original index of the same pair
    key = {}
    for qq, dd, pp in zip(np.repeat(train.query, 10), train.docs.ravel(), train.pidx.ravel()):
        key[(int(qq), int(dd))] = int(pp)
    uq = np.unique(train.query)
    # t.query holds the random ranks; recover the original query of each rank
    for s in range(0, len(t), 97):
        for r in range(10):
            orig_pidx = to_orig[t.pidx[s, r]]
            matches = [k for k, v in key.items() if v == orig_pidx]
            assert len(matches) == 1 and matches[0][1] == int(t.docs[s, r])
    assert len(uq) == len(starts)
