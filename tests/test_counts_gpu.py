"""Count path of PBM and UBM (em_counts.cu): a fused iteration over the
per-(qd, key) unclicked-occurrence counts built at upload.  Checked against the
FP64 oracle (which runs the reference's per-session E-step), for any session
order, and the number of count entries against a numpy restatement of the
keys."""
import numpy as np
import pytest

from conftest import load_case
from massiveclicks_gb300 import api
from massiveclicks_gb300._capi import IMPL_FUSED
from oracle import bindings

pytestmark = pytest.mark.gpu

PARAM_RTOL = 1e-5
PARAM_ATOL = 1e-6
LL_RTOL = 1e-5


def _sset(case, which="train"):
    return api.SessionSet(case[f"{which}_query"], case[f"{which}_docs"], case[f"{which}_pidx"], case[f"{which}_click"])


def _close(a, b, what):
    for k in b:
        err = np.abs(a[k].astype(np.float64) - b[k])
        assert np.all(err <= PARAM_RTOL * np.abs(b[k]) + PARAM_ATOL), f"{what} {k}: max err {err.max():.3g}"


def distinct_keys(model: int, pidx: np.ndarray, click: np.ndarray) -> int:
    """Distinct (qd, key, alive) over the unclicked occurrences: key = rank
    (PBM) or examination slot r(r+1)/2 + previous click rank, 9 when none
    (UBM); alive = no later rank of the session has the same slot."""
    n = len(click)
    bits = (click.astype(np.int64)[:, None] >> np.arange(10)) & 1
    slot = np.empty((n, 10), np.int64)
    last = np.full(n, 9, np.int64)
    for r in range(10):
        slot[:, r] = r if model == api.PBM else r * (r + 1) // 2 + last
        last = np.where(bits[:, r] == 1, r, last)
    alive = np.ones((n, 10), bool)
    for r in range(10):
        for r2 in range(r + 1, 10):
            alive[:, r] &= slot[:, r2] != slot[:, r]
    key = (pidx.astype(np.int64) << 7) | (slot << 1) | alive.astype(np.int64)
    return int(np.unique(key[bits == 0]).size)


@pytest.mark.parametrize("name,model", [("pbm_pbmclicks", api.PBM), ("ubm_dbnclicks", api.UBM),
                                        ("dbn_dbnclicks", api.DBN), ("ccm_ccmclicks", api.CCM)])
def test_path_and_entry_count(name, model):
    case = load_case(name)
    train = _sset(case)
    cm = api.ClickModel.create(model)
    cm.upload(train, int(case["n_qd"]))
    path, n_ent = cm.fused_path()
    if model in (api.PBM, api.UBM):
        assert path == ("dense" if model == api.PBM else "counts")
        assert n_ent == distinct_keys(model, train.pidx, train.click)
    else:
        assert (path, n_ent) == ("tiles", 0)


@pytest.mark.parametrize("model", [api.PBM, api.UBM])
def test_any_session_order(model):
    """Sessions not grouped by query (the tile kernel's precondition) still
    take the count path, with the oracle's results."""
    case = load_case("pbm_pbmclicks" if model == api.PBM else "ubm_dbnclicks")
    t = _sset(case)
    perm = np.random.default_rng(5).permutation(len(t))
    train = api.SessionSet(t.query[perm], t.docs[perm], t.pidx[perm], t.click[perm])
    n_qd = int(case["n_qd"])
    cm = api.ClickModel.create(model)
    cm.upload(train, n_qd)
    assert cm.fused_path()[0] in ("counts", "dense")
    lls = cm.em_trace(3)
    cm.em(4, IMPL_FUSED)
    f = bindings.OracleFit("f64", model, 0, train.query, train.pidx, train.click, n_qd)
    f.run(3)
    assert lls[-1] == pytest.approx(f.evaluate(train.pidx, train.click)["llh"], rel=LL_RTOL)
    f.run(4)
    _close(cm.get_parameters(), f.values(), f"shuffled m{model}")


def test_tile_models_still_need_grouped_sessions():
    case = load_case("dbn_dbnclicks")
    t = _sset(case)
    perm = np.random.default_rng(6).permutation(len(t))
    cm = api.DBNModel()
    cm.upload(api.SessionSet(t.query[perm], t.docs[perm], t.pidx[perm], t.click[perm]), int(case["n_qd"]))
    assert cm.fused_path()[0] == "tiles"
    with pytest.raises(api._capi.MCError):
        cm.em(1, IMPL_FUSED)


@pytest.mark.parametrize("model", [api.PBM, api.UBM])
def test_all_clicked_and_repeated_keys(model):
    """Sessions with every rank clicked give no entries; many sessions of one
    query with one click pattern collapse into a few entries with large counts."""
    rng = np.random.default_rng(11)
    n = 6000
    query = np.sort(rng.integers(0, 3, n)).astype(np.int32)
    docs = np.stack([q * 100 + np.arange(10) for q in query]).astype(np.int32)
    masks = np.where(rng.random(n) < 0.3, 0x3FF, np.where(rng.random(n) < 0.5, 0b101, 0)).astype(np.uint16)
    ds = api.Dataset.from_sessions(query, docs, masks, 0.0)
    cm = api.ClickModel.create(model)
    cm.upload(ds.train, ds.n_qd)
    path, n_ent = cm.fused_path()
    assert path in ("counts", "dense") and n_ent == distinct_keys(model, ds.train.pidx, ds.train.click)
    cm.em(5, IMPL_FUSED)
    f = bindings.OracleFit("f64", model, 0, ds.train.query, ds.train.pidx, ds.train.click, ds.n_qd)
    f.run(5)
    _close(cm.get_parameters(), f.values(), f"repeated m{model}")

    every = api.Dataset.from_sessions(query[:50], docs[:50], np.full(50, 0x3FF, np.uint16), 0.0)
    cm2 = api.ClickModel.create(model)
    cm2.upload(every.train, every.n_qd)
    assert cm2.fused_path() in (("counts", 0), ("dense", 0))
    cm2.em(3, IMPL_FUSED)
    f2 = bindings.OracleFit("f64", model, 0, every.train.query, every.train.pidx, every.train.click, every.n_qd)
    f2.run(3)
    _close(cm2.get_parameters(), f2.values(), f"all clicked m{model}")


def test_pbm_count_above_16_bits_takes_the_entry_path():
    """A (qd, rank) with more than 65535 unclicked occurrences does not fit the
    dense 16-bit table: PBM then runs the entry kernel, with the same results."""
    n = 70000
    query = np.zeros(n, np.int32)
    docs = np.tile(np.arange(10, dtype=np.int32), (n, 1))
    masks = np.where(np.arange(n) % 7 == 0, 0b10, 0).astype(np.uint16)
    ds = api.Dataset.from_sessions(query, docs, masks, 0.0)
    cm = api.PBMModel()
    cm.upload(ds.train, ds.n_qd)
    path, n_ent = cm.fused_path()
    assert path == "counts" and n_ent == distinct_keys(api.PBM, ds.train.pidx, ds.train.click)
    cm.em(4, IMPL_FUSED)
    f = bindings.OracleFit("f64", api.PBM, 0, ds.train.query, ds.train.pidx, ds.train.click, ds.n_qd)
    f.run(4)
    _close(cm.get_parameters(), f.values(), "pbm 16-bit overflow")


@pytest.mark.parametrize("model,shapes", [
    (api.UBM, [(4, 256, 8), (8, 128, 16), (16, 192, 10), (16, 64, 32)]),
    (api.PBM, [(0, 128, 12), (0, 64, 32), (0, 256, 4)]),
])
def test_count_shapes_do_not_change_results(model, shapes):
    """The count kernels' launch shape (bin copies, block, blocks per SM) is a
    tuning knob only; the autotuner picks one of its candidates and leaves
    the parameters where they were."""
    case = load_case("ubm_dbnclicks" if model == api.UBM else "pbm_pbmclicks")
    f = bindings.OracleFit("f64", model, 0, case["train_query"], case["train_pidx"], case["train_click"],
                           int(case["n_qd"]))
    f.run(5)
    for shape in shapes:
        cm = api.ClickModel.create(model)
        cm.upload(_sset(case), int(case["n_qd"]))
        cm.configure_counts(*shape)
        got = cm.count_config()
        assert got[1:] == shape[1:] and (model == api.PBM or got[0] == shape[0])
        cm.em(5)
        _close(cm.get_parameters(), f.values(), f"m{model} shape {shape}")
    cm = api.ClickModel.create(model)
    cm.upload(_sset(case), int(case["n_qd"]))
    cm.em(2)
    before = cm.get_parameters()
    cm.autotune()
    after = cm.get_parameters()
    for k in before:
        assert np.array_equal(before[k], after[k])
    cm.em(3)
    _close(cm.get_parameters(), f.values(), f"m{model} autotuned {cm.count_config()}")


def test_count_shape_rejects_bad_values():
    case = load_case("ubm_dbnclicks")
    cm = api.ClickModel.create(api.UBM)
    cm.upload(_sset(case), int(case["n_qd"]))
    for bad in [(3, 256, 8), (8, 96 + 1, 8), (8, 512, 8), (8, 256, 0), (8, 32, 8)]:
        with pytest.raises(api._capi.MCError):
            cm.configure_counts(*bad)
