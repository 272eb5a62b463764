"""The DBN log-likelihood adjoint (mc_dbn_loglik_forward/backward) against
FP64 central finite differences of the oracle's likelihood (step 1e-4) and,
through the Fisher identity, against the expected complete-data scores of the
exact DBN posterior computed by the oracle."""
import numpy as np
import pytest

from conftest import load_case
from massiveclicks_gb300 import api, gradient
from oracle import bindings

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _setup(name="dbn_dbnclicks", seed=0):
    case = load_case(name)
    n_qd = int(case["n_qd"])
    cm = api.DBNModel()
    cm.upload(api.SessionSet(case["train_query"], case["train_docs"], case["train_pidx"], case["train_click"]), n_qd)
    rng = np.random.default_rng(seed)
    al = rng.normal(-1.0, 1.0, n_qd).astype(np.float32)
    be = rng.normal(-1.0, 1.0, n_qd).astype(np.float32)
    ga = np.array([1.5], np.float32)
    return case, cm, al, be, ga


def _grads(cm, al, be, ga, fp64):
    dev = torch.device("cuda", 0)
    a = torch.tensor(al, device=dev, requires_grad=True)
    b = torch.tensor(be, device=dev, requires_grad=True)
    g = torch.tensor(ga, device=dev, requires_grad=True)
    ll = gradient.dbn_loglik(a, b, g, cm, fp64=fp64)
    ll.backward()
    return float(ll.detach()), a.grad.cpu().numpy().astype(np.float64), b.grad.cpu().numpy().astype(np.float64), \
        float(g.grad.cpu().numpy()[0])


def test_forward_matches_oracle():
    case, cm, al, be, ga = _setup()
    ref = bindings.dbn_loglik(case["train_pidx"], case["train_click"], al.astype(np.float64), be.astype(np.float64),
                              float(ga[0]))
    ll64, *_ = _grads(cm, al, be, ga, True)
    ll32, *_ = _grads(cm, al, be, ga, False)
    assert ll64 == pytest.approx(ref, rel=1e-12)
    assert ll32 == pytest.approx(ref, rel=1e-6)


def _fd_errors(case, al, be, ga, ga_, gb_, gg_, seed=2):
    """Relative errors of a gradient against FP64 central differences of the
    oracle's likelihood (step 1e-4, truncation error about 1e-8 relative) on
    1,000 random parameters.  A pair's difference is taken over the sessions
    that show it: the other sessions' terms are identical on both sides, and
    leaving them in would only add the rounding noise of a 10^4-sized sum
    (about 1e-6 absolute after dividing by 2h).  Parameters whose gradient is
    about 0 compare absolutely (denominator at least 1e-3)."""
    p, m = case["train_pidx"], case["train_click"]
    A, B = al.astype(np.float64), be.astype(np.float64)
    G = float(ga[0])
    h = 1e-4
    rng = np.random.default_rng(seed)
    n_qd = A.shape[0]
    picks = [("a", int(i)) for i in rng.choice(n_qd, 600, replace=False)] + \
            [("b", int(i)) for i in rng.choice(n_qd, 399, replace=False)] + [("g", 0)]
    errs = []
    for kind, i in picks:
        if kind in ("a", "b"):
            rows = np.any(p == i, axis=1)
            ps, ms = p[rows], m[rows]
        if kind == "a":
            x1, x2 = A.copy(), A.copy()
            x1[i] += h; x2[i] -= h
            fd = (bindings.dbn_loglik(ps, ms, x1, B, G) - bindings.dbn_loglik(ps, ms, x2, B, G)) / (2 * h)
            got = ga_[i]
        elif kind == "b":
            x1, x2 = B.copy(), B.copy()
            x1[i] += h; x2[i] -= h
            fd = (bindings.dbn_loglik(ps, ms, A, x1, G) - bindings.dbn_loglik(ps, ms, A, x2, G)) / (2 * h)
            got = gb_[i]
        else:
            fd = (bindings.dbn_loglik(p, m, A, B, G + h) - bindings.dbn_loglik(p, m, A, B, G - h)) / (2 * h)
            got = gg_
        errs.append(abs(got - fd) / max(abs(fd), 1e-3))
    return np.array(errs)


def test_gradient_matches_central_differences():
    """The FP64 instantiation within 1e-6 relative of the differences."""
    case, cm, al, be, ga = _setup(seed=1)
    _, ga_, gb_, gg_ = _grads(cm, al, be, ga, True)
    worst = _fd_errors(case, al, be, ga, ga_, gb_, gg_).max()
    assert worst <= 1e-6, worst


def test_fp32_gradient_matches_central_differences():
    """The FP32 gradient the trainer uses, against the same FP64 differences:
    within 1e-4 relative.  Adam divides each step by the root of a running
    second moment, so the step direction needs a few significant digits; the
    bar is 100 times tighter than the 1e-2 at which Adam's steps would change
    visibly."""
    case, cm, al, be, ga = _setup(seed=1)
    _, ga_, gb_, gg_ = _grads(cm, al, be, ga, False)
    worst = _fd_errors(case, al, be, ga, ga_, gb_, gg_).max()
    assert worst <= 1e-4, worst


def test_tile_path_matches_session_path():
    """A model whose sessions are grouped by query takes the tile path (the
    gradient summed per tile in shared memory); the same sessions in random
    order take one thread per session with global atomics.  Both give the
    same log-likelihood and gradient, also over partial ranges."""
    case, cm, al, be, ga = _setup("dbn_ccmclicks", seed=6)
    train = api.SessionSet(case["train_query"], case["train_docs"], case["train_pidx"], case["train_click"])
    shuffled = gradient.shuffled_sessions(train, seed=3)
    cm2 = api.DBNModel()
    cm2.upload(shuffled, int(case["n_qd"]))
    for fp64 in (True, False):
        l1, a1, b1, g1 = _grads(cm, al, be, ga, fp64)
        l2, a2, b2, g2 = _grads(cm2, al, be, ga, fp64)
        tol = 1e-9 if fp64 else 2e-5
        assert l1 == pytest.approx(l2, rel=tol)
        np.testing.assert_allclose(a1, a2, rtol=tol, atol=tol)
        np.testing.assert_allclose(b1, b2, rtol=tol, atol=tol)
        assert g1 == pytest.approx(g2, rel=tol)
    # a range that starts and ends inside tiles, against the oracle
    dev = torch.device("cuda", 0)
    lo, hi = 777, cm.n_train - 555
    a = torch.tensor(al, device=dev, requires_grad=True)
    b = torch.tensor(be, device=dev, requires_grad=True)
    g = torch.tensor(ga, device=dev, requires_grad=True)
    ll = gradient.dbn_loglik(a, b, g, cm, lo, hi - lo, fp64=True)
    ref = bindings.dbn_loglik(case["train_pidx"][lo:hi], case["train_click"][lo:hi], al.astype(np.float64),
                              be.astype(np.float64), float(ga[0]))
    assert float(ll.detach()) == pytest.approx(ref, rel=1e-12)


def test_gradient_equals_fisher_scores():
    case, cm, al, be, ga = _setup(seed=3)
    _, ga_, gb_, gg_ = _grads(cm, al, be, ga, True)
    sa, sb, sg = bindings.dbn_fisher(case["train_pidx"], case["train_click"], al.astype(np.float64),
                                     be.astype(np.float64), float(ga[0]))
    np.testing.assert_allclose(ga_, sa, rtol=1e-7, atol=1e-7)
    np.testing.assert_allclose(gb_, sb, rtol=1e-7, atol=1e-7)
    assert gg_ == pytest.approx(sg, rel=1e-7)


def test_fp32_gradient_close_to_fp64():
    case, cm, al, be, ga = _setup(seed=4)
    _, a64, b64, g64 = _grads(cm, al, be, ga, True)
    _, a32, b32, g32 = _grads(cm, al, be, ga, False)
    np.testing.assert_allclose(a32, a64, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(b32, b64, rtol=1e-4, atol=1e-5)
    assert g32 == pytest.approx(g64, rel=1e-4)


def _grads_range(cm, al, be, ga, begin, count, fp64=False):
    dev = torch.device("cuda", 0)
    a = torch.tensor(al, device=dev, requires_grad=True)
    b = torch.tensor(be, device=dev, requires_grad=True)
    g = torch.tensor(ga, device=dev, requires_grad=True)
    ll = gradient.dbn_loglik(a, b, g, cm, begin, count, fp64=fp64)
    ll.backward()
    return a.grad.cpu().numpy().astype(np.float64), b.grad.cpu().numpy().astype(np.float64), \
        float(g.grad.cpu().numpy()[0])


def test_fp32_counted_terms_whole_and_cut_tiles():
    """The FP32 tile path counts the constant terms (clicked ranks, unclicked
    ranks before the last click): from the per-tile counts for a tile wholly
    inside the called range, with atomics for a tile the range cuts.  The
    gradient over all training sessions equals the sum over two ranges split
    inside tiles, and both match FP64 at the FP32 bar."""
    case, cm, al, be, ga = _setup("dbn_ccmclicks", seed=8)
    n = cm.n_train
    a_all, b_all, g_all = _grads_range(cm, al, be, ga, 0, n)
    cut = n // 2 + 17
    a1, b1, g1 = _grads_range(cm, al, be, ga, 0, cut)
    a2, b2, g2 = _grads_range(cm, al, be, ga, cut, n - cut)
    a64, b64, g64 = _grads_range(cm, al, be, ga, 0, n, fp64=True)
    np.testing.assert_allclose(a1 + a2, a_all, rtol=2e-5, atol=2e-5)
    np.testing.assert_allclose(b1 + b2, b_all, rtol=2e-5, atol=2e-5)
    assert g1 + g2 == pytest.approx(g_all, rel=1e-5)
    for got in (a_all, a1 + a2):
        np.testing.assert_allclose(got, a64, rtol=1e-4, atol=1e-5)
    for got in (b_all, b1 + b2):
        np.testing.assert_allclose(got, b64, rtol=1e-4, atol=1e-5)


def test_fp32_small_windows_of_split_queries():
    """Queries with thousands of sessions over a few dozen documents are split
    over several tiles whose windows (at most 30 pairs) take the small-window
    layout (per-(warp, lane % 4) copies of the bins), read from the packed
    copy for whole tiles and with count atomics for a tile a range cuts.  The
    FP32 gradient matches FP64 at the FP32 bar in both."""
    cfg = api.synth_config(1, n_sessions=100_000, n_queries=20, pool=30, seed=91)
    q, d, m = api.synth_sessions(cfg)
    ds = api.Dataset.from_sessions(q, d, m, 0.2)
    cm = api.DBNModel()
    cm.upload(ds.train, ds.n_qd)
    assert cm.fused_path()[0] == "tiles"
    rng = np.random.default_rng(12)
    al = rng.normal(-1.0, 1.0, ds.n_qd).astype(np.float32)
    be = rng.normal(-1.0, 1.0, ds.n_qd).astype(np.float32)
    ga = np.array([1.5], np.float32)
    n = cm.n_train
    a64, b64, g64 = _grads_range(cm, al, be, ga, 0, n, fp64=True)
    a32, b32, g32 = _grads_range(cm, al, be, ga, 0, n)
    cut = n // 3 + 101
    a1, b1, _ = _grads_range(cm, al, be, ga, 0, cut)
    a2, b2, _ = _grads_range(cm, al, be, ga, cut, n - cut)
    for got in (a32, a1 + a2):
        np.testing.assert_allclose(got, a64, rtol=1e-4, atol=1e-5)
    for got in (b32, b1 + b2):
        np.testing.assert_allclose(got, b64, rtol=1e-4, atol=1e-5)
    assert g32 == pytest.approx(g64, rel=1e-4)


def test_ranges_add_up():
    case, cm, al, be, ga = _setup(seed=5)
    dev = torch.device("cuda", 0)
    a = torch.tensor(al, device=dev)
    b = torch.tensor(be, device=dev)
    g = torch.tensor(ga, device=dev)
    n = cm.n_train
    whole = float(gradient.dbn_loglik(a, b, g, cm, 0, n, fp64=True))
    parts = float(gradient.dbn_loglik(a, b, g, cm, 0, 1000, fp64=True)) + \
        float(gradient.dbn_loglik(a, b, g, cm, 1000, n - 1000, fp64=True))
    assert parts == pytest.approx(whole, rel=1e-12)


def test_adam_improves_likelihood():
    case = load_case("dbn_ccmclicks")
    n_qd = int(case["n_qd"])
    train = gradient.shuffled_sessions(api.SessionSet(case["train_query"], case["train_docs"], case["train_pidx"],
                                                      case["train_click"]))
    cm = api.DBNModel()
    cm.upload(train, n_qd)
    dev = torch.device("cuda", 0)
    z = torch.zeros(n_qd, device=dev)
    before = float(gradient.dbn_loglik(z, z, torch.zeros(1, device=dev), cm))
    a, b, g = gradient.train_adam(cm, n_qd, steps=60, batch=1024, lr=0.05)
    after = float(gradient.dbn_loglik(a.detach(), b.detach(), g.detach(), cm))
    assert after > before + 0.05 * abs(before)


def test_bad_range_rejected():
    _, cm, al, be, ga = _setup()
    dev = torch.device("cuda", 0)
    a = torch.tensor(al, device=dev)
    with pytest.raises(api._capi.MCError):
        gradient.dbn_loglik(a, a, torch.tensor(ga, device=dev), cm, cm.n_train, 5)
