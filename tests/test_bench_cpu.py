"""Host-side helpers of bench.py: the bounded CPU sample of whole queries and
the workload text."""
import types

import numpy as np

import bench


def _ds(query):
    return types.SimpleNamespace(train=types.SimpleNamespace(query=np.asarray(query, np.int32)))


def test_cpu_sample_takes_whole_queries_within_budget():
    rng = np.random.default_rng(3)
    sizes = rng.integers(1, 40, 500)
    query = np.repeat(np.arange(500), sizes)
    idx = bench.cpu_sample(_ds(query), 1000)
    assert 0 < len(idx) <= 1000
    assert np.all(np.diff(idx) > 0)  # sorted, no repeats
    picked = np.unique(query[idx])
    # every picked query is taken whole
    for q in picked:
        assert np.count_nonzero(query[idx] == q) == sizes[q]
    # deterministic
    assert np.array_equal(idx, bench.cpu_sample(_ds(query), 1000))


def test_cpu_sample_edges():
    assert len(bench.cpu_sample(_ds([]), 10)) == 0
    assert len(bench.cpu_sample(_ds([0] * 50), 10)) == 0  # the only query is above the budget
    assert np.array_equal(bench.cpu_sample(_ds([0, 0, 1]), 3), np.arange(3))


def test_workload_text_follows_the_sizes():
    a = types.SimpleNamespace(sessions=20_000_000, queries=1_000_000)
    assert bench.data_text(a).startswith("synthetic: 20M sessions, 1M queries")
    b = types.SimpleNamespace(sessions=250_000, queries=20_000)
    assert "250,000 sessions, 20,000 queries" in bench.data_text(b)
    assert bench.metric_for("dbn") != bench.metric_for("pbm")
    assert "PBM" in bench.metric_for("pbm")


def test_sample_sets_renumber_densely(native_lib):
    """The bench line's parity sample: whole queries, qd indices renumbered
    densely and in order (so each query still owns a contiguous range), and
    the test sessions of the sampled queries with the same renumbering."""
    from massiveclicks_gb300 import api
    cfg = api.synth_config(2, n_sessions=30_000, n_queries=3_000)
    q, d, m = api.synth_sessions(cfg)
    ds = api.Dataset.from_sessions(q, d, m, 0.2)
    idx = bench.cpu_sample(ds, 5_000)
    train, test, n_qd = bench.sample_sets(ds, idx)
    for k in ("query", "docs", "click"):
        assert np.array_equal(getattr(train, k), getattr(ds.train, k)[idx]), k
    full = ds.train.pidx[idx].ravel()
    mine = train.pidx.ravel()
    assert np.array_equal(np.unique(mine), np.arange(n_qd))
    order = np.argsort(full, kind="stable")
    assert np.all(np.diff(mine[order]) >= 0)                 # the renumbering keeps the order
    assert np.array_equal(np.diff(full[order]) == 0, np.diff(mine[order]) == 0)
    sampled = np.unique(train.query)
    keep = np.isin(ds.test.query, sampled)
    assert len(test) == int(keep.sum())
    assert np.array_equal(test.pidx < 0, ds.test.pidx[keep] < 0)
    seen = ds.test.pidx[keep] >= 0
    lut = dict(zip(full.tolist(), mine.tolist()))
    assert all(lut[a] == b for a, b in zip(ds.test.pidx[keep][seen].tolist(), test.pidx[seen].tolist()))
