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
