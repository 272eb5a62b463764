"""Product ingest (mc_dataset_*) against the reference's partitions: parsing,
the tail test split, the unstable sort by query, the qd indices and the test
filtering must all be bit-exact."""
import ctypes
import tempfile
from pathlib import Path

import numpy as np
import pytest

from conftest import CASES, load_case
from massiveclicks_gb300 import api, _capi


@pytest.mark.parametrize("name", CASES)
def test_parse_matches_reference(name, native_lib):
    case = load_case(name)
    with tempfile.TemporaryDirectory() as tmp:
        log = Path(tmp) / "log.txt"
        log.write_bytes(case["log"].tobytes())
        ds = api.Dataset.parse(str(log), int(case["max_sessions"]), float(case["test_share"]))
    assert ds.n_qd == int(case["n_qd"])
    for s, st in (("train", ds.train), ("test", ds.test)):
        assert np.array_equal(st.query, case[f"{s}_query"]), (name, s, "query")
        assert np.array_equal(st.docs, case[f"{s}_docs"]), (name, s, "docs")
        assert np.array_equal(st.pidx, case[f"{s}_pidx"]), (name, s, "pidx")
        assert np.array_equal(st.click, case[f"{s}_click"]), (name, s, "click")


def _oracle_partition(cfg, tmp):
    from oracle import bindings
    log = Path(tmp) / "log.txt"
    api.write_log(cfg, str(log))
    return log, bindings.parse(str(log), cfg.n_sessions, 0.2)


@pytest.mark.parametrize("preset,n,nq", [(0, 20000, 300), (1, 30000, 3000), (2, 30000, 5000)])
def test_parse_matches_oracle_ingest(preset, n, nq, native_lib, oracle_lib):
    """Larger logs than the fixtures, against the oracle's literal ingest
    (std::sort over session records, map of maps)."""
    cfg = api.synth_config(preset, n_sessions=n, n_queries=nq)
    with tempfile.TemporaryDirectory() as tmp:
        log, part = _oracle_partition(cfg, tmp)
        ds = api.Dataset.parse(str(log), n, 0.2)
    assert ds.n_qd == part["n_qd"]
    for s, st in (("train", ds.train), ("test", ds.test)):
        for k in ("query", "docs", "pidx", "click"):
            assert np.array_equal(getattr(st, k), part[s][k]), (s, k)


def test_from_sessions_equals_parse(native_lib):
    cfg = api.synth_config(1, n_sessions=5000, n_queries=400)
    q, d, m = api.synth_sessions(cfg)
    with tempfile.TemporaryDirectory() as tmp:
        log = Path(tmp) / "log.txt"
        api.write_log(cfg, str(log))
        a = api.Dataset.parse(str(log), cfg.n_sessions, 0.2)
    b = api.Dataset.from_sessions(q, d, m, 0.2)
    assert a.n_qd == b.n_qd
    for s in ("train", "test"):
        for k in ("query", "docs", "pidx", "click"):
            assert np.array_equal(getattr(getattr(a, s), k), getattr(getattr(b, s), k))


def test_split_counts(native_lib):
    """n_train = int(n * (1 - t) - 0.5) + 1 (dataset.cpp:390), float product."""
    cfg = api.synth_config(0, n_sessions=1000, n_queries=1)
    q, d, m = api.synth_sessions(cfg)
    for n, t in [(1000, 0.2), (999, 0.2), (7, 0.5), (1, 0.2), (10, 0.0), (10, 1.0)]:
        ds = api.Dataset.from_sessions(q[:n], d[:n], m[:n], t)
        expect = int(np.float32(n) * (np.float32(1.0) - np.float32(t)) - 0.5) + 1
        assert len(ds.train) == min(expect, n)


def test_sorted_and_contiguous(native_lib):
    cfg = api.synth_config(2, n_sessions=20000, n_queries=2000)
    q, d, m = api.synth_sessions(cfg)
    ds = api.Dataset.from_sessions(q, d, m, 0.2)
    assert np.all(np.diff(ds.train.query) >= 0)
    # qd indices: first appearance order, so each query owns a contiguous range
    lo = {}
    hi = {}
    for qq, p in zip(ds.train.query, ds.train.pidx):
        lo[qq] = min(lo.get(qq, 1 << 30), p.min())
        hi[qq] = max(hi.get(qq, -1), p.max())
    keys = sorted(lo)
    for a, b in zip(keys, keys[1:]):
        assert hi[a] + 1 == lo[b]
    assert ds.n_qd == hi[keys[-1]] + 1


def test_missing_file_is_an_error(native_lib):
    with pytest.raises(_capi.MCError) as e:
        api.Dataset.parse("/nonexistent/path/log.txt", 10, 0.2)
    assert e.value.code == 2


def test_bad_test_share_is_an_error(native_lib):
    with pytest.raises(_capi.MCError):
        api.Dataset.from_sessions(np.zeros(1, np.int32), np.zeros((1, 10), np.int32), np.zeros(1, np.uint16), 1.5)


def test_empty_log(native_lib):
    with tempfile.TemporaryDirectory() as tmp:
        log = Path(tmp) / "empty.txt"
        log.write_text("")
        ds = api.Dataset.parse(str(log), 100, 0.2)
    assert len(ds.train) == 0 and len(ds.test) == 0 and ds.n_qd == 0


def test_max_sessions_limits_reading(native_lib):
    cfg = api.synth_config(0, n_sessions=500, n_queries=50)
    with tempfile.TemporaryDirectory() as tmp:
        log = Path(tmp) / "log.txt"
        api.write_log(cfg, str(log))
        ds = api.Dataset.parse(str(log), 100, 0.2)
    assert len(ds.train) == 80


def _messy_log(seed: int, n_lines: int) -> str:
    """Valid query and click lines mixed with every kind of line the reader
    treats specially: session id -1, wrong token counts, unparsable session
    ids and fields, empty lines, and click lines before the first query."""
    rng = np.random.default_rng(seed)
    lines = [f"{rng.integers(0, 50)} 1 C {rng.integers(0, 5)}" for _ in range(int(rng.integers(0, 3)))]
    sid = 0
    while len(lines) < n_lines:
        u = rng.random()
        if u < 0.55:
            q = int(rng.zipf(1.5)) % 40
            docs = rng.permutation(12)[:10] + q * 10
            s = -1 if rng.random() < 0.05 else sid
            lines.append(f"{s} 0 Q {q} 0 " + " ".join(str(int(d)) for d in docs))
            for k in range(int(rng.integers(0, 3))):
                lines.append(f"{s} {k + 1} C {int(rng.choice(docs)) if rng.random() < 0.9 else 999}")
            sid += 1
        elif u < 0.62:
            lines.append("1 2 3 4 5")                                 # other token count
        elif u < 0.67:
            lines.append("x 0 Q 1 0 1 2 3 4 5 6 7 8 9 10")           # bad session id
        elif u < 0.72:
            lines.append(f"{sid} 0 Q 3 0 1 2 3 4 y 6 7 8 9 10")     # bad doc field
        elif u < 0.76:
            lines.append(f"{sid} 1 C zz")                             # bad click doc
        elif u < 0.80:
            lines.append("")                                          # empty line
        elif u < 0.85:
            lines.append(f"-1 1 C {int(rng.integers(0, 400))}")       # click line with session id -1
        else:
            lines.append(f"{sid} 1 C {int(rng.integers(0, 400))}")   # stray click
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("seed", [1, 2, 3])
@pytest.mark.parametrize("max_sessions", [-1, 0, 1, 37, 400, 100000])
def test_messy_log_matches_oracle_ingest(seed, max_sessions, native_lib, oracle_lib):
    """Runs of lines are replayed on several threads and joined in order; the
    result must be the oracle's line-by-line state machine, whatever mix of
    malformed lines and wherever the session limit falls."""
    from oracle import bindings
    with tempfile.TemporaryDirectory() as tmp:
        log = Path(tmp) / "log.txt"
        log.write_text(_messy_log(seed, 4000))
        ds = api.Dataset.parse(str(log), max_sessions, 0.2)
        part = bindings.parse(str(log), max_sessions, 0.2)
    assert ds.n_qd == part["n_qd"]
    for s, st in (("train", ds.train), ("test", ds.test)):
        for k in ("query", "docs", "pidx", "click"):
            assert np.array_equal(getattr(st, k), part[s][k]), (seed, max_sessions, s, k)


@pytest.fixture
def small_blocks(native_lib):
    """Reads with the given block size and run count, restoring the defaults
    afterwards."""
    def set_(block_bytes: int, runs: int):
        _capi.check(native_lib.mc_ingest_configure(block_bytes, runs))
    yield set_
    _capi.check(native_lib.mc_ingest_configure(0, 0))


@pytest.mark.parametrize("block_bytes,runs", [(40, 1), (333, 3), (4096, 7), (65536, 16)])
@pytest.mark.parametrize("max_sessions", [-1, 37, 400])
def test_messy_log_across_blocks(block_bytes, runs, max_sessions, small_blocks, oracle_lib):
    """Blocks of a few bytes to a few KB put block boundaries inside lines
    (the unfinished line is carried into the next block), lines longer than a
    block (read on until a newline turns up), and sessions open across blocks
    and runs, as a log of several hundred MB does with the default 64 MB
    blocks."""
    from oracle import bindings
    small_blocks(block_bytes, runs)
    with tempfile.TemporaryDirectory() as tmp:
        log = Path(tmp) / "log.txt"
        log.write_text(_messy_log(11, 3000))
        ds = api.Dataset.parse(str(log), max_sessions, 0.2)
        part = bindings.parse(str(log), max_sessions, 0.2)
    assert ds.n_qd == part["n_qd"]
    for s, st in (("train", ds.train), ("test", ds.test)):
        for k in ("query", "docs", "pidx", "click"):
            assert np.array_equal(getattr(st, k), part[s][k]), (block_bytes, runs, max_sessions, s, k)


@pytest.mark.parametrize("name", CASES)
def test_goldens_across_blocks(name, small_blocks):
    """The reference's own partitions, read in 1 KB blocks cut into 5 runs."""
    small_blocks(1024, 5)
    case = load_case(name)
    with tempfile.TemporaryDirectory() as tmp:
        log = Path(tmp) / "log.txt"
        log.write_bytes(case["log"].tobytes())
        ds = api.Dataset.parse(str(log), int(case["max_sessions"]), float(case["test_share"]))
    assert ds.n_qd == int(case["n_qd"])
    for s, st in (("train", ds.train), ("test", ds.test)):
        for k in ("query", "docs", "pidx", "click"):
            assert np.array_equal(getattr(st, k), case[f"{s}_{k}"]), (name, s, k)


def test_log_over_64mb_matches_oracle_ingest(native_lib, oracle_lib):
    """A log larger than one default 64 MB block (about 900k sessions, 80 MB)
    with the default block size and runs, against the oracle's line-by-line
    reader; the session limit falls in the second block."""
    from oracle import bindings
    cfg = api.synth_config(1, n_sessions=900_000, n_queries=50_000)
    with tempfile.TemporaryDirectory() as tmp:
        log = Path(tmp) / "log.txt"
        api.write_log(cfg, str(log))
        assert log.stat().st_size > (64 << 20)
        for limit in (-1, 850_000):
            ds = api.Dataset.parse(str(log), limit, 0.2)
            part = bindings.parse(str(log), limit, 0.2)
            assert ds.n_qd == part["n_qd"]
            for s, st in (("train", ds.train), ("test", ds.test)):
                for k in ("query", "docs", "pidx", "click"):
                    assert np.array_equal(getattr(st, k), part[s][k]), (limit, s, k)
