"""The C-ABI library loads and exports every entry point that include/*.h
declares; host-only behaviour (synthetic generator, error reporting) without a
GPU."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from conftest import ROOT
from massiveclicks_gb300 import api, _capi, build


def declared_in_headers() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(mc_[a-z0-9_]+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported(native_lib):
    lib = ctypes.CDLL(str(build.LIB))
    missing = [n for n in sorted(declared_in_headers()) if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header():
    assert declared_in_headers() == set(_capi.declared_symbols())


def test_version(native_lib):
    assert native_lib.mc_version().decode().startswith("massiveclicks-gb300")


def test_synth_deterministic_and_chunkable(native_lib):
    cfg = api.synth_config(2, n_sessions=3000, n_queries=500)
    q1, d1, m1 = api.synth_sessions(cfg)
    q2, d2, m2 = api.synth_sessions(cfg)
    assert np.array_equal(q1, q2) and np.array_equal(d1, d2) and np.array_equal(m1, m2)
    qa, da, ma = api.synth_sessions(cfg, 0, 1234)
    qb, db, mb = api.synth_sessions(cfg, 1234, 3000 - 1234)
    assert np.array_equal(np.concatenate([qa, qb]), q1)
    assert np.array_equal(np.concatenate([da, db]), d1)
    assert np.array_equal(np.concatenate([ma, mb]), m1)


def test_synth_shapes(native_lib):
    cfg = api.synth_config(1, n_sessions=20000, n_queries=1000)
    q, d, m = api.synth_sessions(cfg)
    assert q.min() >= 0 and q.max() < 1000
    # shown docs come from the query's pool, all distinct
    assert np.all(d // cfg.pool == q[:, None])
    assert np.all(np.sort(d, axis=1)[:, 1:] != np.sort(d, axis=1)[:, :-1])
    # Zipf: query 0 is the most frequent
    counts = np.bincount(q, minlength=1000)
    assert counts[0] == counts.max()
    # DBN ground truth: some sessions with clicks, some without
    assert 0 < (m == 0).mean() < 1


def test_synth_rejects_bad_config(native_lib):
    cfg = api.synth_config(0, n_sessions=10, n_queries=10, pool=5)
    with pytest.raises(_capi.MCError):
        api.synth_sessions(cfg)


def test_log_roundtrip(native_lib, tmp_path):
    cfg = api.synth_config(0, n_sessions=200, n_queries=20)
    api.write_log(cfg, str(tmp_path / "log.txt"))
    lines = (tmp_path / "log.txt").read_text().splitlines()
    q_lines = [l for l in lines if l.split()[2] == "Q"]
    assert len(q_lines) == 201  # one trailing session for the reader to drop
    assert all(len(l.split()) == 15 for l in q_lines)


def test_model_errors_without_device(native_lib):
    """Invalid arguments are rejected before any CUDA call."""
    h = ctypes.c_void_p()
    assert native_lib.mc_model_create(7, 0, 0, ctypes.byref(h)) == 1
    buf = ctypes.create_string_buffer(256)
    assert native_lib.mc_last_error(buf, 256) == 1
    assert b"model type" in buf.value
    assert native_lib.mc_model_em(None, 1, 0, None) == 1
    assert native_lib.mc_model_param_count(None) == 0


def test_device_cache_entry_points_without_device(native_lib):
    """With nothing cached, the cache queries and release make no CUDA call."""
    b = ctypes.c_int64(-1)
    assert native_lib.mc_cache_bytes(-1, ctypes.byref(b)) == 0 and b.value == 0
    assert native_lib.mc_empty_cache(-1, ctypes.byref(b)) == 0 and b.value == 0
    assert native_lib.mc_empty_cache(0, None) == 0
    assert native_lib.mc_cache_bytes(0, None) == 1  # null output rejected
    h = ctypes.c_int32()
    assert native_lib.mc_model_fused_path(None, ctypes.byref(h), ctypes.byref(b)) == 1
