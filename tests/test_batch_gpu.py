"""Batched fits (mc_batch_*): several independent fits of mixed model types in
one persistent launch per iteration must give each fit the result it gets
alone, and match the FP64 oracle."""
import numpy as np
import pytest

from conftest import load_case
from massiveclicks_gb300 import api
from oracle import bindings

pytestmark = pytest.mark.gpu

PARAM_RTOL = 1e-5
PARAM_ATOL = 1e-6


def _sset(case, which):
    return api.SessionSet(case[f"{which}_query"], case[f"{which}_docs"], case[f"{which}_pidx"], case[f"{which}_click"])


def _parts():
    """(model type, train SessionSet, n_qd) for a mix of fixtures and synthetic partitions."""
    out = []
    for name, model in [("pbm_pbmclicks", 0), ("ubm_dbnclicks", 3), ("dbn_dbnclicks", 2), ("ccm_ccmclicks", 1),
                        ("edge", 2), ("dbn_ccmclicks", 0)]:
        c = load_case(name)
        out.append((model, _sset(c, "train"), int(c["n_qd"])))
    for k, (n, model) in enumerate([(30000, 2), (5000, 3), (120000, 0)]):
        cfg = api.synth_config(1, n_sessions=n, n_queries=max(50, n // 40), seed=777 + k)
        q, d, m = api.synth_sessions(cfg)
        ds = api.Dataset.from_sessions(q, d, m, 0.2)
        out.append((model, ds.train, ds.n_qd))
    return out


def _close(a, b, rtol, atol, what):
    for k in b:
        err = np.abs(a[k].astype(np.float64) - b[k])
        assert np.all(err <= rtol * np.abs(b[k]) + atol), f"{what} {k}: max err {err.max():.3g}"


@pytest.mark.parametrize("config", [None, (64, 96, 128)])
def test_batch_equals_separate_fits(config):
    parts = _parts()
    batch_models, single_models = [], []
    for model, train, n_qd in parts:
        for target in (batch_models, single_models):
            cm = api.ClickModel.create(model)
            cm.upload(train, n_qd)
            if config and target is batch_models and not batch_models:
                cm.configure(*config)
            if config and target is single_models:
                cm.configure(*config)
            target.append(cm)
    b = api.Batch(batch_models)
    n_models, n_tiles, mixed = b.info()
    assert n_models == len(parts) and mixed and n_tiles > 0
    b.em(7)
    for cm in single_models:
        cm.em(7)
    for (model, train, n_qd), bm, sm in zip(parts, batch_models, single_models):
        got, alone = bm.get_parameters(), sm.get_parameters()
        # Shared-memory FP32 bins are summed in a run-dependent order, so two
        # runs of the same fit differ by a few ulp per iteration (~1e-6 after
        # 7 iterations); statistics lost or mixed between fits would show as
        # errors of 1e-3 and more.
        _close(got, {k: v.astype(np.float64) for k, v in alone.items()}, 5e-6, 1e-6, f"batch vs alone m{model}")
        f = bindings.OracleFit("f64", model, 0, train.query, train.pidx, train.click, n_qd)
        f.run(7)
        _close(got, f.values(), PARAM_RTOL, PARAM_ATOL, f"batch vs oracle m{model}")
    # continuing alone after the batch keeps working
    batch_models[0].em(1)
    b.close()


def test_batch_rejects_models_without_sessions():
    cm = api.ClickModel.create(0)
    with pytest.raises(api._capi.MCError):
        api.Batch([cm])


def _fit_all(parts):
    models = []
    for model, train, n_qd in parts:
        cm = api.ClickModel.create(model)
        cm.upload(train, n_qd)
        models.append(cm)
    return models


def test_count_path_fits_batch_without_tiles():
    """PBM and UBM fits take the batched count launch and build no tiles."""
    parts = []
    for name, model in [("pbm_pbmclicks", 0), ("ubm_dbnclicks", 3), ("dbn_ccmclicks", 0)]:
        c = load_case(name)
        parts.append((model, _sset(c, "train"), int(c["n_qd"])))
    cfg = api.synth_config(1, n_sessions=40000, n_queries=1000, seed=4242)
    q, d, m = api.synth_sessions(cfg)
    ds = api.Dataset.from_sessions(q, d, m, 0.0)
    parts.append((3, ds.train, ds.n_qd))
    models = _fit_all(parts)
    b = api.Batch(models)
    n_models, n_tiles, mixed = b.info()
    assert (n_models, n_tiles, mixed) == (len(parts), 0, 0)
    assert b.launches_per_iteration() == 1
    b.em(6)
    for (model, train, n_qd), cm in zip(parts, models):
        f = bindings.OracleFit("f64", model, 0, train.query, train.pidx, train.click, n_qd)
        f.run(6)
        _close(cm.get_parameters(), f.values(), PARAM_RTOL, PARAM_ATOL, f"count batch m{model}")
    b.close()


@pytest.mark.parametrize("single_launch", [False, True])
def test_batch_of_both_paths_runs_the_specialised_tile_kernel(single_launch):
    """DBN tile fits next to PBM/UBM count fits: the tile launch holds DBN
    only; its count chunks go to a count launch after it, or (single_launch)
    to the tile launch itself after its tiles."""
    parts = []
    for name, model in [("dbn_dbnclicks", 2), ("pbm_pbmclicks", 0), ("ubm_dbnclicks", 3), ("edge", 2)]:
        c = load_case(name)
        parts.append((model, _sset(c, "train"), int(c["n_qd"])))
    models = _fit_all(parts)
    b = api.Batch(models)
    n_models, n_tiles, mixed = b.info()
    assert n_models == len(parts) and n_tiles > 0 and not mixed
    assert b.launches_per_iteration() == 2
    b.configure(single_launch)
    assert b.launches_per_iteration() == (1 if single_launch else 2)
    b.em(5)
    for (model, train, n_qd), cm in zip(parts, models):
        f = bindings.OracleFit("f64", model, 0, train.query, train.pidx, train.click, n_qd)
        f.run(5)
        _close(cm.get_parameters(), f.values(), PARAM_RTOL, PARAM_ATOL, f"two-path batch m{model}")
    b.close()
