"""The timeout path of the fused kernel, reached without a fault: every wait
inside the kernel is bounded, and an expired wait is reported to the host.

A testing hook shortens the wait limit to 1 ms and makes the stage fill of
one tile declare 16 bytes more than it copies, so that the wait for that stage
never completes although every copy lands (no copy is left in flight when the
CTA leaves).  The fit must then report MC_ERR_DEVICE with a timeout message,
the GPU context must stay usable, and a fresh model must run and match the
FP64 oracle.  The reference stops the job on such an error
(communicator.cpp:119-133); here the host sees a status code."""
import numpy as np
import pytest

from conftest import load_case
from massiveclicks_gb300 import api, _capi
from oracle import bindings

pytestmark = pytest.mark.gpu


def _fit(case, iters):
    cm = api.ClickModel.create(api.DBN)
    cm.upload(api.SessionSet(case["train_query"], case["train_docs"], case["train_pidx"], case["train_click"]),
              int(case["n_qd"]))
    cm.configure(64, 256, 256)  # several tiles, so tile 0 is one of many
    cm.em(iters)
    return cm


@pytest.mark.parametrize("stall_tile", [0, 3])
def test_stalled_stage_times_out_and_the_device_stays_usable(stall_tile):
    lib = _capi.load()
    case = load_case("dbn_dbnclicks")
    _capi.check(lib.mc_test_wait_hooks(0, 1_000_000, stall_tile))
    try:
        with pytest.raises(_capi.MCError) as e:
            cm = _fit(case, 2)
            cm.get_parameters()
        assert e.value.code == 6
        assert "timed out" in str(e.value)
    finally:
        _capi.check(lib.mc_test_wait_hooks(0, 0, -1))
    cm = _fit(case, 5)
    got = cm.get_parameters()
    f = bindings.OracleFit("f64", api.DBN, 0, case["train_query"], case["train_pidx"], case["train_click"],
                           int(case["n_qd"]))
    f.run(5)
    for name, ref in f.values().items():
        err = np.abs(got[name].astype(np.float64) - ref)
        assert np.all(err <= 1e-5 * np.abs(ref) + 1e-6), name


def test_hook_arguments_are_checked():
    lib = _capi.load()
    assert lib.mc_test_wait_hooks(0, -1, -1) == 1
    assert lib.mc_test_wait_hooks(0, 0, -2) == 1
