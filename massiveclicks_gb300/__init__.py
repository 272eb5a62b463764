"""GB300-native EM trainer for web-search click models (PBM, UBM, CCM, DBN).

The hot path (one EM iteration over all training sessions) is hand-written
sm_103a CUDA behind the C-ABI in include/mclicks.h; this package holds the
in-tree build, the ctypes bindings and a Python mirror of the reference's host
API.
"""
from ._capi import CCM, DBN, IMPL_FUSED, IMPL_PLAIN, MAX_SERP, MODE_CLEAN, MODE_PARITY, PBM, UBM, MCError, load
from .api import (CCMModel, ClickModel, Dataset, DBNModel, Evaluation, PBMModel, SessionSet, UBMModel,
                  clicks_to_mask, em_parallel, mask_to_clicks, synth_config, synth_sessions, write_log)

__all__ = [
    "PBM", "CCM", "DBN", "UBM", "MODE_PARITY", "MODE_CLEAN", "IMPL_FUSED", "IMPL_PLAIN", "MAX_SERP",
    "MCError", "load", "ClickModel", "PBMModel", "CCMModel", "DBNModel", "UBMModel", "Dataset", "SessionSet",
    "Evaluation", "em_parallel", "synth_config", "synth_sessions", "write_log", "clicks_to_mask",
    "mask_to_clicks",
]
