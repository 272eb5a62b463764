"""ctypes bindings of include/mclicks.h (libmclicks.so).

The library is loaded from the in-tree build directory; a missing library is an
error, never a fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

MAX_SERP = 10
PBM, CCM, DBN, UBM = 0, 1, 2, 3
MODEL_NAMES = {PBM: "PBM", CCM: "CCM", DBN: "DBN", UBM: "UBM"}
MODE_PARITY, MODE_CLEAN = 0, 1
IMPL_FUSED, IMPL_PLAIN = 0, 1

_VP = C.c_void_p
_I32, _I64, _F32, _F64 = C.c_int32, C.c_int64, C.c_float, C.c_double


class SynthConfig(C.Structure):
    _fields_ = [
        ("n_sessions", C.c_int64), ("n_queries", C.c_int32), ("pool", C.c_int32), ("zipf_s", C.c_double),
        ("click_model", C.c_int32), ("reserved", C.c_int32), ("atr_beta_b", C.c_double),
        ("sat_beta_b", C.c_double), ("gamma", C.c_double), ("tau1", C.c_double), ("tau2", C.c_double),
        ("tau3", C.c_double), ("pbm_exam_scale", C.c_double), ("seed", C.c_uint64),
    ]


# name -> (restype, argtypes)
_SIGS = {
    "mc_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "mc_version": (C.c_char_p, []),
    "mc_synth_config_default": (None, [C.POINTER(SynthConfig), C.c_int]),
    "mc_synth_generate": (C.c_int, [C.POINTER(SynthConfig), _I64, _I64, _VP, _VP, _VP]),
    "mc_synth_write_log": (C.c_int, [C.POINTER(SynthConfig), C.c_char_p]),
    "mc_dataset_parse": (C.c_int, [C.c_char_p, _I32, _F32, C.POINTER(_VP)]),
    "mc_ingest_configure": (C.c_int, [_I64, _I32]),
    "mc_dataset_from_sessions": (C.c_int, [_I64, _VP, _VP, _VP, _F32, C.POINTER(_VP)]),
    "mc_dataset_info": (C.c_int, [_VP, C.POINTER(_I64), C.POINTER(_I64), C.POINTER(_I64)]),
    "mc_dataset_copy": (C.c_int, [_VP, C.c_int, _VP, _VP, _VP, _VP]),
    "mc_dataset_free": (None, [_VP]),
    "mc_model_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(_VP)]),
    "mc_model_upload": (C.c_int, [_VP, _I64, _VP, _VP, _VP, _I64, _VP]),
    "mc_model_upload_test": (C.c_int, [_VP, _I64, _VP, _VP, _VP]),
    "mc_model_init_parameters": (C.c_int, [_VP, _VP]),
    "mc_model_configure": (C.c_int, [_VP, _I32, _I32, _I32]),
    "mc_model_get_config": (C.c_int, [_VP, C.POINTER(_I32), C.POINTER(_I32), C.POINTER(_I32)]),
    "mc_model_autotune": (C.c_int, [_VP, _VP]),
    "mc_model_configure_counts": (C.c_int, [_VP, _I32, _I32, _I32]),
    "mc_model_get_count_config": (C.c_int, [_VP, C.POINTER(_I32), C.POINTER(_I32), C.POINTER(_I32)]),
    "mc_model_em": (C.c_int, [_VP, _I32, C.c_int, _VP]),
    "mc_model_process_sessions": (C.c_int, [_VP, _VP]),
    "mc_model_update_parameters": (C.c_int, [_VP, _VP]),
    "mc_model_param_count": (C.c_int, [_VP]),
    "mc_model_param_info": (C.c_int, [_VP, C.c_int, C.c_char_p, C.c_size_t, C.POINTER(_I64), C.POINTER(C.c_int)]),
    "mc_model_get_param": (C.c_int, [_VP, C.c_int, _VP, _VP]),
    "mc_model_set_param": (C.c_int, [_VP, C.c_int, _VP, _VP]),
    "mc_model_evaluate": (C.c_int, [_VP, C.c_int, C.POINTER(_F64), _VP, C.POINTER(_I64), _VP]),
    "mc_model_em_trace": (C.c_int, [_VP, C.c_int32, _VP, _VP]),
    "mc_model_fused_path": (C.c_int, [_VP, C.POINTER(C.c_int32), C.POINTER(_I64)]),
    "mc_model_memory": (C.c_int, [_VP, C.POINTER(_I64)]),
    "mc_test_wait_hooks": (C.c_int, [C.c_int, _I64, _I32]),
    "mc_empty_cache": (C.c_int, [C.c_int, C.POINTER(_I64)]),
    "mc_cache_bytes": (C.c_int, [C.c_int, C.POINTER(_I64)]),
    "mc_model_destroy": (None, [_VP]),
    "mc_batch_create": (C.c_int, [C.c_int, _VP, C.POINTER(_VP)]),
    "mc_batch_em": (C.c_int, [_VP, _I32, _VP]),
    "mc_batch_info": (C.c_int, [_VP, C.POINTER(_I32), C.POINTER(_I32), C.POINTER(_I32)]),
    "mc_batch_launches": (C.c_int, [_VP, C.POINTER(_I32)]),
    "mc_batch_configure": (C.c_int, [_VP, C.c_int]),
    "mc_batch_destroy": (None, [_VP]),
    "mc_dbn_loglik_forward": (C.c_int, [_VP, _I64, _I64, _VP, _VP, _VP, C.c_int, C.POINTER(_F64), _VP]),
    "mc_dbn_loglik_backward": (C.c_int, [_VP, _I64, _I64, _VP, _VP, _VP, C.c_int, _F64, _VP, _VP, _VP,
                                         C.POINTER(_F64), _VP]),
    "mc_dbn_loglik_grad": (C.c_int, [_VP, _I64, _I64, _VP, _VP, _VP, C.c_int, _VP, _VP, _VP, _VP, _VP]),
    "mc_evaluate_static": (C.c_int, [C.c_int, _I64, _VP, _VP, _I64, _VP, _VP, _VP, C.POINTER(_F64), _VP, _VP]),
}

_lib: C.CDLL | None = None


class MCError(RuntimeError):
    """A non-zero status from the native library."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"mclicks error {code}: {msg}")
        self.code = code


def lib_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads libmclicks.so (building it first if it is missing) and declares
    every exported entry point."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if build_if_missing:
        _build.build_library()  # no-op when the sources are unchanged
    elif not path.exists():
        raise FileNotFoundError(f"{path} is not built")
    lib = C.CDLL(str(path))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != 0:
        buf = C.create_string_buffer(1024)
        code = load().mc_last_error(buf, len(buf))
        raise MCError(rc if rc else code, buf.value.decode(errors="replace"))


def declared_symbols() -> list[str]:
    return list(_SIGS)
