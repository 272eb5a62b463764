"""ORACLE — test infrastructure, not product code.

ctypes bindings of oracle_capi.cpp: the CPU restatement of the reference's
training path (FP32 = bit-exact with the compiled reference at one thread,
FP64 = the oracle the GPU is measured against).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
REF_DRIVER = HERE / "_ref" / "ref_driver"
R = 10

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        import sys
        sys.path.insert(0, str(HERE.parent))
        from massiveclicks_gb300 import build
        build.build_oracle()
    lib = C.CDLL(str(LIB_PATH))
    vp = C.c_void_p
    lib.orc_parse.restype = vp
    lib.orc_parse.argtypes = [C.c_char_p, C.c_int, C.c_float]
    lib.orc_part_info.restype = C.c_int64
    lib.orc_part_info.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    lib.orc_part_copy.argtypes = [vp, C.c_int, vp, vp, vp, vp]
    lib.orc_part_free.argtypes = [vp]
    lib.orc_fit_new.restype = vp
    lib.orc_fit_new.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int64, vp, vp, vp, C.c_int64]
    lib.orc_fit_run.argtypes = [vp, C.c_int, C.c_int]
    lib.orc_fit_set_copies.argtypes = [vp, C.c_int]
    lib.orc_fit_n_params.restype = C.c_int64
    lib.orc_fit_n_params.argtypes = [vp]
    lib.orc_fit_get.argtypes = [vp, vp, vp, vp]
    lib.orc_fit_set_values.argtypes = [vp, vp]
    lib.orc_fit_eval.argtypes = [vp, C.c_int64, vp, vp, vp, vp, vp, vp]
    lib.orc_fit_free.argtypes = [vp]
    lib.orc_dbn_loglik.restype = C.c_double
    lib.orc_dbn_loglik.argtypes = [C.c_int64, vp, vp, vp, vp, C.c_double]
    lib.orc_dbn_fisher.argtypes = [C.c_int64, vp, vp, vp, vp, C.c_double, vp, vp, vp]
    _lib = lib
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def parse(path: str, max_sessions: int, test_share: float):
    """The oracle's own ingest: dict of train/test arrays and n_qd."""
    lib = load()
    h = lib.orc_parse(str(path).encode(), int(max_sessions), float(test_share))
    if not h:
        raise FileNotFoundError(path)
    nt, ns = C.c_int64(), C.c_int64()
    nqd = lib.orc_part_info(h, C.byref(nt), C.byref(ns))
    out = {"n_qd": int(nqd)}
    for which, name, n in ((0, "train", nt.value), (1, "test", ns.value)):
        q = np.empty(n, np.int32)
        d = np.empty((n, R), np.int32)
        p = np.empty((n, R), np.int32)
        m = np.empty(n, np.uint16)
        lib.orc_part_copy(h, which, _p(q), _p(d), _p(p), _p(m))
        out[name] = {"query": q, "docs": d, "pidx": p, "click": m}
    lib.orc_part_free(h)
    return out


def param_sizes(model: int, n_qd: int) -> list[tuple[str, int]]:
    """Parameter arrays in get_parameters(ALL) order."""
    if model == 0:
        return [("examination", R), ("attractiveness", n_qd)]
    if model == 3:
        return [("examination", R * (R - 1) // 2 + R), ("attractiveness", n_qd)]
    if model == 2:
        return [("attractiveness", n_qd), ("satisfaction", n_qd), ("continuation", 1)]
    return [("attractiveness", n_qd), ("continuation", 3)]


class OracleFit:
    """One CPU fit.  dtype 'f32' reproduces the reference exactly (1 thread);
    'f64' is the FP64 oracle."""

    def __init__(self, dtype: str, model: int, mode: int, query, pidx, click_mask, n_qd: int):
        self.lib = load()
        self.model = model
        self.n_qd = int(n_qd)
        self._q = np.ascontiguousarray(query, np.int32)
        self._p = np.ascontiguousarray(pidx, np.int32).reshape(-1)
        self._m = np.ascontiguousarray(click_mask, np.uint16)
        self.h = self.lib.orc_fit_new(0 if dtype == "f32" else 1, model, mode, self._q.shape[0], _p(self._q),
                                      _p(self._p), _p(self._m), self.n_qd)

    def run(self, iterations: int, threads: int = 1, copy_sessions: bool = True) -> None:
        """copy_sessions=False skips the reference's per-thread dataset copies
        of DBN/CCM (same results, less time and memory)."""
        self.lib.orc_fit_set_copies(self.h, int(bool(copy_sessions)))
        self.lib.orc_fit_run(self.h, int(iterations), int(threads))

    def flat(self):
        k = self.lib.orc_fit_n_params(self.h)
        num, den, val = np.empty(k), np.empty(k), np.empty(k)
        self.lib.orc_fit_get(self.h, _p(num), _p(den), _p(val))
        return num, den, val

    def values(self) -> dict[str, np.ndarray]:
        _, _, val = self.flat()
        out, off = {}, 0
        for name, size in param_sizes(self.model, self.n_qd):
            out[name] = val[off:off + size]
            off += size
        return out

    def set_values(self, values: dict[str, np.ndarray]) -> None:
        flat = np.concatenate([np.asarray(values[name], np.float64) for name, _ in param_sizes(self.model, self.n_qd)])
        self.lib.orc_fit_set_values(self.h, _p(flat))

    def evaluate(self, pidx, click_mask) -> dict:
        p = np.ascontiguousarray(pidx, np.int32).reshape(-1)
        m = np.ascontiguousarray(click_mask, np.uint16)
        ls, llh, ppl = C.c_double(), C.c_double(), C.c_double()
        l2 = np.zeros(R)
        self.lib.orc_fit_eval(self.h, m.shape[0], _p(p), _p(m), C.byref(ls), _p(l2), C.byref(llh), C.byref(ppl))
        return {"llh_sum": ls.value, "log2_sums": l2, "llh": llh.value, "ppl": ppl.value, "n": int(m.shape[0])}

    def __del__(self):
        try:
            if self.h:
                self.lib.orc_fit_free(self.h)
                self.h = None
        except Exception:
            pass


def dbn_loglik(pidx, click_mask, alpha, beta, gamma: float) -> float:
    """FP64 DBN log-likelihood (conditional model of the reference) of sessions."""
    p = np.ascontiguousarray(pidx, np.int32).reshape(-1)
    m = np.ascontiguousarray(click_mask, np.uint16)
    a = np.ascontiguousarray(alpha, np.float64)
    b = np.ascontiguousarray(beta, np.float64)
    return load().orc_dbn_loglik(m.shape[0], _p(p), _p(m), _p(a), _p(b), float(gamma))


def dbn_fisher(pidx, click_mask, alpha, beta, gamma: float):
    """Expected complete-data scores under the exact DBN posterior (Fisher identity)."""
    p = np.ascontiguousarray(pidx, np.int32).reshape(-1)
    m = np.ascontiguousarray(click_mask, np.uint16)
    a = np.ascontiguousarray(alpha, np.float64)
    b = np.ascontiguousarray(beta, np.float64)
    sa = np.zeros_like(a)
    sb = np.zeros_like(b)
    sg = C.c_double(0.0)
    load().orc_dbn_fisher(m.shape[0], _p(p), _p(m), _p(a), _p(b), float(gamma), _p(sa), _p(sb), C.byref(sg))
    return sa, sb, sg.value
