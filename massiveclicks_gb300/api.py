"""Python host API over the C-ABI.

Names follow the reference's host API (click_models/base.cuh:30-53,
data/dataset.h, parallel_em/parallel_em.cuh:39-42): a ``Dataset`` is the
partition that ``Dataset::parse_dataset`` produces, a ``ClickModel`` (with the
``PBM``/``CCM``/``DBN``/``UBM`` subclasses) owns its device buffers, and
``em_parallel`` runs the EM loop and the evaluation.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _capi
from ._capi import DBN, CCM, IMPL_FUSED, IMPL_PLAIN, MAX_SERP, MODE_CLEAN, MODE_PARITY, PBM, UBM, check

R = MAX_SERP


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _stream(stream) -> C.c_void_p:
    if stream is None:
        return C.c_void_p(0)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    handle = getattr(stream, "cuda_stream", None)  # a torch.cuda.Stream
    if handle is not None:
        return C.c_void_p(handle)
    raise TypeError(f"unsupported stream object {stream!r}")


# ---------------------------------------------------------------------------
# Synthetic sessions
# ---------------------------------------------------------------------------
def synth_config(preset: int = 0, **overrides) -> _capi.SynthConfig:
    cfg = _capi.SynthConfig()
    _capi.load().mc_synth_config_default(C.byref(cfg), preset)
    for k, v in overrides.items():
        if not hasattr(cfg, k):
            raise AttributeError(k)
        setattr(cfg, k, v)
    return cfg


def synth_sessions(cfg: _capi.SynthConfig, first: int = 0, count: int | None = None):
    """Sessions in arrival order: (query[n], docs[n, 10], click_mask[n])."""
    n = cfg.n_sessions - first if count is None else count
    q = np.empty(n, np.int32)
    d = np.empty((n, R), np.int32)
    m = np.empty(n, np.uint16)
    check(_capi.load().mc_synth_generate(C.byref(cfg), first, n, _ptr(q), _ptr(d), _ptr(m)))
    return q, d, m


def write_log(cfg: _capi.SynthConfig, path: str) -> None:
    check(_capi.load().mc_synth_write_log(C.byref(cfg), str(path).encode()))


def clicks_to_mask(clicks: np.ndarray) -> np.ndarray:
    """(n, 10) 0/1 array -> uint16 bit mask (bit r = rank r)."""
    c = np.asarray(clicks).astype(np.uint16).reshape(-1, R)
    return (c << np.arange(R, dtype=np.uint16)).sum(axis=1).astype(np.uint16)


def mask_to_clicks(mask: np.ndarray) -> np.ndarray:
    m = np.asarray(mask, dtype=np.uint16).reshape(-1, 1)
    return ((m >> np.arange(R, dtype=np.uint16)) & 1).astype(np.uint8)


# ---------------------------------------------------------------------------
# Dataset (Dataset::parse_dataset for one worker)
# ---------------------------------------------------------------------------
@dataclass
class SessionSet:
    query: np.ndarray   # int32 [n]
    docs: np.ndarray    # int32 [n, 10]
    pidx: np.ndarray    # int32 [n, 10]; -1 for a test doc unseen in training
    click: np.ndarray   # uint16 [n] bit masks

    def __len__(self) -> int:
        return int(self.query.shape[0])


class Dataset:
    """A (train, test, n_qd) partition, like the reference's ``Partition``
    tuple (utils/types.h:26-30)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle
        lib = _capi.load()
        nt, ns, nq = C.c_int64(), C.c_int64(), C.c_int64()
        check(lib.mc_dataset_info(self._h, C.byref(nt), C.byref(ns), C.byref(nq)))
        self.n_qd = int(nq.value)
        self.train = self._copy(0, int(nt.value))
        self.test = self._copy(1, int(ns.value))

    def _copy(self, which: int, n: int) -> SessionSet:
        s = SessionSet(np.empty(n, np.int32), np.empty((n, R), np.int32), np.empty((n, R), np.int32),
                       np.empty(n, np.uint16))
        check(_capi.load().mc_dataset_copy(self._h, which, _ptr(s.query), _ptr(s.docs), _ptr(s.pidx), _ptr(s.click)))
        return s

    @classmethod
    def parse(cls, path: str, max_sessions: int = 40000, test_share: float = 0.2) -> "Dataset":
        h = C.c_void_p()
        check(_capi.load().mc_dataset_parse(str(path).encode(), int(max_sessions), float(test_share), C.byref(h)))
        return cls(h)

    @classmethod
    def from_sessions(cls, query, docs, click_mask, test_share: float = 0.2) -> "Dataset":
        q = np.ascontiguousarray(query, np.int32)
        d = np.ascontiguousarray(docs, np.int32)
        m = np.ascontiguousarray(click_mask, np.uint16)
        h = C.c_void_p()
        check(_capi.load().mc_dataset_from_sessions(q.shape[0], _ptr(q), _ptr(d), _ptr(m), float(test_share), C.byref(h)))
        return cls(h)

    def close(self) -> None:
        if self._h:
            _capi.load().mc_dataset_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Click models
# ---------------------------------------------------------------------------
@dataclass
class Evaluation:
    llh: float                 # mean over sessions of (sum_r log p_r) / 10
    perplexity: float          # mean over ranks of 2^(-sum log2 q_r / n)
    rank_perplexity: list      # per rank
    n_sessions: int
    llh_sum: float
    log2_sums: np.ndarray


class ClickModel:
    """A click model fit on one GPU (ClickModel_Hst, click_models/base.cuh:30-53)."""

    model_type = PBM

    def __init__(self, mode: int = MODE_PARITY, device: int = 0, model_type: int | None = None):
        if model_type is not None:
            self.model_type = model_type
        self.mode = mode
        self._h = C.c_void_p()
        check(_capi.load().mc_model_create(self.model_type, mode, device, C.byref(self._h)))
        self.n_train = 0
        self.n_qd = 0

    @staticmethod
    def create(model_type: int, mode: int = MODE_PARITY, device: int = 0) -> "ClickModel":
        """create_cm_host (click_models/base.cu:19-49)."""
        cls = {PBM: PBMModel, CCM: CCMModel, DBN: DBNModel, UBM: UBMModel}.get(model_type)
        if cls is None:
            raise ValueError(f"unknown model type {model_type}")
        return cls(mode=mode, device=device)

    # -- data -----------------------------------------------------------------
    def upload(self, train: SessionSet, n_qd: int, stream=None) -> None:
        q = np.ascontiguousarray(train.query, np.int32)
        p = np.ascontiguousarray(train.pidx, np.int32)
        m = np.ascontiguousarray(train.click, np.uint16)
        check(_capi.load().mc_model_upload(self._h, q.shape[0], _ptr(q), _ptr(p), _ptr(m), int(n_qd), _stream(stream)))
        self.n_train = int(q.shape[0])
        self.n_qd = int(n_qd)

    def upload_test(self, test: SessionSet, stream=None) -> None:
        p = np.ascontiguousarray(test.pidx, np.int32)
        m = np.ascontiguousarray(test.click, np.uint16)
        check(_capi.load().mc_model_upload_test(self._h, p.shape[0], _ptr(p), _ptr(m), _stream(stream)))

    def init_parameters(self, dataset: Dataset, stream=None) -> None:
        """init_parameters + the dataset upload (common.cu:31-61, search.cu:342-356)."""
        self.upload(dataset.train, dataset.n_qd, stream)
        self.upload_test(dataset.test, stream)

    def reset_to_prior(self, stream=None) -> None:
        """Every parameter back to 1/2, iteration counter to 0."""
        check(_capi.load().mc_model_init_parameters(self._h, _stream(stream)))

    # -- tiling / tuning ----------------------------------------------------------
    def configure(self, sessions_per_tile: int = 0, window_qd: int = 0, block_size: int = 0) -> None:
        check(_capi.load().mc_model_configure(self._h, sessions_per_tile, window_qd, block_size))

    def get_config(self) -> tuple[int, int, int]:
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        check(_capi.load().mc_model_get_config(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def autotune(self, stream=None) -> tuple[int, int, int]:
        check(_capi.load().mc_model_autotune(self._h, _stream(stream)))
        return self.get_config()

    # -- EM -------------------------------------------------------------------------
    def configure_counts(self, copies: int, block: int, blocks_per_sm: int) -> None:
        """Launch shape of the count-path kernels (PBM, UBM)."""
        check(_capi.load().mc_model_configure_counts(self._h, int(copies), int(block), int(blocks_per_sm)))

    def count_config(self) -> tuple[int, int, int]:
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        check(_capi.load().mc_model_get_count_config(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def em(self, iterations: int, impl: int = IMPL_FUSED, stream=None) -> None:
        check(_capi.load().mc_model_em(self._h, int(iterations), int(impl), _stream(stream)))

    def em_trace(self, iterations: int, stream=None) -> np.ndarray:
        """Fused iterations with the training log-likelihood (per session, as
        evaluate(0).llh) after each one, computed on the device."""
        out = np.zeros(max(int(iterations), 0), np.float64)  # a negative count is the library's to reject
        check(_capi.load().mc_model_em_trace(self._h, int(iterations), _ptr(out), _stream(stream)))
        return out / max(self.n_train, 1)

    def process_session(self, stream=None) -> None:
        check(_capi.load().mc_model_process_sessions(self._h, _stream(stream)))

    def update_parameters(self, stream=None) -> None:
        check(_capi.load().mc_model_update_parameters(self._h, _stream(stream)))

    # -- parameters -----------------------------------------------------------------
    def parameter_information(self) -> list[tuple[str, int, bool]]:
        lib = _capi.load()
        out = []
        for i in range(lib.mc_model_param_count(self._h)):
            name = C.create_string_buffer(64)
            size = C.c_int64()
            pub = C.c_int()
            check(lib.mc_model_param_info(self._h, i, name, 64, C.byref(size), C.byref(pub)))
            out.append((name.value.decode(), int(size.value), bool(pub.value)))
        return out

    def get_parameters(self, stream=None) -> dict[str, np.ndarray]:
        """All parameter values in get_parameters(ALL) order (FP32)."""
        out = {}
        for i, (name, size, _) in enumerate(self.parameter_information()):
            v = np.empty(size, np.float32)
            check(_capi.load().mc_model_get_param(self._h, i, _ptr(v), _stream(stream)))
            out[name] = v
        return out

    def set_parameters(self, values: dict[str, np.ndarray], stream=None) -> None:
        for i, (name, size, _) in enumerate(self.parameter_information()):
            if name in values:
                v = np.ascontiguousarray(values[name], np.float32)
                if v.shape[0] != size:
                    raise ValueError(f"{name}: expected {size} values, got {v.shape[0]}")
                check(_capi.load().mc_model_set_param(self._h, i, _ptr(v), _stream(stream)))

    def flat_parameters(self, stream=None) -> np.ndarray:
        return np.concatenate(list(self.get_parameters(stream).values()))

    # -- evaluation -----------------------------------------------------------------
    def evaluate(self, which: int = 1, stream=None) -> Evaluation:
        """LogLikelihood / Perplexity (click_models/evaluation.cpp:25-66) on the GPU."""
        ll = C.c_double()
        l2 = np.zeros(R, np.float64)
        n = C.c_int64()
        check(_capi.load().mc_model_evaluate(self._h, which, C.byref(ll), _ptr(l2), C.byref(n), _stream(stream)))
        nn = int(n.value)
        if nn == 0:
            return Evaluation(float("nan"), float("nan"), [float("nan")] * R, 0, 0.0, l2)
        rank_ppl = [2.0 ** (-l2[r] / nn) for r in range(R)]
        return Evaluation(ll.value / nn, sum(rank_ppl) / R, rank_ppl, nn, ll.value, l2)

    def fused_path(self) -> tuple:
        """("tiles", 0) when a fused iteration runs the tile kernel over the
        sessions, ("counts", n_entries) when it runs the count kernel over the
        per-(qd, key) occurrence counts (UBM), ("dense", n_entries) for the PBM
        kernel over dense per-rank counts."""
        p, n = C.c_int32(), C.c_int64()
        check(_capi.load().mc_model_fused_path(self._h, C.byref(p), C.byref(n)))
        return ({0: "tiles", 1: "counts", 2: "dense"}[p.value], int(n.value))

    def memory(self) -> int:
        b = C.c_int64()
        check(_capi.load().mc_model_memory(self._h, C.byref(b)))
        return int(b.value)

    def destroy_parameters(self) -> None:
        if self._h:
            _capi.load().mc_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy_parameters()
        except Exception:
            pass


class PBMModel(ClickModel):
    model_type = PBM


class CCMModel(ClickModel):
    model_type = CCM


class DBNModel(ClickModel):
    model_type = DBN


class UBMModel(ClickModel):
    model_type = UBM


class Batch:
    """Several fits advanced together, one persistent launch per iteration."""

    def __init__(self, models: list):
        self.models = list(models)
        arr = (C.c_void_p * len(self.models))(*[m._h.value for m in self.models])
        self._h = C.c_void_p()
        check(_capi.load().mc_batch_create(len(self.models), C.cast(arr, C.c_void_p), C.byref(self._h)))

    def em(self, iterations: int, stream=None) -> None:
        check(_capi.load().mc_batch_em(self._h, int(iterations), _stream(stream)))

    def info(self) -> tuple[int, int, bool]:
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        check(_capi.load().mc_batch_info(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, bool(c.value)

    def configure(self, single_launch: bool) -> None:
        """single_launch: the tile launch takes the count fits' chunks too."""
        check(_capi.load().mc_batch_configure(self._h, int(bool(single_launch))))

    def launches_per_iteration(self) -> int:
        n = C.c_int32()
        check(_capi.load().mc_batch_launches(self._h, C.byref(n)))
        return n.value

    def close(self) -> None:
        if self._h:
            _capi.load().mc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def empty_cache(device: int = -1) -> int:
    """Frees the device blocks the library keeps for reuse (one device, or all
    with -1) and returns the bytes released."""
    b = C.c_int64()
    check(_capi.load().mc_empty_cache(int(device), C.byref(b)))
    return int(b.value)


def cache_bytes(device: int = -1) -> int:
    """Bytes of freed device blocks the library keeps for reuse."""
    b = C.c_int64()
    check(_capi.load().mc_cache_bytes(int(device), C.byref(b)))
    return int(b.value)


def em_parallel(model_type: int, dataset: Dataset, iterations: int = 50, mode: int = MODE_PARITY,
                impl: int = IMPL_FUSED, device: int = 0) -> tuple[ClickModel, Evaluation]:
    """em_parallel (parallel_em/parallel_em.cu:349-746) for one GPU: upload,
    `iterations` EM iterations, test-set evaluation."""
    cm = ClickModel.create(model_type, mode=mode, device=device)
    cm.init_parameters(dataset)
    cm.em(iterations, impl)
    ev = cm.evaluate(1)
    return cm, ev


def rank_perplexity_mean(log2_sums: np.ndarray, n: int) -> float:
    return sum(2.0 ** (-float(v) / n) for v in log2_sums) / R if n else math.nan
