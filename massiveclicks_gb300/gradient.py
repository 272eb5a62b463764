"""Gradient-based DBN training beside EM.

``DBNLogLikelihood`` is a torch autograd Function over the C-ABI: the DBN
session log-likelihood (the reference's conditional click model,
dbn.cu:611-639) of a range of a model's uploaded training sessions as a
function of logit parameters alpha (attractiveness), beta (satisfaction),
gamma (continuation).  When a gradient is wanted, the forward pass runs the
hand-written adjoint kernel once (``mc_dbn_loglik_grad``: log-likelihood and
gradient, no host round trip) and the backward pass scales the stored
gradient; otherwise it runs ``mc_dbn_loglik_forward``.

``train_adam`` fits the logits with torch's Adam on minibatches of sessions.
``query_order`` lays sessions out in a random order of whole queries, so that
consecutive ranges are random sets of queries (unbiased minibatches) while
each query's sessions stay together (the adjoint's tile path).
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _capi
from .api import ClickModel, SessionSet, check


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def _stream_handle():
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _function():
    import torch

    class DBNLogLikelihood(torch.autograd.Function):
        """log-likelihood = f(alpha, beta, gamma) over sessions [begin, begin + count)."""

        @staticmethod
        def forward(ctx, alpha, beta, gamma, model: ClickModel, begin: int, count: int, fp64: bool = False):
            for t in (alpha, beta, gamma):
                if t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous():
                    raise TypeError("alpha, beta and gamma must be contiguous float32 CUDA tensors")
            lib = _capi.load()
            if any(ctx.needs_input_grad[:3]):
                ll = torch.empty((), dtype=torch.float64, device=alpha.device)
                da = torch.empty_like(alpha)
                db = torch.empty_like(beta)
                dg = torch.empty_like(gamma)
                check(lib.mc_dbn_loglik_grad(model._h, int(begin), int(count), _ptr(alpha), _ptr(beta), _ptr(gamma),
                                             int(bool(fp64)), _ptr(da), _ptr(db), _ptr(dg), _ptr(ll),
                                             _stream_handle()))
                ctx.save_for_backward(da, db, dg)
                return ll
            ll = C.c_double()
            check(lib.mc_dbn_loglik_forward(model._h, int(begin), int(count), _ptr(alpha), _ptr(beta), _ptr(gamma),
                                            int(bool(fp64)), C.byref(ll), _stream_handle()))
            return torch.tensor(ll.value, dtype=torch.float64, device=alpha.device)

        @staticmethod
        def backward(ctx, grad_out):
            da, db, dg = ctx.saved_tensors
            w = grad_out.to(torch.float32)
            return da * w, db * w, dg * w, None, None, None, None

    return DBNLogLikelihood


_FN = None


def dbn_loglik(alpha, beta, gamma, model: ClickModel, begin: int = 0, count: int | None = None, fp64: bool = False):
    """Differentiable DBN log-likelihood of the model's training sessions."""
    global _FN
    if _FN is None:
        _FN = _function()
    if count is None:
        count = model.n_train - begin
    return _FN.apply(alpha, beta, gamma, model, begin, count, fp64)


def shuffled_sessions(train: SessionSet, seed: int = 0) -> SessionSet:
    """The training sessions in a random order (for unbiased minibatches)."""
    perm = np.random.default_rng(seed).permutation(len(train))
    return SessionSet(train.query[perm], train.docs[perm], train.pidx[perm], train.click[perm])


def query_order(train: SessionSet, seed: int = 0):
    """The training sessions grouped by query, the queries in a random order,
    with query-document indices renumbered in that order (the layout ingest
    gives sessions sorted by query).  Returns (sessions, n_qd, to_original):
    to_original[i] is the original index of renumbered pair i."""
    from .api import Dataset
    q = np.ascontiguousarray(train.query, np.int64)
    uq, inv = np.unique(q, return_inverse=True)
    perm = np.random.default_rng(seed).permutation(len(uq))
    relabel = perm[inv].astype(np.int32)       # a random rank for every query
    ds = Dataset.from_sessions(relabel, train.docs, train.click, 0.0)
    # pair key (query, doc) -> original index, looked up for the new indices
    orig_q = uq[np.argsort(perm)][ds.train.query.astype(np.int64)]
    key_new = (orig_q[:, None] << 32) | ds.train.docs.astype(np.int64)
    key_old = (q[:, None] << 32) | train.docs.astype(np.int64)
    ko, first = np.unique(key_old.ravel(), return_index=True)
    old_idx = train.pidx.ravel()[first]
    pos = np.searchsorted(ko, key_new.ravel())
    to_original = np.empty(ds.n_qd, np.int64)
    to_original[ds.train.pidx.ravel()] = old_idx[pos]
    return ds.train, ds.n_qd, to_original


def logits_to_values(alpha, beta, gamma) -> dict:
    import torch
    return {"attractiveness": torch.sigmoid(alpha).detach().cpu().numpy(),
            "satisfaction": torch.sigmoid(beta).detach().cpu().numpy(),
            "continuation": torch.sigmoid(gamma).detach().cpu().numpy()}


def train_adam(model: ClickModel, n_qd: int, steps: int, batch: int = 262144, lr: float = 0.05,
               callback=None, callback_every: int = 0, device: int = 0):
    """Adam on the logits, minibatches of `batch` consecutive sessions of the
    model's training set (lay it out with query_order or shuffle it for
    unbiased batches), loss = -log-likelihood / batch.  Every callback_every
    steps the device is synchronised and callback(step, seconds, alpha, beta,
    gamma) runs; `seconds` is the training time so far, and the callback's own
    time is not counted.  No step waits for the host otherwise."""
    import torch
    dev = torch.device("cuda", device)
    alpha = torch.zeros(n_qd, dtype=torch.float32, device=dev, requires_grad=True)
    beta = torch.zeros(n_qd, dtype=torch.float32, device=dev, requires_grad=True)
    gamma = torch.zeros(1, dtype=torch.float32, device=dev, requires_grad=True)
    opt = torch.optim.Adam([alpha, beta, gamma], lr=lr, fused=True)  # one kernel per step for all three
    n = model.n_train
    torch.cuda.synchronize(dev)
    elapsed = 0.0
    t0 = time.perf_counter()
    begin = 0
    for step in range(steps):
        count = min(batch, n - begin)
        loss = -dbn_loglik(alpha, beta, gamma, model, begin, count) / count
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
        begin = begin + count if begin + count < n else 0
        if callback and callback_every and (step + 1) % callback_every == 0:
            torch.cuda.synchronize(dev)
            elapsed += time.perf_counter() - t0
            callback(step + 1, elapsed, alpha, beta, gamma)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
    return alpha, beta, gamma
