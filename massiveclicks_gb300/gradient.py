"""Gradient-based DBN training beside EM.

``DBNLogLikelihood`` is a torch autograd Function over the C-ABI pair
``mc_dbn_loglik_forward`` / ``mc_dbn_loglik_backward``: the DBN session
log-likelihood (the reference's conditional click model, dbn.cu:611-639) of a
range of a model's uploaded training sessions as a function of logit
parameters alpha (attractiveness), beta (satisfaction), gamma (continuation).
Its backward pass is the hand-written adjoint kernel.

``train_adam`` fits the logits with torch's Adam on minibatches of sessions.
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
            ll = C.c_double()
            check(_capi.load().mc_dbn_loglik_forward(model._h, int(begin), int(count), _ptr(alpha), _ptr(beta),
                                                     _ptr(gamma), int(bool(fp64)), C.byref(ll), _stream_handle()))
            ctx.save_for_backward(alpha, beta, gamma)
            ctx.model, ctx.begin, ctx.count, ctx.fp64 = model, int(begin), int(count), bool(fp64)
            return torch.tensor(ll.value, dtype=torch.float64, device=alpha.device)

        @staticmethod
        def backward(ctx, grad_out):
            alpha, beta, gamma = ctx.saved_tensors
            da = torch.empty_like(alpha)
            db = torch.empty_like(beta)
            dg = torch.empty_like(gamma)
            check(_capi.load().mc_dbn_loglik_backward(ctx.model._h, ctx.begin, ctx.count, _ptr(alpha), _ptr(beta),
                                                      _ptr(gamma), int(ctx.fp64), float(grad_out), _ptr(da), _ptr(db),
                                                      _ptr(dg), None, _stream_handle()))
            return da, db, dg, None, None, None, None

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


def logits_to_values(alpha, beta, gamma) -> dict:
    import torch
    return {"attractiveness": torch.sigmoid(alpha).detach().cpu().numpy(),
            "satisfaction": torch.sigmoid(beta).detach().cpu().numpy(),
            "continuation": torch.sigmoid(gamma).detach().cpu().numpy()}


def train_adam(model: ClickModel, n_qd: int, steps: int, batch: int = 262144, lr: float = 0.05,
               callback=None, callback_every: int = 0, device: int = 0):
    """Adam on the logits, minibatches of `batch` consecutive sessions of the
    model's (shuffled) training set, loss = -log-likelihood / batch.  The
    callback gets (step, seconds, alpha, beta, gamma) every callback_every steps."""
    import torch
    dev = torch.device("cuda", device)
    alpha = torch.zeros(n_qd, dtype=torch.float32, device=dev, requires_grad=True)
    beta = torch.zeros(n_qd, dtype=torch.float32, device=dev, requires_grad=True)
    gamma = torch.zeros(1, dtype=torch.float32, device=dev, requires_grad=True)
    opt = torch.optim.Adam([alpha, beta, gamma], lr=lr)
    n = model.n_train
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
            torch.cuda.synchronize()
            callback(step + 1, time.perf_counter() - t0, alpha, beta, gamma)
    return alpha, beta, gamma
