"""Gradients of a trajectory misfit with respect to log rate constants.

``adjoint_batch`` integrates independent instances on the GPU (mixed form),
recording their step sequences, and runs the discrete adjoint of those exact
step sequences (``lassie_adjoint_batch``) for

    L_q = sum over samples i and sampled species j of (y_ij - target_ij)^2.

``TrajectoryMisfit`` wraps it as a ``torch.autograd.Function``: the forward
takes log k of shape [B, R] and returns the B losses; the backward returns
dL/dlog k.  The reference has no gradient capability; its GUI lists
parameter estimation as planned work and its Python comparator computes a
misfit (``LSODAsim.py:104-121``) without gradients.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _native as nat
from .model import Model
from .solver import NativeModel, _Packed, make_opts


def adjoint_batch(models: Sequence[Model], targets: Sequence[np.ndarray],
                  ckpt_every: int = 8, max_record: int = 0, deadline_s: float = 0.0,
                  root: str = "pow", native: Optional[Sequence[NativeModel]] = None,
                  engine: str = "mixed"):
    """Returns (loss [B], grad_logk [B][R], grad_x0 [B][N], trajectories, stats).

    ``engine`` is the form of the recorded forward integration ("mixed" or
    "fp64"); the backward pass is the same for both."""
    L = nat.load()
    n = len(models)
    cache = {}
    packs = []
    for q, m in enumerate(models):
        if native is not None:
            nm = native[q]
        else:
            nm = cache.get(id(m.left))
            if nm is None:
                nm = cache[id(m.left)] = NativeModel.of(m)
        packs.append(_Packed(m, nm))
    inst = (nat.Instance * max(n, 1))(*[p.instance() for p in packs])
    tg = [np.ascontiguousarray(t, np.float64) for t in targets]
    for p, t in zip(packs, tg):
        if t.shape != p.out.shape:
            raise ValueError(f"target shape {t.shape} != trajectory shape {p.out.shape}")
    gk = [np.zeros(m.n_reactions) for m in models]
    gx = [np.zeros(m.n_species) for m in models]
    loss = np.zeros(n)
    stats = (nat.Stats * max(n, 1))()
    arr = lambda lst: (C.c_void_p * max(n, 1))(*[a.ctypes.data for a in lst])  # noqa: E731
    o = make_opts(models[0] if n else None, engine, 0, deadline_s, root=root)
    rc = L.lassie_adjoint_batch(C.cast(inst, C.c_void_p), n, C.cast(arr(tg), C.c_void_p),
                                C.byref(o), int(ckpt_every), int(max_record),
                                loss.ctypes.data, C.cast(arr(gk), C.c_void_p),
                                C.cast(arr(gx), C.c_void_p), C.cast(stats, C.c_void_p))
    nat.check(rc, "lassie_adjoint_batch")
    return loss, gk, gx, [p.out for p in packs], [stats[q].as_dict() for q in range(n)]


def _torch_function():
    import torch

    class TrajectoryMisfit(torch.autograd.Function):
        """loss[b] = sum (y_b(t_i) - target_b,i)^2 for k_b = exp(log_k[b]); the
        networks, initial states and sampling times come from `models`."""

        @staticmethod
        def forward(ctx, log_k, models, targets, ckpt_every=8):
            lk = log_k.detach().to("cpu", torch.float64).numpy()
            ms = []
            for b, m in enumerate(models):
                mm = Model(left=m.left, right=m.right, k=np.exp(lk[b]), x0=m.x0, t=m.t,
                           cs=m.cs, feed=m.feed, atol=m.atol, rkf_step=m.rkf_step,
                           be_step=m.be_step, newton_iter=m.newton_iter,
                           newton_tol=m.newton_tol, stiffness_tol=m.stiffness_tol)
                ms.append(mm)
            loss, gk, _, _, _ = adjoint_batch(ms, targets, ckpt_every=ckpt_every)
            ctx.save_for_backward(torch.as_tensor(np.stack(gk)))
            return torch.as_tensor(loss, dtype=log_k.dtype, device=log_k.device)

        @staticmethod
        def backward(ctx, grad_loss):
            (g,) = ctx.saved_tensors
            g = g.to(device=grad_loss.device, dtype=grad_loss.dtype)
            return grad_loss[:, None] * g, None, None, None

    return TrajectoryMisfit


def trajectory_misfit(log_k, models: Sequence[Model], targets: Sequence[np.ndarray],
                      ckpt_every: int = 8):
    """Differentiable misfit: ``trajectory_misfit(log_k, models, targets).sum().backward()``."""
    return _torch_function().apply(log_k, list(models), list(targets), ckpt_every)


def fit_rate_constants(models: Sequence[Model], targets: Sequence[np.ndarray],
                       log_k0: Optional[np.ndarray] = None, iters: int = 50, lr: float = 0.05,
                       ckpt_every: int = 8):
    """Parameter estimation (the misfit of LASSIE's LSODA comparator,
    ``LSODAsim.py:104-121``, minimised over log k): Adam on
    sum_b trajectory_misfit(log_k[b]) with the adjoint gradients.  One row
    of log k per model (initial values log_k0, default the models' own).
    Returns (log_k [B, R], loss per iteration)."""
    import torch
    if log_k0 is None:
        log_k0 = np.stack([np.log(m.k) for m in models])
    log_k = torch.tensor(np.asarray(log_k0, np.float64), requires_grad=True)
    opt = torch.optim.Adam([log_k], lr=lr)
    history = []
    for _ in range(iters):
        opt.zero_grad()
        loss = trajectory_misfit(log_k, models, targets, ckpt_every).sum()
        loss.backward()
        opt.step()
        history.append(float(loss.detach()))
    return log_k.detach().numpy(), history
