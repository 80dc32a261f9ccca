"""Differentiable direct-sum KDK integration with a hand-written adjoint.

``simulate(x0, v0, m, G=..., softening=..., dt=..., nsteps=...)`` returns the
final positions and velocities of ``nsteps`` KDK leapfrog steps
(core/engine.py:108-116 with direct forces, core/solvers/gravity.py:13-26),
as a ``torch.autograd.Function``: the backward pass is the hand-written
reverse-mode step of the CUDA library (``gb_adjoint_step``), not torch
autograd.  Memory: the forward pass keeps the state every
``checkpoint_every`` steps; the backward pass re-runs each segment forward
from its checkpoint (the same kernels and tile shapes, so bit-identical
positions) and walks it in reverse.
"""
from __future__ import annotations

import torch

from . import _lib
from ._dev import ptr, require_cuda, stream_handle
from .solvers.gravity import DirectGravity


class KDKConfig:
    def __init__(self, G, softening, dt, nsteps, checkpoint_every, solver):
        self.G = float(G)
        self.eps2 = float(softening) ** 2
        self.dt = float(dt)
        self.nsteps = int(nsteps)
        self.every = max(1, int(checkpoint_every))
        self.solver = solver


def _pack(x, v, m):
    n = x.shape[0]
    xm = torch.empty((n, 4), dtype=torch.float32, device=x.device)
    xm[:, :3] = x.detach().float()
    xm[:, 3] = m.detach().float()
    v4 = torch.zeros((n, 4), dtype=torch.float32, device=x.device)
    v4[:, :3] = v.detach().float()
    return xm, v4


def _segments(nsteps, every):
    return [(c, min(every, nsteps - c)) for c in range(0, nsteps, every)]


class DirectKDK(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, m, cfg: KDKConfig):
        xm, v4 = _pack(x0, v0, m)
        a4 = torch.zeros_like(xm)
        s = cfg.solver
        s.acc(xm, a4, cfg.G, cfg.eps2)
        ckpts = []
        for c, length in _segments(cfg.nsteps, cfg.every):
            ckpts.append((xm.clone(), v4.clone(), a4.clone()))
            s.kdk(xm, v4, a4, cfg.G, cfg.eps2, cfg.dt, length)
        ctx.cfg = cfg
        ctx.ckpts = ckpts
        ctx.x_final = xm.clone()
        return xm[:, :3].clone(), v4[:, :3].clone()

    @staticmethod
    def backward(ctx, gx, gv):
        cfg, s = ctx.cfg, ctx.cfg.solver
        x0m = ctx.ckpts[0][0]
        n, dev = x0m.shape[0], x0m.device
        lx = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        lv = torch.zeros_like(lx)
        la = torch.zeros_like(lx)
        lm = torch.zeros(n, dtype=torch.float32, device=dev)
        if gx is not None:
            lx[:, :3] = gx.float()
        if gv is not None:
            lv[:, :3] = gv.float()
        stream = stream_handle(dev)
        segs = _segments(cfg.nsteps, cfg.every)
        traj = torch.empty((cfg.every, n, 4), dtype=torch.float32, device=dev)
        ends = [ck[0] for ck in ctx.ckpts[1:]] + [ctx.x_final]
        for (c, length), (xm, v4, a4), x_end in zip(reversed(segs), reversed(ctx.ckpts), reversed(ends)):
            xm, v4, a4 = xm.clone(), v4.clone(), a4.clone()
            for k in range(length - 1):
                s.kdk(xm, v4, a4, cfg.G, cfg.eps2, cfg.dt, 1)
                traj[k].copy_(xm)
            for k in reversed(range(length)):
                xk = x_end if k == length - 1 else traj[k]
                _lib.call("gb_adjoint_step", s.handle, ptr(xk, "xm"), ptr(lx, "lx"), ptr(lv, "lv"),
                          ptr(la, "la"), lm.data_ptr(), n, cfg.G, cfg.eps2, cfg.dt, 0, stream)
        _lib.call("gb_adjoint_step", s.handle, ptr(x0m, "xm"), ptr(lx, "lx"), ptr(lv, "lv"),
                  ptr(la, "la"), lm.data_ptr(), n, cfg.G, cfg.eps2, cfg.dt, 1, stream)
        return lx[:, :3].clone(), lv[:, :3].clone(), lm, None


def simulate(x0: torch.Tensor, v0: torch.Tensor, m: torch.Tensor, *, G: float, softening: float,
             dt: float, nsteps: int, checkpoint_every: int = 20, solver: DirectGravity | None = None,
             symmetric: bool = True, packed: bool = True):
    """(x_T, v_T) after nsteps KDK steps; differentiable in x0, v0 and m.
    symmetric selects the adjoint's pair evaluation (each unordered pair once,
    or each ordered pair in one pass per target); packed selects, for the
    symmetric form, FP32x2 arithmetic with dynamically fetched tile-pair
    units over the scalar form with static CTA runs.  The forward steps (and
    the backward's segment re-runs) use solver's force pass: a new solver
    runs the per-target pass; one with set_variant(2) the symmetric pass,
    about 20% faster forward steps at N = 65,536."""
    require_cuda(x0.device)
    if solver is None:
        solver = DirectGravity(x0.shape[0], x0.device)
    _lib.call("gb_adjoint_set_variant", solver.handle, (2 if packed else 1) if symmetric else 0)
    cfg = KDKConfig(G, softening, dt, nsteps, checkpoint_every, solver)
    return DirectKDK.apply(x0, v0, m, cfg)
