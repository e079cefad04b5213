"""Gradients through SSP-RK3 trajectories: sqrt(N) checkpointing over f3d_rk3_step_vjp.

The forward pass stores the conserved state U every `every` steps (default ceil(sqrt(N))).
The backward pass walks the segments from the last to the first: it recomputes the states
of one segment from its checkpoint, keeps them, and applies the step VJP to each state in
reverse order. Memory: about N/every checkpoints plus `every` segment states; compute:
one extra forward pass plus, per step, two recomputed RHS and three RHS VJPs.

`RK3Rollout` wraps this as a torch.autograd.Function (the counterpart of a ChainRulesCore
rrule on the Julia side): U_N = RK3Rollout.apply(U0, solver, dt, nsteps).
"""
from __future__ import annotations

import math

import torch

from .solver import Flame3D


def _advance(solver: Flame3D, U: torch.Tensor, dt: float, steps: int, Un: torch.Tensor, Q: torch.Tensor):
    """U <- `steps` RK3 steps of U in place (Q recomputed from U first)."""
    if steps <= 0:
        return
    solver.q_from_u(U, Q)
    solver.time_step(U, Un, Q, dt, steps)


def forward_with_checkpoints(solver: Flame3D, U0: torch.Tensor, dt: float, nsteps: int, every: int | None = None):
    """(U_N, {step: U_step}) with checkpoints at steps 0, every, 2 every, ..."""
    every = every or max(1, math.ceil(math.sqrt(nsteps)))
    U = U0.clone()
    Un, Q = solver.field(5), solver.field(6)
    ckpt = {0: U0.clone()}
    done = 0
    while done < nsteps:
        k = min(every, nsteps - done)
        _advance(solver, U, dt, k, Un, Q)
        done += k
        if done < nsteps:
            ckpt[done] = U.clone()
    return U, ckpt, every


def backward_from_checkpoints(solver: Flame3D, ckpt: dict, every: int, dt: float, nsteps: int,
                              Ubar_final: torch.Tensor) -> torch.Tensor:
    """Cotangent of U0 from the cotangent of U_N, recomputing one segment at a time."""
    Ubar = Ubar_final.clone()
    tmp = solver.field(5)
    Un, Q = solver.field(5), solver.field(6)
    starts = sorted(ckpt)
    for s0 in reversed(starts):
        s1 = min(s0 + every, nsteps)
        states = [ckpt[s0].clone()]
        for _ in range(s0, s1 - 1):
            U = states[-1].clone()
            _advance(solver, U, dt, 1, Un, Q)
            states.append(U)
        for U in reversed(states):
            solver.rk3_step_vjp(dt, U, Ubar, tmp)
            Ubar, tmp = tmp, Ubar
    return Ubar


def gradient(solver: Flame3D, U0: torch.Tensor, dt: float, nsteps: int, loss_grad, every: int | None = None):
    """(U_N, dJ/dU0) for J = loss(U_N); loss_grad(U_N) returns dJ/dU_N."""
    UN, ckpt, every = forward_with_checkpoints(solver, U0, dt, nsteps, every)
    return UN, backward_from_checkpoints(solver, ckpt, every, dt, nsteps, loss_grad(UN))


class RK3Rollout(torch.autograd.Function):
    """U_N = RK3Rollout.apply(U0, solver, dt, nsteps, every): differentiable in U0."""

    @staticmethod
    def forward(ctx, U0, solver, dt, nsteps, every=None):
        UN, ckpt, ev = forward_with_checkpoints(solver, U0.detach(), dt, nsteps, every)
        ctx.solver, ctx.ckpt, ctx.every, ctx.dt, ctx.nsteps = solver, ckpt, ev, dt, nsteps
        return UN

    @staticmethod
    def backward(ctx, grad_out):
        g = backward_from_checkpoints(ctx.solver, ctx.ckpt, ctx.every, ctx.dt, ctx.nsteps,
                                      grad_out.contiguous())
        return g, None, None, None, None
