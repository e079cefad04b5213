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

import functools
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


# ---- memory-bounded reversal -----------------------------------------------------------
# A segment [a, b) whose start state U_a is held is reversed with `s` further states: if its
# b - a - 1 intermediate states fit, they are recomputed once and held; with a single state
# each U_n is recomputed from U_a in place (quadratic cost); otherwise c checkpoints are
# placed evenly, and the sub-segments are reversed from the last, the i-th (i = 0 starts at
# U_a) with s - i states (its own start and the checkpoints before it stay held). `plan`
# picks the cheapest option by recomputed steps; the forward pass places the top level for
# free. `slots` counts the trajectory states held at once, U_0's copy included; U_N, the
# cotangent and the step scratch come on top.

INF = float("inf")


@functools.lru_cache(maxsize=None)
def _segment_cost(n: int, s: int) -> tuple[float, int]:
    """(recomputed steps, checkpoints placed; -1 = recompute from the start) to reverse n
    steps from a held start with s further states."""
    if n <= 1:
        return 0, 0
    if n - 1 <= s:
        return n - 1, 0
    if s <= 0:
        return INF, 0
    best = (n * (n - 1) // 2, -1)
    for c in range(1, min(s, n - 1) + 1):
        bounds = _split(n, c)
        cost = bounds[-2]  # steps run to place the last checkpoint
        for i in range(c + 1):
            cost += _segment_cost(bounds[i + 1] - bounds[i], s - i)[0]
        if cost < best[0]:
            best = (cost, c)
    return best


def _split(n: int, c: int) -> list[int]:
    """0 = b_0 < b_1 < ... < b_c < b_{c+1} = n, near-even lengths."""
    return [round(i * n / (c + 1)) for i in range(c + 2)]


def plan(nsteps: int, slots: int) -> dict:
    """Top-level checkpoint count and the recomputed steps of the backward pass for nsteps
    steps with `slots` (>= 2) trajectory states held at a time."""
    if slots < 2:
        raise ValueError("the reversal needs at least two states (the start and a working state)")
    s = slots - 1
    if nsteps - 1 <= s:
        return {"top": max(nsteps - 1, 0), "recomputed_steps": 0, "slots": slots}
    best = (_segment_cost(nsteps, s)[0] if s >= 1 else INF, 0)  # no top-level checkpoints
    for c in range(1, min(s, nsteps - 1) + 1):
        bounds = _split(nsteps, c)
        cost = sum(_segment_cost(bounds[i + 1] - bounds[i], s - i)[0] for i in range(c + 1))
        if cost < best[0]:
            best = (cost, c)
    return {"top": best[1], "recomputed_steps": best[0], "slots": slots}


class _Reverser:
    def __init__(self, solver: Flame3D, dt: float, source, stage_sink):
        self.s, self.dt, self.source, self.stage_sink = solver, dt, source, stage_sink
        self.Un, self.Q, self.tmp = solver.field(5), solver.field(6), solver.field(5)
        self.Ust = self.Lbt = None
        if stage_sink is not None:
            self.Ust = torch.zeros((3, 5, *solver.shape3), dtype=torch.float64, device=solver.device)
            self.Lbt = torch.zeros_like(self.Ust)
        self.recomputed = 0

    def clone(self, U: torch.Tensor) -> torch.Tensor:
        return U.clone()

    def advance(self, V: torch.Tensor, k: int):
        _advance(self.s, V, self.dt, k, self.Un, self.Q)
        self.recomputed += k

    def visit(self, n: int, Un_state: torch.Tensor, Ubar: torch.Tensor):
        """Ubar: cotangent of U_{n+1} -> cotangent of U_n (plus the source at n)."""
        self.s.rk3_step_vjp(self.dt, Un_state, Ubar, self.tmp, self.Ust, self.Lbt)
        Ubar.copy_(self.tmp)
        if self.stage_sink is not None:
            self.stage_sink(n, self.Ust, self.Lbt)
        if self.source is not None:
            g = self.source(n, Un_state)
            if g is not None:
                Ubar.add_(g)

    def segment(self, Ua: torch.Tensor, a: int, b: int, s: int, Ubar: torch.Tensor):
        n = b - a
        if n <= 1:
            self.visit(a, Ua, Ubar)
            return
        cost, c = _segment_cost(n, s)
        if cost == INF:
            raise RuntimeError("no state left for the reversal")
        if n - 1 <= s:
            states = [Ua]
            for _ in range(n - 1):
                V = self.clone(states[-1])
                self.advance(V, 1)
                states.append(V)
            del V  # only the list holds the states, so popping frees them
            for idx in range(n - 1, -1, -1):
                self.visit(a + idx, states[idx], Ubar)
                states.pop()
            return
        if c < 0:  # one working state, each U_n recomputed from the start
            for idx in range(n - 1, 0, -1):
                V = self.clone(Ua)
                self.advance(V, idx)
                self.visit(a + idx, V, Ubar)
                del V
            self.visit(a, Ua, Ubar)
            return
        bounds = _split(n, c)
        held = [Ua]
        for i in range(1, c + 1):
            V = self.clone(held[-1])
            self.advance(V, bounds[i] - bounds[i - 1])
            held.append(V)
        del V
        for i in range(c, -1, -1):
            self.segment(held[i], a + bounds[i], a + bounds[i + 1], s - i, Ubar)
            held.pop()


def trajectory_gradient(solver: Flame3D, U0: torch.Tensor, dt: float, nsteps: int, slots: int, final_grad=None,
                        source=None, observe=None, stage_sink=None) -> tuple[torch.Tensor, torch.Tensor, dict]:
    """Gradient of an objective over the states U_0 .. U_N of N SSP-RK3 steps, holding at
    most `slots` (>= 2) states of the trajectory at a time (U_0's copy included; U_N, the
    cotangent and the step scratch come on top).

    observe(n, U_n) sees every state of the forward pass (to evaluate the objective);
    final_grad(U_N) returns dJ/dU_N and source(n, U_n) the explicit dJ/dU_n of the earlier
    states (None: no dependence); stage_sink(n, Ustage, Lbar_stage) receives, for each step
    n -> n + 1, its three stage states and the cotangents of their RHS values (to form the
    gradient with respect to parameters of the RHS). Inflow-profile cotangents accumulate in
    the buffers set with solver.set_inflow_profile_cotangent. Returns (U_N, dJ/dU_0, stats)."""
    p = plan(nsteps, slots)
    bounds = _split(nsteps, p["top"])
    r = _Reverser(solver, dt, source, stage_sink)
    U = U0.clone()
    Un, Q = solver.field(5), solver.field(6)
    held = [r.clone(U0)]
    if observe is not None:
        observe(0, U)
    n = 0
    for i in range(1, len(bounds)):
        while n < bounds[i]:
            _advance(solver, U, dt, 1, Un, Q)
            n += 1
            if observe is not None:
                observe(n, U)
        if i < len(bounds) - 1:
            held.append(r.clone(U))
    Ubar = final_grad(U) if final_grad is not None else torch.zeros_like(U)
    Ubar = Ubar.clone()
    s = slots - 1
    for i in range(len(held) - 1, -1, -1):
        r.segment(held[i], bounds[i], bounds[i + 1], s - i, Ubar)
        held.pop()
    return U, Ubar, {"top_checkpoints": len(bounds) - 2, "recomputed_steps": r.recomputed,
                     "planned_recomputed_steps": p["recomputed_steps"], "slots": slots}
