"""The memory-bounded reversal of adjoint.trajectory_gradient, on the CPU with a stand-in
solver whose step is U <- a U + 1 (elementwise) and whose step VJP is Ubar <- a Ubar: every
step is reversed exactly once, in order, from the right state; the number of trajectory
states alive never exceeds the slot budget (the trajectory start counted, the working state
of the forward pass not); recomputed steps match the plan; the gradient of a windowed
objective J = sum_{n > N - W} w_n . U_n matches the closed form."""
import weakref

import pytest
import torch

from flame3d_mhd_gb300 import adjoint

A = 1.01


class FakeSolver:
    shape3 = (1, 1, 1)
    device = "cpu"

    def __init__(self):
        self.visits = []
        self.live = 0
        self.peak = 0

    def field(self, nvar):
        return torch.zeros((nvar, 1, 1, 1), dtype=torch.float64)

    def q_from_u(self, U, Q):
        return Q

    def time_step(self, U, Un, Q, dt, nsteps):
        for _ in range(nsteps):
            U.mul_(A).add_(1.0)

    def rk3_step_vjp(self, dt, U0, Ubar_next, Ubar, Ustage=None, Lbar_stage=None):
        self.visits.append(float(U0[0, 0, 0, 0]))
        Ubar.copy_(Ubar_next * A)
        return Ubar


def _track(solver):
    """Count the live trajectory states (every copy the reversal makes goes through clone)."""
    orig = adjoint._Reverser.clone

    def clone(self, U):
        V = orig(self, U)
        solver.live += 1
        solver.peak = max(solver.peak, solver.live)

        def gone():
            solver.live -= 1
        weakref.finalize(V, gone)
        return V
    return clone


def _state(n):
    """U_n for U_0 = 0 under U <- A U + 1."""
    return (A ** n - 1.0) / (A - 1.0)


@pytest.mark.parametrize("N,slots", [(1, 2), (7, 2), (9, 3), (40, 5), (100, 8), (60, 61), (50, 2), (333, 12)])
def test_reversal_order_memory_and_plan(N, slots, monkeypatch):
    s = FakeSolver()
    monkeypatch.setattr(adjoint._Reverser, "clone", _track(s))
    U0 = torch.zeros((5, 1, 1, 1), dtype=torch.float64)
    W = max(1, N // 3)
    w = lambda n: 1.0 + 0.1 * n
    src = lambda n, U: torch.full_like(U, w(n)) if n > N - W else None
    UN, g, st = adjoint.trajectory_gradient(s, U0, 0.1, N, slots, final_grad=lambda U: torch.full_like(U, w(N)),
                                            source=src)
    assert float(UN[0, 0, 0, 0]) == pytest.approx(_state(N))
    # step n -> n+1 is reversed from U_n, last step first
    assert s.visits == pytest.approx([_state(n) for n in range(N - 1, -1, -1)])
    # dJ/dU_0 = sum_{n > N-W} w_n A^n
    want = sum(w(n) * A ** n for n in range(N - W + 1, N + 1))
    assert float(g[0, 0, 0, 0]) == pytest.approx(want, rel=1e-12)
    assert st["recomputed_steps"] == st["planned_recomputed_steps"]
    assert s.peak <= slots
    assert s.live == 0


def test_plan_costs():
    # everything fits: nothing recomputed
    assert adjoint.plan(10, 10)["recomputed_steps"] == 0
    # fewer slots never costs less
    c = [adjoint.plan(1000, s)["recomputed_steps"] for s in (64, 30, 20, 10)]
    assert c == sorted(c)
    # about one extra forward pass with sqrt(N) x 2 slots
    assert adjoint.plan(400, 40)["recomputed_steps"] <= 400
