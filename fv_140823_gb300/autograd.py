"""torch.autograd wrappers of the residual and of fixed-dt RK steps.

Forward passes run the FP64 CUDA path of a :class:`~fv_140823_gb300.solver.Solver`;
backward passes run its hand-written reverse kernels (``fvgpu_residual_vjp``,
``fvgpu_adjoint_steps``).  Tensors are float64 ``[neq, ncells]`` on any
device; they cross the C ABI as host arrays.  The solver's state is
overwritten by every call.

    from fv_140823_gb300.autograd import residual, steps
    U = torch.tensor(U0, dtype=torch.float64, requires_grad=True)
    J = (steps(solver, U, dt, "ssprk3", 10)[0] ** 2).sum()
    J.backward()          # U.grad = dJ/dU0 through 10 SSP-RK3 steps

Derivatives are those of the branch the forward takes (minmod limiter,
wave-speed maxima, HLLC region); ``dt`` is held constant.
"""
from __future__ import annotations

import numpy as np
import torch


def _host(t: torch.Tensor) -> np.ndarray:
    return np.ascontiguousarray(t.detach().to("cpu", torch.float64).numpy())


class ResidualFunction(torch.autograd.Function):
    """R(U) of residual_faces_AMR.c (with faceinterp.c for MUSCL)."""

    @staticmethod
    def forward(ctx, U: torch.Tensor, solver) -> torch.Tensor:
        Uh = _host(U)
        R = solver.residual(Uh)
        ctx.solver = solver
        ctx.U = Uh
        return torch.from_numpy(R).to(U.device)

    @staticmethod
    def backward(ctx, gR: torch.Tensor):
        solver = ctx.solver
        solver.set_state(ctx.U)
        g = solver.residual_vjp(_host(gR))
        return torch.from_numpy(g).to(gR.device), None


class StepsFunction(torch.autograd.Function):
    """nsteps RK steps (RK.c) at the fixed time step dt."""

    @staticmethod
    def forward(ctx, U: torch.Tensor, solver, dt: float, scheme: str, nsteps: int) -> torch.Tensor:
        Uh = _host(U)
        solver.set_state(Uh)
        solver.step(scheme, dt=dt, nsteps=nsteps)
        S = solver.state()
        ctx.solver, ctx.U, ctx.dt, ctx.scheme, ctx.nsteps = solver, Uh, float(dt), scheme, int(nsteps)
        return torch.from_numpy(S).to(U.device)

    @staticmethod
    def backward(ctx, gS: torch.Tensor):
        solver = ctx.solver
        solver.set_state(ctx.U)
        g = solver.adjoint_steps(_host(gS), ctx.dt, ctx.scheme, ctx.nsteps)
        return torch.from_numpy(g).to(gS.device), None, None, None, None


def residual(solver, U: torch.Tensor) -> torch.Tensor:
    return ResidualFunction.apply(U, solver)


def steps(solver, U: torch.Tensor, dt: float, scheme: str = "ssprk3", nsteps: int = 1) -> torch.Tensor:
    return StepsFunction.apply(U, solver, dt, scheme, nsteps)
