"""torch.autograd wrappers of the residual and of fixed-dt RK steps.

Forward passes run the FP64 CUDA path of a :class:`~fv_140823_gb300.solver.Solver`;
backward passes run its hand-written reverse kernels (``fvgpu_residual_vjp``,
``fvgpu_adjoint_steps``).  Tensors are float64 ``[neq, ncells]``.  CUDA
tensors cross the C ABI as device pointers (the library copies device to
device on its stream; no host round trip); CPU tensors cross it as host
arrays.  The solver's state is overwritten by every call.

    from fv_140823_gb300.autograd import residual, steps
    U = torch.tensor(U0, dtype=torch.float64, device="cuda", requires_grad=True)
    J = (steps(solver, U, dt, "ssprk3", 10)[0] ** 2).sum()
    J.backward()          # U.grad = dJ/dU0 through 10 SSP-RK3 steps

Derivatives are those of the branch the forward takes (minmod limiter,
wave-speed maxima, HLLC region); ``dt`` is held constant.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import abi


def _host(t: torch.Tensor) -> np.ndarray:
    return np.ascontiguousarray(t.detach().to("cpu", torch.float64).numpy())


def _dev(t: torch.Tensor) -> torch.Tensor:
    """Contiguous float64 copy-or-view on the tensor's device, complete
    before the library's stream reads it."""
    d = t.detach().to(torch.float64).contiguous()
    torch.cuda.synchronize(d.device)
    return d


def _set_state_dev(solver, U: torch.Tensor) -> None:
    solver._call("fvgpu_upload_state", C.c_void_p(U.data_ptr()), C.c_int64(solver.n))


def _residual_dev(solver, U: torch.Tensor) -> torch.Tensor:
    _set_state_dev(solver, U)
    if solver.cfg.ischeme == 2:
        solver.faceinterp()
    if solver.cfg.ns == 1:
        solver.gradcalc()
    solver.rhs()
    R = torch.empty_like(U)
    solver._call("fvgpu_download", int(abi.FIELD_RHS), C.c_void_p(R.data_ptr()))
    solver.synchronize()
    return R


class ResidualFunction(torch.autograd.Function):
    """R(U) of residual_faces_AMR.c (with faceinterp.c for MUSCL)."""

    @staticmethod
    def forward(ctx, U: torch.Tensor, solver) -> torch.Tensor:
        ctx.solver = solver
        if U.is_cuda:
            Ud = _dev(U)
            ctx.U = Ud
            return _residual_dev(solver, Ud)
        Uh = _host(U)
        R = solver.residual(Uh)
        ctx.U = Uh
        return torch.from_numpy(R).to(U.device)

    @staticmethod
    def backward(ctx, gR: torch.Tensor):
        solver = ctx.solver
        if isinstance(ctx.U, torch.Tensor):
            w = _dev(gR)
            _set_state_dev(solver, ctx.U)
            g = torch.empty_like(w)
            solver.residual_vjp_device(w.data_ptr(), g.data_ptr())
            solver.synchronize()
            return g, None
        solver.set_state(ctx.U)
        g = solver.residual_vjp(_host(gR))
        return torch.from_numpy(g).to(gR.device), None


class StepsFunction(torch.autograd.Function):
    """nsteps RK steps (RK.c) at the fixed time step dt."""

    @staticmethod
    def forward(ctx, U: torch.Tensor, solver, dt: float, scheme: str, nsteps: int) -> torch.Tensor:
        ctx.solver, ctx.dt, ctx.scheme, ctx.nsteps = solver, float(dt), scheme, int(nsteps)
        if U.is_cuda:
            Ud = _dev(U)
            ctx.U = Ud
            _set_state_dev(solver, Ud)
            solver.step(scheme, dt=dt, nsteps=nsteps)
            S = torch.empty_like(Ud)
            solver._call("fvgpu_download_state", C.c_void_p(S.data_ptr()), C.c_int64(solver.n))
            solver.synchronize()
            return S
        Uh = _host(U)
        solver.set_state(Uh)
        solver.step(scheme, dt=dt, nsteps=nsteps)
        ctx.U = Uh
        return torch.from_numpy(solver.state()).to(U.device)

    @staticmethod
    def backward(ctx, gS: torch.Tensor):
        solver = ctx.solver
        sc = abi.SCHEMES[ctx.scheme]
        if isinstance(ctx.U, torch.Tensor):
            g = _dev(gS).clone()
            _set_state_dev(solver, ctx.U)
            solver._call("fvgpu_adjoint_steps", sc, ctx.dt, ctx.nsteps, C.c_void_p(g.data_ptr()),
                         C.c_void_p(g.data_ptr()), C.c_int64(solver.n))
            solver.synchronize()
            return g, None, None, None, None
        solver.set_state(ctx.U)
        g = solver.adjoint_steps(_host(gS), ctx.dt, ctx.scheme, ctx.nsteps)
        return torch.from_numpy(g).to(gS.device), None, None, None, None


def residual(solver, U: torch.Tensor) -> torch.Tensor:
    return ResidualFunction.apply(U, solver)


def steps(solver, U: torch.Tensor, dt: float, scheme: str = "ssprk3", nsteps: int = 1) -> torch.Tensor:
    return StepsFunction.apply(U, solver, dt, scheme, nsteps)
