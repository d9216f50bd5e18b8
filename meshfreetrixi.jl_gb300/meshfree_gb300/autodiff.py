"""Reverse-mode differentiation of rhs! and of SSP-RK3 solves as torch.autograd
Functions: the Python counterpart of ChainRulesCore rrules for rhs! and solve().

MeshfreeTrixi.jl itself differentiates rhs! only through ForwardDiff.jl duals; here the
pullbacks are the engine's hand-written adjoint (mft_rhs_adjoint*, mft_ssprk33_adjoint*):
a transpose-stencil gather over the reverse adjacency fused with the flux-Jacobian-
transpose products, and a checkpointed reverse sweep over the SSP-RK3 stages.

Tensors are (nvars, n) float64 CUDA tensors (the StructArray layout, SoA).  The engine
runs on its own CUDA stream and returns synchronised, so each call first waits for the
producer stream of its inputs.
"""
import numpy as np
import torch


def _ctx_of(semi):
    return semi.domain.ctx


def _ready(t):
    if not (t.is_cuda and t.dtype == torch.float64):
        raise TypeError("expected a float64 CUDA tensor")
    torch.cuda.synchronize(t.device)
    return t.contiguous()


class RHS(torch.autograd.Function):
    """du = rhs!(u, t) with pullback lam -> (d rhs!/du)^T lam.  u is not mutated (the
    strong-BC pass works on a copy)."""

    @staticmethod
    def forward(ctx, u, semi, t=0.0):
        u = _ready(u.detach())
        uu = u.clone()
        du = torch.empty_like(uu)
        torch.cuda.synchronize(u.device)
        _ctx_of(semi).rhs_device(du.data_ptr(), uu.data_ptr(), t)
        ctx.save_for_backward(u)
        ctx.semi, ctx.t = semi, t
        return du

    @staticmethod
    def backward(ctx, g):
        (u,) = ctx.saved_tensors
        g = _ready(g)
        out = torch.empty_like(g)
        _ctx_of(ctx.semi).rhs_adjoint_device(out.data_ptr(), g.data_ptr(), u.data_ptr(), ctx.t)
        return out, None, None


class SSPRK33Solve(torch.autograd.Function):
    """u(T) after nsteps SSP-RK3 steps of size dt from u0 at t0, recorded with a
    checkpoint every `every` steps (0: every stage state kept).  The pullback is the
    engine's reverse sweep with recomputation between checkpoints."""

    @staticmethod
    def forward(ctx, u0, semi, t0, dt, nsteps, every=0):
        c = _ctx_of(semi)
        u0h = _ready(u0.detach()).cpu().numpy()
        c.set_state(np.ascontiguousarray(u0h), t0)
        c.ssprk33_record(dt, nsteps, every)
        uT, _ = c.get_state()
        ctx.semi = semi
        return torch.from_numpy(uT).to(u0.device)

    @staticmethod
    def backward(ctx, g):
        lam = _ready(g).cpu().numpy()
        out = _ctx_of(ctx.semi).ssprk33_adjoint(lam)
        return torch.from_numpy(out).to(g.device), None, None, None, None, None


def rhs(u, semi, t=0.0):
    return RHS.apply(u, semi, t)


def ssprk33_solve(u0, semi, t0, dt, nsteps, every=0):
    return SSPRK33Solve.apply(u0, semi, t0, dt, nsteps, every)
