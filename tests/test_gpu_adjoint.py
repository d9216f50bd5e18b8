"""GPU adjoint of rhs! and of the SSP-RK3 trajectory.

Checked against (1) the oracle's adjoint (CPU restatement) on identical inputs:
per variable max |gpu - ref| <= 1e-12 * s with the rounding scale
s = max_i [ sum_d (|D_d|^T sum_v |lam_v|)_i * Jmax_i + gamma (|H|^T |lam_v|)_i ]
(Jmax_i = largest flux-Jacobian entry at node i); (2) centred finite differences of
the GPU's own forward rhs! and trajectory (1e-7 for rhs!, 1e-6 for the trajectory
gradient), and forward-mode (complex-step) derivatives of the numpy restatement of rhs!
(1e-12: dot products on the reference fixture, the full Jacobian at N = 64); (3) checkpointed sweeps (recomputation between checkpoints) equal the
sweep over stored stage states bit for bit; (4) the torch.autograd mirror.
"""
import types

import numpy as np
import pytest

from helpers import (GAMMA, flux_np, ic_bumpy, jacobian_complex, jvp_complex,
                     load_ops_into, stencil_ops, trajectory_jvp_complex)
from test_gpu_rhs import _setup

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def cyl_ops(oracle, cyl):
    pts = cyl["positions"]
    ops, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=3)
    lap_parts, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=3, order=2)
    lap = oracle.csr_add(lap_parts)
    fly_parts, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=5, order=4)
    return dict(ops=ops, lap=lap, H_tom=oracle.ata(lap), H_fly=oracle.csr_add(fly_parts))


@pytest.fixture(scope="module")
def vortex(oracle):
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(16, seed=11)
    idx, _, _, _ = oracle.knn(pts, 20, period=per)
    ops, _ = stencil_ops(oracle, pts, idx, period=per)
    return pts, ops, h


def vortex_ctx(oracle, vortex):
    from meshfree_gb300 import _lib as L
    pts, ops, _h = vortex
    semi = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA)
    ctx = L.Context(0)
    ctx.set_points(pts)
    load_ops_into(ctx, ops)
    ctx.set_equations(L.EQ_EULER2D, [GAMMA])
    ctx.set_bcs([], [0], np.zeros(0, np.int32), None)
    ctx.set_sources([], [])
    return semi, ctx


def jac_max(u, eq):
    """Largest |entry| of dF/du, dG/du per node (finite differences; a scale only)."""
    if eq != "euler":
        return np.full(u.shape[1], 1.0)
    out = np.zeros(u.shape[1])
    for k in range(4):
        e = 1e-7 * np.maximum(np.abs(u[k]), 1.0)
        up = u.copy()
        up[k] += e
        for d in range(2):
            out = np.maximum(out, (np.abs(flux_np(up, d) - flux_np(u, d)) / e).max(axis=0))
    return out


def adj_scale(ops, u, lam, eq, hv=None, hv_gamma=0.0):
    A = [abs(o.to_scipy()) for o in ops]
    la = np.abs(lam).sum(axis=0)
    base = sum(a.T @ la for a in A) * jac_max(u, eq)
    out = np.zeros(lam.shape[0])
    for v in range(lam.shape[0]):
        s = base.copy()
        if hv is not None:
            s += hv_gamma * (abs(hv.to_scipy()).T @ np.abs(lam[v]))
        out[v] = s.max()
    return out


CASES = ["plain", "tominec", "flyer"]


@pytest.mark.parametrize("case", CASES)
def test_rhs_adjoint_euler_matches_oracle(oracle, gpu_lib, cyl, cyl_ops, case):
    semi, ctx, hv, g = _setup(oracle, gpu_lib, cyl, cyl_ops, case)
    u = ic_bumpy(cyl["positions"])
    lam = np.random.default_rng(1).standard_normal(u.shape)
    ref = semi.rhs_adjoint(u, lam)
    got = ctx.rhs_adjoint(lam, u)
    err = np.abs(got - ref).max(axis=1) / adj_scale(cyl_ops["ops"], u, lam, "euler", hv, g)
    assert np.all(err <= TOL), err


@pytest.mark.parametrize("case", ["plain", "flyer"])
def test_rhs_adjoint_staged_equals_direct(oracle, gpu_lib, cyl, cyl_ops, case):
    """The double-word adjoint gather with each row group's cotangent pairs staged in
    shared memory (default) and read directly (a direct variant forced): bit-identical."""
    from meshfree_gb300 import _lib as L
    semi, ctx, hv, g = _setup(oracle, gpu_lib, cyl, cyl_ops, case, arith="dw")
    u = ic_bumpy(cyl["positions"])
    lam = np.random.default_rng(2).standard_normal(u.shape)
    staged = ctx.rhs_adjoint(lam, u)
    assert ctx.get_option(L.OPT_HALO_STAGED_REV) > 0
    ctx.set_option(L.OPT_DW_VARIANT, 2)
    direct = ctx.rhs_adjoint(lam, u)
    assert np.array_equal(staged, direct)
    ctx.close()


def test_rhs_adjoint_advection_matches_oracle(oracle, gpu_lib, cyl, cyl_ops):
    semi, ctx, hv, g = _setup(oracle, gpu_lib, cyl, cyl_ops, "tominec", eq="advection")
    x = cyl["positions"]
    u = np.ascontiguousarray(np.sin(2 * x[:, 0] + x[:, 1])[None, :])
    lam = np.random.default_rng(2).standard_normal(u.shape)
    ref = semi.rhs_adjoint(u, lam)
    got = ctx.rhs_adjoint(lam, u)
    err = np.abs(got - ref).max(axis=1) / adj_scale(cyl_ops["ops"], u, lam, "adv", hv, g)
    assert np.all(err <= TOL), err


def test_rhs_adjoint_vortex_matches_oracle(oracle, gpu_lib, vortex):
    from meshfree_gb300 import workloads as W
    semi, ctx = vortex_ctx(oracle, vortex)
    u = W.isentropic_vortex(vortex[0], 0.0)
    lam = np.random.default_rng(3).standard_normal(u.shape)
    ref = semi.rhs_adjoint(u, lam)
    got = ctx.rhs_adjoint(lam, u)
    err = np.abs(got - ref).max(axis=1) / adj_scale(vortex[1], u, lam, "euler")
    assert np.all(err <= TOL), err


@pytest.mark.parametrize("case", CASES)
def test_rhs_adjoint_dot_product_with_forward_mode(oracle, gpu_lib, cyl, cyl_ops, case):
    """<lam, J v> by the complex step through the numpy restatement of rhs! (forward
    mode, exact to rounding) against <J^T lam, v> from the GPU adjoint: 1e-12 relative."""
    semi, ctx, _hv, _g = _setup(oracle, gpu_lib, cyl, cyl_ops, case)
    u = ic_bumpy(cyl["positions"])
    rng = np.random.default_rng(6)
    lam = rng.standard_normal(u.shape)
    v = rng.standard_normal(u.shape) * np.abs(u).max(axis=1, keepdims=True)
    lhs = float(np.sum(lam * jvp_complex(semi, u, v)))
    rhs = float(np.sum(ctx.rhs_adjoint(lam, u) * v))
    assert abs(lhs - rhs) / abs(rhs) < TOL, (lhs, rhs)


def test_rhs_adjoint_equals_forward_mode_jacobian_small(oracle, gpu_lib):
    """N = 64 vortex cloud (256 unknowns): the GPU adjoint equals J^T lam of the dense
    complex-step Jacobian entry by entry (1e-12 of the product's scale)."""
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(8, seed=11)
    idx, _, _, _ = oracle.knn(pts, 20, period=per)
    ops, _ = stencil_ops(oracle, pts, idx, period=per)
    semi, ctx = vortex_ctx(oracle, (pts, ops, h))
    u = W.isentropic_vortex(pts, 0.0)
    J = jacobian_complex(semi, u)
    lam = np.random.default_rng(7).standard_normal(u.shape)
    ref = (J.T @ lam.ravel()).reshape(u.shape)
    got = ctx.rhs_adjoint(lam, u)
    assert np.abs(got - ref).max() <= TOL * (np.abs(J).T @ np.abs(lam).ravel()).max()


@pytest.mark.parametrize("case", ["plain", "flyer"])
def test_rhs_adjoint_dot_product_with_gpu_fd(oracle, gpu_lib, cyl, cyl_ops, case):
    _semi, ctx, _hv, _g = _setup(oracle, gpu_lib, cyl, cyl_ops, case)
    u = ic_bumpy(cyl["positions"])
    rng = np.random.default_rng(4)
    lam = rng.standard_normal(u.shape)
    v = rng.standard_normal(u.shape) * np.abs(u).max(axis=1, keepdims=True)
    e = 1e-6
    dp, dm = np.empty_like(u), np.empty_like(u)
    up, um = u + e * v, u - e * v
    ctx.rhs(dp, up, 0.0)
    ctx.rhs(dm, um, 0.0)
    lhs = float(np.sum(lam * (dp - dm) / (2 * e)))
    rhs = float(np.sum(ctx.rhs_adjoint(lam, u) * v))
    assert abs(lhs - rhs) / abs(rhs) < 1e-7, (lhs, rhs)


def test_rhs_adjoint_rejects_viscosity_after_hyperviscosity(oracle, gpu_lib, cyl, cyl_ops):
    """The residual viscosity's partial du would include the hyperviscosity term, whose
    adjoint the viscosity path does not route: MFT_ERR_UNSUPPORTED (the viscosity sources
    before or without hyperviscosity are covered in test_gpu_adjoint_visc.py)."""
    from meshfree_gb300._lib import MFTError, MFT_ERR_UNSUPPORTED
    _semi, ctx, _hv, _g = _setup(oracle, gpu_lib, cyl, cyl_ops, "tominec_rv")
    u = ic_bumpy(cyl["positions"])
    with pytest.raises(MFTError) as e:
        ctx.rhs_adjoint(u, u)
    assert e.value.code == MFT_ERR_UNSUPPORTED


def _trajectory(oracle, gpu_lib, cyl, cyl_ops, vortex, case):
    from meshfree_gb300 import workloads as W
    if case == "vortex":
        semi, ctx = vortex_ctx(oracle, vortex)
        u0 = W.isentropic_vortex(vortex[0], 0.0)
        h = vortex[2]
    else:
        semi, ctx, _hv, _g = _setup(oracle, gpu_lib, cyl, cyl_ops, "tominec")
        u0 = ic_bumpy(cyl["positions"])
        h = float(cyl["dx"][0])
    return semi, ctx, u0, 0.1 * h


@pytest.mark.parametrize("case", ["vortex", "cyl"])
def test_trajectory_adjoint_matches_oracle(oracle, gpu_lib, cyl, cyl_ops, vortex, case):
    semi, ctx, u0, dt = _trajectory(oracle, gpu_lib, cyl, cyl_ops, vortex, case)
    nsteps = 6
    rng = np.random.default_rng(7)
    target = u0[0] * (1.0 + 0.01 * rng.standard_normal(u0.shape[1]))
    uT_o, _, rec = oracle.ssprk33_record(semi, u0, 0.0, dt, nsteps)
    lamT = np.zeros_like(uT_o)
    lamT[0] = uT_o[0] - target
    ref = oracle.ssprk33_adjoint(semi, rec, dt, lamT)
    from meshfree_gb300 import _lib as L
    grads, states = {}, {}
    for every in (0, 2, 4, -1):
        ctx.set_state(u0, 0.0)
        ctx.ssprk33_record(dt, nsteps, every)
        if every == -1:
            # the default policy stores every stage state of so small a problem
            assert ctx.get_option(L.OPT_ADJ_EVERY) == 0
        states[every] = ctx.get_state()[0]
        grads[every] = ctx.ssprk33_adjoint(lamT)
    assert np.array_equal(grads[0], grads[-1])
    # the recording integrator is the plain one
    ctx.set_state(u0, 0.0)
    ctx.ssprk33(dt, nsteps, use_graph=False)
    assert np.array_equal(ctx.get_state()[0], states[0])
    # recomputation between checkpoints reproduces the stored stage states exactly
    assert np.array_equal(grads[0], grads[2]) and np.array_equal(grads[0], grads[4])
    assert np.array_equal(states[0], states[2])
    assert np.abs(states[0] - uT_o).max() <= 1e-10 * np.abs(uT_o).max()
    err = np.linalg.norm(grads[0] - ref) / np.linalg.norm(ref)
    assert err < 1e-10, err


@pytest.mark.parametrize("case", ["vortex", "cyl"])
def test_trajectory_adjoint_matches_forward_mode(oracle, gpu_lib, cyl, cyl_ops, vortex, case):
    """Checkpointed GPU reverse sweep (every 2 steps) against the forward-mode derivative
    of the whole 6-step trajectory (complex step through the numpy restatement):
    <lam_T, (du_T/du_0) v> = <lam_0, v>.  The GPU linearises about its own stage states
    (within 1e-14 of the restatement's), hence 1e-11 rather than the 1e-12 of a single
    rhs!."""
    semi, ctx, u0, dt = _trajectory(oracle, gpu_lib, cyl, cyl_ops, vortex, case)
    nsteps = 6
    rng = np.random.default_rng(9)
    lamT = rng.standard_normal(u0.shape)
    v = rng.standard_normal(u0.shape) * np.abs(u0).max(axis=1, keepdims=True)
    ctx.set_state(u0, 0.0)
    ctx.ssprk33_record(dt, nsteps, 2)
    lam0 = ctx.ssprk33_adjoint(lamT)
    lhs = float(np.sum(lamT * trajectory_jvp_complex(semi, u0, v, dt, nsteps)))
    rhs = float(np.sum(lam0 * v))
    assert abs(lhs - rhs) / abs(rhs) < 1e-11, (lhs, rhs)


def test_solve_adjoint_vortex_matches_gpu_fd():
    """Host API: gradient of J = 0.5 |rho(T) - rho*|^2 w.r.t. u0 (GPU stencils and
    weights, 10 steps, checkpoint every 3) against centred differences of GPU solves."""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(24, seed=3)
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=20)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision="fp64"))
    dom = M.PointCloudDomain(solver, pts, period=per)
    eq = M.CompressibleEulerEquations2D(1.4)
    semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                          solver)
    dt, nsteps = 0.1 * h, 10
    ode = M.semidiscretize(semi, (0.0, nsteps * dt))
    rng = np.random.default_rng(9)
    target = ode.u0[0] * (1.0 + 0.01 * rng.standard_normal(ode.u0.shape[1]))

    def J(u):
        d = u[0] - target
        return 0.5 * float(d @ d)

    def dJ(u):
        g = np.zeros_like(u)
        g[0] = u[0] - target
        return g

    _sol, grad = M.solve_adjoint(ode, dt, dJ, checkpoint_every=3)
    v = rng.standard_normal(ode.u0.shape) * np.abs(ode.u0).max(axis=1, keepdims=True)
    e = 1e-6
    vals = []
    for s in (1.0, -1.0):
        o = M.ODEProblem(np.ascontiguousarray(ode.u0 + s * e * v), ode.tspan, semi)
        vals.append(J(M.solve(o, M.SSPRK33(), dt=dt).u))
    fd = (vals[0] - vals[1]) / (2 * e)
    ad = float(np.sum(grad * v))
    assert abs(fd - ad) / abs(ad) < 1e-6, (fd, ad)


def test_torch_autograd_mirror(oracle, gpu_lib, vortex):
    import torch
    from meshfree_gb300 import autodiff
    from meshfree_gb300 import workloads as W
    _semi, ctx = vortex_ctx(oracle, vortex)
    semi = types.SimpleNamespace(domain=types.SimpleNamespace(ctx=ctx))
    u0 = W.isentropic_vortex(vortex[0], 0.0)
    w = np.random.default_rng(5).standard_normal(u0.shape)
    u = torch.tensor(u0, device="cuda", requires_grad=True)
    du = autodiff.rhs(u, semi)
    (du * torch.tensor(w, device="cuda")).sum().backward()
    ref_du = np.empty_like(u0)
    ctx.rhs(ref_du, u0.copy(), 0.0)
    assert np.array_equal(du.detach().cpu().numpy(), ref_du)
    assert np.array_equal(u.grad.cpu().numpy(), ctx.rhs_adjoint(w, u0))
    # trajectory: gradient of 0.5 |rho(T)|^2 through SSPRK33Solve
    dt = 0.1 * vortex[2]
    u = torch.tensor(u0, device="cuda", requires_grad=True)
    uT = autodiff.ssprk33_solve(u, semi, 0.0, dt, 4, 2)
    (0.5 * (uT[0] ** 2).sum()).backward()
    ctx.set_state(u0, 0.0)
    ctx.ssprk33_record(dt, 4, 0)
    uT_h = ctx.get_state()[0]
    lam = np.zeros_like(uT_h)
    lam[0] = uT_h[0]
    assert np.array_equal(u.grad.cpu().numpy(), ctx.ssprk33_adjoint(lam))
