"""The GPU against the oracle at the benchmarked sizes.

* 2D Euler isentropic vortex on the periodic square [-5,5]^2, N = 262,144 jittered nodes,
  PHS r^3 + degree 3, k = 35, residual viscosity + HistoryCallback (order 3), SSP-RK3
  dt = 0.2 h: one rhs! (FP64 form, both gather arithmetics) within 1e-12 of the condition
  scale; the trajectory to t = 1 (256 steps) within 1e-10 of the oracle's; the L2 density
  error against the exact vortex at t = 1 (this workload's own accuracy check) equal for
  both and below 2e-3; the FP32-apply form's density after 20 steps within 1e-5 (relative
  L2) of the oracle's FP64 trajectory.
* Four-quadrant Riemann problem on the periodic unit square, N = 1,048,576 jittered nodes,
  residual viscosity + Tominec hyperviscosity (c = 1), dt = 0.1 h: one rhs! within 1e-12
  of the condition scale and 3 SSP-RK3 steps within 1e-10 of the oracle's.
The oracle runs on all host cores (OpenMP); its KNN stencils and weights are compared bit
for bit with the GPU's before they are used.
"""
import os

import numpy as np
import pytest

from helpers import cond_scale, flux_np

pytestmark = pytest.mark.gpu

NT = os.cpu_count() or 8


def _oracle_problem(oracle, pts, per, k=35, tominec=False):
    n = pts.shape[0]
    idx, _, dmin, davg = oracle.knn(pts, k, period=per, nthreads=NT)
    rowptr = np.arange(n + 1, dtype=np.int64) * k
    w = oracle.weights(pts, rowptr, idx.ravel(), period=per, nthreads=NT)
    ops = oracle.operators_from_stencils(n, rowptr, idx.ravel(), w)
    out = dict(idx=idx, w=w, ops=ops, dmin=dmin, davg=davg)
    if tominec:
        w2 = oracle.weights(pts, rowptr, idx.ravel(), period=per, deriv_order=2, nthreads=NT)
        lap = oracle.csr_add(oracle.operators_from_stencils(n, rowptr, idx.ravel(), w2))
        out.update(lap=lap, H=oracle.ata(lap), hv_gamma=1.0 * dmin ** 4.5)
    return out


def _gpu_problem(kind, pts, per, arith="auto", prec="fp64"):
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    eq = M.CompressibleEulerEquations2D(1.4)
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision=prec, fp64_arith=arith))
    dom = M.PointCloudDomain(solver, pts, period=per)
    if kind == "vortex":
        src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom))
        ic = lambda x, t, e: W.isentropic_vortex(x, t)
    else:
        src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom),
                            hv=M.SourceHyperviscosityTominec(solver, eq, dom))
        ic = lambda x, t, e: W.riemann_ic(x)
    semi = M.SemidiscretizationHyperbolic(dom, eq, ic, solver, source_terms=src)
    return M, dom, semi


def _fresh(osemi):
    """The module's oracle semidiscretization as a new one starts: no history yet (the
    first rhs! of a solve runs before the first history push, with success_iter 0)."""
    osemi.s.success_iter = 0
    osemi.approx_du[:] = 0.0
    return osemi


def _check_rhs(oracle, o, osemi, ctx, u0, tominec=False):
    u_ref = u0.copy()
    du_ref, eps_ref = osemi.rhs(u_ref, 0.0, nthreads=NT, want_eps=True)
    du = np.empty_like(u0)
    ug = u0.copy()
    ctx.rhs(du, ug, 0.0)
    fl = [flux_np(u_ref, 0), flux_np(u_ref, 1)]
    scale = cond_scale(o["ops"], u_ref, fluxes=fl, eps=eps_ref,
                       lap=o.get("lap") if tominec else None,
                       hv_gamma=o.get("hv_gamma", 0.0))
    err = np.abs(du - du_ref).max(axis=1) / scale
    assert np.all(err <= 1e-12), err
    return err


@pytest.fixture(scope="module")
def vortex(oracle):
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(512)
    o = _oracle_problem(oracle, pts, per)
    osemi = oracle.Semi(pts, o["ops"], eq="euler", gamma=1.4, sources=(oracle.SRC_RV,),
                        h=o["davg"])
    return W, pts, per, h, o, osemi


@pytest.mark.parametrize("arith", ["dw", "dfma"])
def test_vortex_262k_rhs_matches_oracle(oracle, gpu_lib, vortex, arith):
    W, pts, per, h, o, osemi = vortex
    M, dom, semi = _gpu_problem("vortex", pts, per, arith=arith)
    assert np.array_equal(dom.pd.neighbors, o["idx"])
    u0 = W.isentropic_vortex(pts, 0.0)
    _check_rhs(oracle, o, _fresh(osemi), dom.ctx, u0)
    dom.ctx.close()


def test_vortex_262k_to_t1_matches_oracle_and_exact(oracle, gpu_lib, vortex):
    W, pts, per, h, o, osemi = vortex
    M, dom, semi = _gpu_problem("vortex", pts, per)
    dt = 0.2 * h
    nsteps = int(round(1.0 / dt))
    ode = M.semidiscretize(semi, (0.0, nsteps * dt))
    sol = M.solve(ode, M.SSPRK33(), dt=dt, callback=M.HistoryCallback(approx_order=3))
    u_ref, t_ref = oracle.ssprk33(_fresh(osemi), ode.u0, 0.0, dt, nsteps,
                                  history=oracle.History(osemi, 3), nthreads=NT)
    assert abs(sol.t - t_ref) <= 1e-14
    err = np.abs(sol.u - u_ref).max(axis=1) / np.abs(u_ref).max(axis=1)
    assert np.all(err < 1e-10), err
    exact = W.isentropic_vortex(pts, t_ref)
    l2_gpu = np.linalg.norm(sol.u[0] - exact[0]) / np.linalg.norm(exact[0])
    l2_ref = np.linalg.norm(u_ref[0] - exact[0]) / np.linalg.norm(exact[0])
    assert abs(l2_gpu - l2_ref) <= 1e-6 * l2_ref
    assert l2_gpu < 2e-3, l2_gpu
    dom.ctx.close()


def test_vortex_262k_fp32_apply_vs_oracle(oracle, gpu_lib, vortex):
    W, pts, per, h, o, osemi = vortex
    M, dom, semi = _gpu_problem("vortex", pts, per, prec="fp32")
    dt, nsteps = 0.2 * h, 20
    ode = M.semidiscretize(semi, (0.0, nsteps * dt))
    sol = M.solve(ode, M.SSPRK33(), dt=dt, callback=M.HistoryCallback(approx_order=3))
    u_ref, _ = oracle.ssprk33(_fresh(osemi), ode.u0, 0.0, dt, nsteps,
                              history=oracle.History(osemi, 3), nthreads=NT)
    l2 = np.linalg.norm(sol.u[0] - u_ref[0]) / np.linalg.norm(u_ref[0])
    assert l2 <= 1e-5, l2
    dom.ctx.close()


@pytest.fixture(scope="module")
def riemann(oracle):
    from meshfree_gb300 import workloads as W
    pts, h = W.riemann_cloud(1024)
    per = (1.0, 1.0)
    o = _oracle_problem(oracle, pts, per, tominec=True)
    osemi = oracle.Semi(pts, o["ops"], eq="euler", gamma=1.4,
                        sources=(oracle.SRC_RV, oracle.SRC_HV_TOMINEC), h=o["davg"],
                        hv=o["H"], hv_gamma=o["hv_gamma"])
    return W, pts, per, h, o, osemi


@pytest.mark.parametrize("arith", ["dw", "dfma"])
def test_riemann_1m_rhs_and_steps_match_oracle(oracle, gpu_lib, riemann, arith):
    W, pts, per, h, o, osemi = riemann
    M, dom, semi = _gpu_problem("riemann", pts, per, arith=arith)
    assert np.array_equal(dom.pd.neighbors, o["idx"])
    assert dom.pd.dx_min == o["dmin"] and dom.pd.dx_avg == o["davg"]
    u0 = W.riemann_ic(pts)
    _check_rhs(oracle, o, _fresh(osemi), dom.ctx, u0, tominec=True)
    dt, nsteps = 0.1 * h, 3
    ode = M.semidiscretize(semi, (0.0, nsteps * dt))
    sol = M.solve(ode, M.SSPRK33(), dt=dt, callback=M.HistoryCallback(approx_order=3))
    u_ref, _ = oracle.ssprk33(_fresh(osemi), ode.u0, 0.0, dt, nsteps,
                              history=oracle.History(osemi, 3), nthreads=NT)
    err = np.abs(sol.u - u_ref).max(axis=1) / np.abs(u_ref).max(axis=1)
    assert np.all(err < 1e-10), err
    dom.ctx.close()
