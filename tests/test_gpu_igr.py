"""GPU IGR source (SourceIGR) against the oracle: rhs! with the regularisation (a
conjugate-gradient solve per evaluation) and a short SSP-RK3 trajectory.  Both sides
run the same CG iteration count unless a residual lands within rounding of the
tolerance; rounding differences in the CG stay below 1e-9 of max |du| (asserted)."""
import numpy as np
import pytest

from helpers import GAMMA, load_ops_into, stencil_ops

pytestmark = pytest.mark.gpu


def _setup(oracle, alpha_h2=1.0):
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(32, seed=3)
    idx, _, _, _ = oracle.knn(pts, 35, period=per)
    ops, _ = stencil_ops(oracle, pts, idx, period=per)
    alpha = alpha_h2 * h * h
    semi = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA, sources=[oracle.SRC_IGR],
                       igr_alpha=alpha, igr_maxiter=20)
    ctx = L.Context(0)
    ctx.set_points(pts)
    load_ops_into(ctx, ops)
    ctx.set_equations(L.EQ_EULER2D, [GAMMA])
    ctx.set_bcs([], [0], np.zeros(0, np.int32), None)
    ctx.set_sources([L.SRC_IGR], [[alpha, 20.0, 0.0, 0.0]])
    return semi, ctx, pts, h


@pytest.mark.parametrize("alpha_h2", [1.0, 20.0])
def test_rhs_igr_matches_oracle(oracle, gpu_lib, alpha_h2):
    from meshfree_gb300 import workloads as W
    semi, ctx, pts, _h = _setup(oracle, alpha_h2)
    u = W.isentropic_vortex(pts, 0.0)
    ref = semi.rhs(u.copy(), 0.0)
    got = np.empty_like(u)
    ctx.rhs(got, u.copy(), 0.0)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 1e-9, err
    # the regularisation is active: without it the momentum rows differ
    ctx.set_sources([], [])
    plain = np.empty_like(u)
    ctx.rhs(plain, u.copy(), 0.0)
    assert np.abs(plain[1:3] - got[1:3]).max() > 1e-6 * np.abs(got).max()
    assert np.array_equal(plain[0], got[0]) and np.array_equal(plain[3], got[3])


def test_igr_trajectory_matches_oracle(oracle, gpu_lib):
    from meshfree_gb300 import workloads as W
    semi, ctx, pts, h = _setup(oracle)
    u0 = W.isentropic_vortex(pts, 0.0)
    dt, nsteps = 0.1 * h, 5
    ref, _ = oracle.ssprk33(semi, u0, 0.0, dt, nsteps)
    ctx.set_state(u0, 0.0)
    ctx.ssprk33(dt, nsteps, use_graph=True)
    got, _ = ctx.get_state()
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 1e-9, err


def test_igr_in_fp32_form_close_to_fp64(gpu_lib):
    """The IGR term is computed in FP64 and added in the FP64 stage epilogue of the
    FP32-apply kernels: the FP32 form's rhs! stays within FP32 rounding of the FP64 one."""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(64, seed=5)
    out = {}
    for prec in ("fp64", "fp32"):
        basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
        solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision=prec))
        dom = M.PointCloudDomain(solver, pts, period=per)
        eq = M.CompressibleEulerEquations2D(1.4)
        src = M.SourceTerms(igr=M.SourceIGR(solver, eq, dom, alpha=h * h))
        semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                              solver, source_terms=src)
        u = W.isentropic_vortex(pts, 0.0)
        du = np.empty_like(u)
        M.rhs_(du, u.copy(), semi, 0.0)
        out[prec] = du
    err = np.linalg.norm(out["fp32"] - out["fp64"]) / np.linalg.norm(out["fp64"])
    assert err < 2e-4, err
