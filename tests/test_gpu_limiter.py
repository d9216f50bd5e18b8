"""GPU Zhang-Shu positivity limiter against the oracle.

The device sums a node's stencil mean in its operator layout's entry order: ascending node
index with MFT_OPT_ENTRY_ORDER 0, where the oracle fed that same order gives bit-identical
states.  In the default bank-spreading order, and against the reference's stencil order
(by distance), the mean differs by rounding only: 1e-14 relative.  A limited SSP-RK3
trajectory matches the oracle's SSPRK33(stage_limiter!) to 1e-10."""
import numpy as np
import pytest

from test_limiter_oracle import GAMMA, dip_state

pytestmark = pytest.mark.gpu


def _domain(n=32):
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, (h, _) = W.jittered_grid(n, n, jitter=0.25)
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision="fp64"))
    dom = M.PointCloudDomain(solver, pts)
    eq = M.CompressibleEulerEquations2D(GAMMA)
    semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: dip_state(x), solver)
    return M, semi, dom, pts, h


@pytest.mark.parametrize("order", ["row", "spread", "stencil"])
def test_limit_matches_oracle(oracle, gpu_lib, order):
    from meshfree_gb300 import _lib as L
    M, semi, dom, pts, _h = _domain()
    if order == "row":
        dom.ctx.set_option(L.OPT_ENTRY_ORDER, 0)
    lim = M.PositivityPreservingLimiterZhangShu(thresholds=(0.05, 0.05),
                                                variables=(M.density, M.pressure))
    u0 = dip_state(pts)
    got = lim(u0.copy(), semi)
    nb = dom.pd.neighbors
    cols = np.sort(nb, axis=1) if order in ("row", "spread") else nb
    rp = np.arange(pts.shape[0] + 1, dtype=np.int64) * nb.shape[1]
    ref = u0.copy()
    oracle.stage_limiter(rp, cols.ravel(), [oracle.LIM_DENSITY, oracle.LIM_PRESSURE],
                         [0.05, 0.05], GAMMA)(ref)
    assert np.any(ref != u0)
    if order == "row":
        assert np.array_equal(got, ref)
    else:
        assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()


def test_limited_trajectory_matches_oracle(oracle, gpu_lib):
    M, semi, dom, pts, h = _domain()
    lim = M.PositivityPreservingLimiterZhangShu(thresholds=(0.05, 0.05),
                                                variables=(M.density, M.pressure))
    dt, nsteps = 0.05 * h, 10
    ode = M.semidiscretize(semi, (0.0, nsteps * dt))
    sol = M.solve(ode, M.SSPRK33(stage_limiter=lim), dt=dt)
    idx, _, _, _ = oracle.knn(pts, 35)
    assert np.array_equal(idx, dom.pd.neighbors)
    n = pts.shape[0]
    rp = np.arange(n + 1, dtype=np.int64) * 35
    w = oracle.weights(pts, rp, idx.ravel())
    ops = oracle.operators_from_stencils(n, rp, idx.ravel(), w)
    osemi = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA)
    olim = oracle.stage_limiter(rp, np.sort(idx, axis=1).ravel(),
                                [oracle.LIM_DENSITY, oracle.LIM_PRESSURE], [0.05, 0.05], GAMMA)
    ref, _ = oracle.ssprk33(osemi, ode.u0, 0.0, dt, nsteps, stage_limiter=olim)
    err = np.abs(sol.u - ref).max() / np.abs(ref).max()
    assert err < 1e-10, err
    # the limiter was active: the unlimited run differs
    free = M.solve(ode, M.SSPRK33(), dt=dt)
    assert np.any(free.u != sol.u)


def test_adjoint_refuses_limiter(gpu_lib):
    from meshfree_gb300._lib import MFTError
    M, semi, dom, pts, _h = _domain(16)
    dom.ctx.set_limiter([0], [0.05])
    u0 = dip_state(pts)
    with pytest.raises(MFTError):
        dom.ctx.rhs_adjoint(u0, u0)


def test_limited_trajectory_fp32_form_close_to_fp64(gpu_lib):
    """The limiter runs on the FP64 stage state and refreshes the FP32 shadow the FP32
    gathers read: the FP32 form's limited trajectory stays within 1e-5 of the FP64 one."""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, (h, _) = W.jittered_grid(32, 32, jitter=0.25)
    res = {}
    for prec in ("fp64", "fp32"):
        basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
        solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision=prec))
        dom = M.PointCloudDomain(solver, pts)
        eq = M.CompressibleEulerEquations2D(GAMMA)
        semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: dip_state(x), solver)
        lim = M.PositivityPreservingLimiterZhangShu(thresholds=(0.05, 0.05),
                                                    variables=(M.density, M.pressure))
        ode = M.semidiscretize(semi, (0.0, 10 * 0.05 * h))
        res[prec] = M.solve(ode, M.SSPRK33(stage_limiter=lim), dt=0.05 * h).u
    err = np.linalg.norm(res["fp32"][0] - res["fp64"][0]) / np.linalg.norm(res["fp64"][0])
    assert err < 1e-5, err
