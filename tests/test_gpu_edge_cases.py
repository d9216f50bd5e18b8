"""Edge cases of the engine on the GPU: empty and degenerate inputs are refused with status
codes; the smallest clouds, a KNN that takes every node, a cloud whose size leaves a
partial 32-row slice, and zero-step integration behave like the oracle."""
import numpy as np
import pytest

from helpers import GAMMA, ic_bumpy, stencil_ops

pytestmark = pytest.mark.gpu


def _code(fn):
    from meshfree_gb300._lib import MFTError
    with pytest.raises(MFTError) as e:
        fn()
    return e.value.code


def test_empty_and_degenerate_inputs_are_refused(gpu_lib):
    from meshfree_gb300 import _lib as L
    ctx = L.Context(0)
    assert _code(lambda: ctx.set_points(np.zeros((0, 2)))) == L.MFT_ERR_ARG
    pts = np.random.default_rng(1).uniform(size=(10, 2))
    ctx.set_points(pts)
    assert _code(lambda: ctx.knn(11)) == L.MFT_ERR_ARG          # k > n
    assert _code(lambda: ctx.knn(0)) == L.MFT_ERR_ARG
    assert _code(lambda: ctx.set_points(pts, period=(1.0, 0.0))) == L.MFT_ERR_ARG
    ctx.set_points(pts)
    bad = np.array([0, 3, 3], dtype=np.int64)                    # rowptr of 2 rows for 10 nodes
    assert _code(lambda: ctx.set_stencils(bad, np.zeros(3, np.int32))) == L.MFT_ERR_ARG
    rp = np.arange(11, dtype=np.int64) * 2
    dup = np.repeat(np.arange(10, dtype=np.int32), 2)            # every node listed twice
    assert _code(lambda: ctx.set_stencils(rp, dup)) == L.MFT_ERR_ARG
    ctx.close()


def test_knn_taking_every_node_matches_oracle(oracle, gpu_lib):
    from meshfree_gb300 import _lib as L
    pts = np.random.default_rng(2).uniform(size=(40, 2))
    ctx = L.Context(0)
    ctx.set_points(pts)
    idx, dist, dmin, davg = ctx.knn(40, want_dist=True)
    idx_o, dist_o, dmin_o, davg_o = oracle.knn(pts, 40)
    assert np.array_equal(idx, idx_o)
    assert np.array_equal(dist, dist_o)
    assert dmin == dmin_o and davg == davg_o
    ctx.close()


@pytest.mark.parametrize("n", [33, 95])
def test_partial_slice_rhs_matches_oracle(oracle, gpu_lib, n):
    """n not a multiple of the 32-row slice: the last slice is partial in both layouts
    (and, in the FP64 form, inside a partial 256-row ordering window)."""
    from meshfree_gb300 import _lib as L
    pts = np.random.default_rng(3).uniform(size=(n, 2))
    idx, _, _, _ = oracle.knn(pts, 20)
    ops, _ = stencil_ops(oracle, pts, idx)
    semi = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA)
    u = ic_bumpy(pts)
    ref = semi.rhs(u.copy(), 0.0)
    ctx = L.Context(0)
    ctx.set_points(pts)
    ctx.set_stencils(np.arange(n + 1, dtype=np.int64) * 20, idx.ravel())
    ctx.weights(L.OP_GRAD, 3, 3, 1)
    ctx.set_equations(L.EQ_EULER2D, [GAMMA])
    ctx.set_bcs([], [0], np.zeros(0, np.int32), None)
    ctx.set_sources([], [])
    du = np.empty_like(u)
    ctx.rhs(du, u.copy(), 0.0)
    assert np.abs(du - ref).max() <= 1e-11 * np.abs(ref).max()
    ctx.set_precision(L.PREC_FP32)
    du32 = np.empty_like(u)
    ctx.rhs(du32, u.copy(), 0.0)
    assert np.abs(du32 - ref).max() <= 1e-4 * np.abs(ref).max()
    ctx.close()


def test_zero_steps_leave_the_state_unchanged(gpu_lib):
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(24)
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis)
    dom = M.PointCloudDomain(solver, pts, period=per)
    eq = M.CompressibleEulerEquations2D(1.4)
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom))
    semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                          solver, source_terms=src)
    ctx = dom.ctx
    u0 = semi.compute_coefficients(0.0)
    ctx.history_init(3)
    ctx.set_state(u0, 0.25)
    ctx.ssprk33(0.1 * h, 0)
    u, t = ctx.get_state()
    assert t == 0.25 and np.array_equal(u, u0)
    uh = u0.copy()
    t = ctx.ssprk33_host(uh, 0.25, 0.1 * h, 0)
    assert t == 0.25 and np.array_equal(uh, u0)
