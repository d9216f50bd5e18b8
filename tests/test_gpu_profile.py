"""The per-kernel profile (mft_profile / mft_profile_get) and the launch forms it changes.

With profiling on, every kernel is launched directly with a CUDA-event pair around it; with
it off, the steps are replayed as per-step CUDA graphs (or launched directly), and the
double-word forward gather is launched as a programmatic dependent of the viscosity-norm
reductions just before it.  All three forms run the same kernels on the same data, so an
SSP-RK3 run gives the same bits in each: the 2D Euler Riemann problem with residual
viscosity (history order 3) and Tominec hyperviscosity, in the double-word FP64 form
(fused flux records, staged gathers) and in the FP32-apply form.  The profile reports
the step's kernels with one launch per evaluation."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(prec):
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, h = W.riemann_cloud(96)
    eq = M.CompressibleEulerEquations2D(1.4)
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision=prec))
    dom = M.PointCloudDomain(solver, pts, period=(1.0, 1.0))
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom),
                        hv=M.SourceHyperviscosityTominec(solver, eq, dom))
    M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.riemann_ic(x), solver,
                                   source_terms=src)
    return dom.ctx, W.riemann_ic(pts), 0.1 * h


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_profiled_graph_and_direct_steps_agree(gpu_lib, prec):
    from meshfree_gb300 import _lib as L
    ctx, u0, dt = _problem(prec)
    warm, steps = 4, 5
    out = {}
    for mode in ("graph", "direct", "profiled"):
        ctx.history_init(3)
        ctx.set_state(u0, 0.0)
        ctx.ssprk33(dt, warm, use_graph=(mode == "graph"))
        if mode == "profiled":
            ctx.profile(True)
        ctx.ssprk33(dt, steps, use_graph=(mode == "graph"))
        if mode == "profiled":
            prof = ctx.profile_report()
            ctx.profile(False)
        out[mode] = ctx.get_state()
    assert out["graph"][1] == out["direct"][1] == out["profiled"][1]
    assert np.array_equal(out["graph"][0], out["direct"][0])
    assert np.array_equal(out["graph"][0], out["profiled"][0])
    rhs = 3 * steps
    assert prof["fwd_gather"][1] == rhs and prof["rev_gather"][1] == rhs
    assert prof["mean"][1] == rhs and prof["lexmax"][1] == rhs
    assert prof["history"][1] == steps
    assert all(v[0] > 0 for v in prof.values())
    if prec == "fp64":
        # the flux records are formed in the staged forward gather: no flux kernel
        assert ctx.get_option(L.OPT_FLUX_FUSED) == 1
        assert "flux" not in prof
    else:
        assert prof["eps"][1] == rhs
    ctx.close()
