"""The kernel variants of the double-word gathers (MFT_OPT_DW_VARIANT 0-12) form the same
sums in the same order, so one rhs! is bit-identical across them: the 2D Euler
four-quadrant Riemann problem with residual viscosity (history estimate set) and Tominec
hyperviscosity, which runs the forward gather with t and q and the transpose gather with
both terms.  Three layouts exercise the staged variants (6-12): every row group's
neighbour records staged (Morton row order), none (a shuffled node order kept as the
layout order: each group of rows then gathers from thousands of nodes), and a mix (a
32 x 32 cloud in row order with its second half shuffled: the groups of the first half
gather from a few hundred nodes each, those of the second half from more than 640)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(pts, layout_order):
    import meshfree_gb300 as M
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    eq = M.CompressibleEulerEquations2D(1.4)
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision="fp64", fp64_arith="dw"))
    dom = M.PointCloudDomain(solver, pts, period=(1.0, 1.0))
    dom.ctx.set_option(L.OPT_LAYOUT_ORDER, layout_order)
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom),
                        hv=M.SourceHyperviscosityTominec(solver, eq, dom))
    semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.riemann_ic(x), solver,
                                          source_terms=src)
    return L, dom, semi


LAYOUTS = {"morton": (96, None, 1), "shuffled": (96, 1.0, 0), "half_shuffled": (32, 0.5, 0)}


@pytest.mark.parametrize("layout", list(LAYOUTS))
def test_dw_variants_bit_identical(gpu_lib, layout):
    from meshfree_gb300 import workloads as W
    side, frac, order = LAYOUTS[layout]
    pts, h = W.riemann_cloud(side)
    n = pts.shape[0]
    if frac is not None:
        rng = np.random.default_rng(4)
        k = int(frac * n)
        perm = np.arange(n)
        perm[n - k:] = n - k + rng.permutation(k)
        pts = np.ascontiguousarray(pts[perm])
    L, dom, semi = _problem(pts, order)
    ctx = dom.ctx
    u0 = W.riemann_ic(pts)
    # a history estimate, so that the residual viscosity is formed from it
    du0 = np.empty_like(u0)
    ctx.rhs(du0, u0.copy(), 0.0)
    rng = np.random.default_rng(9)
    ctx.set_rv_state(du0 * (1.0 + 0.05 * rng.standard_normal(du0.shape)), 2)
    ref = None
    for v in range(13):
        ctx.set_option(L.OPT_DW_VARIANT, v)
        du = np.empty_like(u0)
        ctx.rhs(du, u0.copy(), 0.0)
        assert np.all(np.isfinite(du))
        if ref is None:
            ref = du
        else:
            assert np.array_equal(du, ref), (v, np.abs(du - ref).max())
    groups = ctx.get_option(L.OPT_HALO_GROUPS)
    staged = (ctx.get_option(L.OPT_HALO_STAGED_FWD), ctx.get_option(L.OPT_HALO_STAGED_REV))
    assert groups in ((n + 255) // 256, (n + 127) // 128)
    if layout == "morton":
        assert staged == (groups, groups)
    elif layout == "shuffled":
        assert staged == (0, 0)
    else:
        assert 0 < staged[0] < groups and 0 < staged[1] < groups
    ctx.close()
