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


@pytest.mark.parametrize("case", ["rv_tominec", "tominec_rv", "rv_flyer", "upwind"])
def test_dw_variants_bit_identical_with_bcs(oracle, gpu_lib, cyl, case):
    """The same on the reference's cylinder fixture with its strong BCs (Dirichlet inlet,
    do-nothing outlet, slip walls) and the source orderings, a history estimate set."""
    from helpers import ic_bumpy, stencil_ops
    from test_gpu_rhs import _setup
    from meshfree_gb300 import _lib as L
    pts = cyl["positions"]
    ops, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=3)
    lap_parts, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=3, order=2)
    lap = oracle.csr_add(lap_parts)
    fly_parts, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=5, order=4)
    cyl_ops = dict(ops=ops, lap=lap, H_tom=oracle.ata(lap), H_fly=oracle.csr_add(fly_parts))
    u0 = ic_bumpy(pts)
    rng = np.random.default_rng(3)
    approx = u0 * 0.1 * rng.standard_normal(u0.shape)
    semi, ctx, _hv, _g = _setup(oracle, gpu_lib, cyl, cyl_ops, case, success_iter=2,
                                approx_du=approx, arith="dw")
    ref = None
    for v in range(13):
        ctx.set_option(L.OPT_DW_VARIANT, v)
        du = np.empty_like(u0)
        u = u0.copy()
        ctx.rhs(du, u, 0.0)
        if ref is None:
            ref = (du, u)
        else:
            assert np.array_equal(du, ref[0]), (v, np.abs(du - ref[0]).max())
            assert np.array_equal(u, ref[1])
    assert ctx.get_option(L.OPT_HALO_STAGED_FWD) > 0
    ctx.close()


def test_entry_order_spreads_banks_and_keeps_the_sums(gpu_lib):
    """The bank-spreading entry order of the staged rows (MFT_OPT_ENTRY_ORDER 1, the
    default) against the structure order (0): fewer serialised shared-memory accesses per
    quarter-warp load in both staged layouts (as counted when they are built), and one
    rhs! that differs only by the rounding of the reordered sums (within 1e-12 of each
    variable's largest |du|); under either order every variant gives the same bits."""
    from meshfree_gb300 import workloads as W
    pts, h = W.riemann_cloud(96)
    L, dom, semi = _problem(pts, 1)
    ctx = dom.ctx
    u0 = W.riemann_ic(pts)
    du0 = np.empty_like(u0)
    ctx.rhs(du0, u0.copy(), 0.0)
    ctx.set_rv_state(du0 * 1.01, 2)
    out, banks = {}, {}
    for order in (0, 1):
        ctx.set_option(L.OPT_ENTRY_ORDER, order)
        ref = None
        for v in (0, 7, 11):
            ctx.set_option(L.OPT_DW_VARIANT, v)
            du = np.empty_like(u0)
            ctx.rhs(du, u0.copy(), 0.0)
            if ref is None:
                ref = du
            else:
                assert np.array_equal(du, ref), (order, v)
        out[order] = ref
        banks[order] = (ctx.get_option(L.OPT_BANK_FWD), ctx.get_option(L.OPT_BANK_REV))
        assert ctx.get_option(L.OPT_ENTRY_ORDER) == order
    assert all(b >= 1000 for b in banks[0] + banks[1]), banks
    assert banks[1][0] < 0.8 * banks[0][0] and banks[1][1] < 0.8 * banks[0][1], banks
    scale = np.abs(out[0]).max(axis=1, keepdims=True)
    assert np.all(np.abs(out[1] - out[0]) <= 1e-12 * scale)
    with pytest.raises(L.MFTError):
        ctx.set_option(L.OPT_ENTRY_ORDER, 2)
    ctx.close()


def test_fused_flux_records_are_bit_identical(gpu_lib):
    """With every row group staged, the forward variants 7, 11 and 12 form the neighbours'
    state and flux pairs while staging and the flux kernel is skipped
    (MFT_OPT_FUSE_FLUX 1, the default; MFT_OPT_FLUX_FUSED reads back 1): the same bits as
    with the flux kernel (MFT_OPT_FUSE_FLUX 0) and as an unfused variant, for forced
    variants and for the autotuned choice, over several evaluations and an SSP-RK3 run
    (graph-replayed steps).  With groups left unstaged (a half-shuffled layout) nothing is
    fused."""
    from meshfree_gb300 import workloads as W
    pts, h = W.riemann_cloud(96)
    L, dom, semi = _problem(pts, 1)
    ctx = dom.ctx
    u0 = W.riemann_ic(pts)
    du0 = np.empty_like(u0)
    ctx.rhs(du0, u0.copy(), 0.0)
    ctx.set_rv_state(du0 * 1.01, 2)

    def rhs():
        du = np.empty_like(u0)
        ctx.rhs(du, u0.copy(), 0.0)
        return du

    ctx.set_option(L.OPT_DW_VARIANT, 6)
    ref = rhs()
    assert ctx.get_option(L.OPT_FLUX_FUSED) == 0
    for fuse in (1, 0):
        ctx.set_option(L.OPT_FUSE_FLUX, fuse)
        for v in (7, 11, 12, -1):
            ctx.set_option(L.OPT_DW_VARIANT, v)
            for _ in range(3 if v == -1 else 2):
                assert np.array_equal(rhs(), ref), (fuse, v)
            if v >= 0:
                assert ctx.get_option(L.OPT_FLUX_FUSED) == fuse
    # trajectories: graph-replayed steps with the fused and the unfused forward variant
    out = []
    for v in (7, 8):
        ctx.set_option(L.OPT_FUSE_FLUX, 1)
        ctx.set_option(L.OPT_DW_VARIANT, v)
        ctx.set_state(u0, 0.0)
        ctx.history_init(2)
        ctx.ssprk33(0.05 * h, 6)
        out.append(ctx.get_state()[0])
    assert np.array_equal(out[0], out[1])
    ctx.close()
    # groups without a list (a 32 x 32 cloud in node order, second half shuffled): the
    # forced variant 7 runs unfused
    pts2, _ = W.riemann_cloud(32)
    n = pts2.shape[0]
    rng = np.random.default_rng(4)
    perm = np.arange(n)
    perm[n // 2:] = n // 2 + rng.permutation(n - n // 2)
    pts2 = np.ascontiguousarray(pts2[perm])
    L, dom, semi = _problem(pts2, 0)
    ctx = dom.ctx
    u2 = W.riemann_ic(pts2)
    ctx.set_option(L.OPT_DW_VARIANT, 7)
    du = np.empty_like(u2)
    ctx.rhs(du, u2.copy(), 0.0)
    assert ctx.get_option(L.OPT_HALO_STAGED_FWD) < ctx.get_option(L.OPT_HALO_GROUPS)
    assert ctx.get_option(L.OPT_FLUX_FUSED) == 0
    ctx.set_option(L.OPT_DW_VARIANT, 6)
    du6 = np.empty_like(u2)
    ctx.rhs(du6, u2.copy(), 0.0)
    assert np.array_equal(du, du6)
    ctx.close()
