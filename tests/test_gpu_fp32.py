"""FP32-apply form: the bulk-copy-staged gathers and the halo-staged gathers (neighbour
records of each 256-row group in shared memory) against the one-node-per-thread gathers
(same operations in the same order, so bit-identical), and against the FP64 oracle
(condition-scaled error within FP32 rounding)."""
import numpy as np
import pytest

from helpers import GAMMA, cond_scale, flux_np, ic_bumpy
from test_gpu_rhs import CASES, _setup, cyl_ops  # noqa: F401  (fixture re-export)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["plain", "rv", "tominec", "rv_tominec", "tominec_rv",
                                  "flyer", "rv_flyer", "flyer_rv", "upwind"])
def test_fp32_staged_equals_thread_and_tracks_fp64(oracle, gpu_lib, cyl, cyl_ops, case):
    from meshfree_gb300 import _lib as L
    pts = cyl["positions"]
    u0 = ic_bumpy(pts)
    semi, ctx, hv, g = _setup(oracle, gpu_lib, cyl, cyl_ops, case)
    ctx.set_precision(L.PREC_FP32)
    out = {}
    for mode in (L.GATHER_THREAD, L.GATHER_STAGED, L.GATHER_HALO, L.GATHER_AUTO):
        ctx.set_option(L.OPT_GATHER, mode)
        du = np.empty_like(u0)
        u = u0.copy()
        ctx.rhs(du, u, 0.0)
        out[mode] = (du, u)
    assert ctx.get_option(L.OPT_TUNED_FWD) in (0, 1, 4, 8)
    assert ctx.get_option(L.OPT_HALO_STAGED_FWD) > 0
    for mode in (L.GATHER_STAGED, L.GATHER_HALO, L.GATHER_AUTO):
        assert np.array_equal(out[L.GATHER_THREAD][0], out[mode][0])
        assert np.array_equal(out[L.GATHER_THREAD][1], out[mode][1])
    u_ref = u0.copy()
    du_ref, eps_ref = semi.rhs(u_ref, 0.0, want_eps=True)
    srcs = CASES[case]
    visc = any(s in ("rv", "upwind") for s in srcs)
    scale = cond_scale(cyl_ops["ops"], u_ref, fluxes=[flux_np(u_ref, 0), flux_np(u_ref, 1)],
                       eps=eps_ref if visc else None,
                       lap=cyl_ops["lap"] if "tominec" in srcs else None, hv_gamma=g,
                       hvop=hv if "flyer" in srcs else None)
    err = np.abs(out[L.GATHER_STAGED][0] - du_ref).max(axis=1) / scale
    assert np.all(err < 1e-5), err


def test_fp32_staged_equals_thread_large(gpu_lib):
    """262,144 nodes: every warp of the persistent staged kernel walks several slices."""
    import meshfree_gb300 as M
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(512)
    eq = M.CompressibleEulerEquations2D(GAMMA)
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision="fp32"))
    domain = M.PointCloudDomain(solver, pts, period=per)
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, domain))
    semi = M.SemidiscretizationHyperbolic(domain, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                          solver, source_terms=src)
    ctx = domain.ctx
    u0 = semi.compute_coefficients(0.0)
    res = {}
    for mode in (L.GATHER_THREAD, L.GATHER_STAGED, L.GATHER_HALO, L.GATHER_AUTO):
        ctx.set_option(L.OPT_GATHER, mode)
        ctx.history_init(3)
        ctx.set_state(u0, 0.0)
        ctx.ssprk33(0.2 * h, 4)
        res[mode] = ctx.get_state()[0]
    assert np.array_equal(res[L.GATHER_THREAD], res[L.GATHER_STAGED])
    assert np.array_equal(res[L.GATHER_THREAD], res[L.GATHER_HALO])
    assert np.array_equal(res[L.GATHER_THREAD], res[L.GATHER_AUTO])
    assert ctx.get_option(L.OPT_HALO_STAGED_FWD) == ctx.get_option(L.OPT_HALO_GROUPS)
