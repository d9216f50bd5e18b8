"""rhs! on ragged stencils: interior rows of 35 and a boundary band of 40-60 neighbours
(scrambled Halton nodes in the unit square), so that the forward sliced ELL carries
padded slots as well as the reverse adjacency.  FP64 against the oracle (condition-scaled
1e-12, residual viscosity cold and with a history estimate); the FP32-apply form's
staged, per-thread and autotuned mappings bit-identical to each other and within FP32
rounding (1e-5 of the condition scale) of the oracle."""
import numpy as np
import pytest

from helpers import GAMMA, cond_scale, flux_np, ic_bumpy

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ragged(oracle):
    from meshfree_gb300 import workloads as W
    pts = W.halton_points(6000, 2)
    ks = W.halton_stencil_sizes(pts)
    idx, _, _, davg = oracle.knn(pts, int(ks.max()))
    rowptr = np.concatenate([[0], np.cumsum(ks)]).astype(np.int64)
    cols = np.concatenate([idx[i, :ks[i]] for i in range(pts.shape[0])]).astype(np.int32)
    w = oracle.weights(pts, rowptr, cols, rbf_pow=3, polydeg=3, deriv_order=1)
    ops = oracle.operators_from_stencils(pts.shape[0], rowptr, cols, w)
    return pts, rowptr, cols, ops, float(davg)


def _pair(oracle, ragged, success_iter, approx):
    from meshfree_gb300 import _lib as L
    pts, rowptr, cols, ops, davg = ragged
    semi = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA, sources=[oracle.SRC_RV], c_rv=1.0,
                       c_uw=1.0, h=davg)
    semi.s.success_iter = success_iter
    if approx is not None:
        semi.approx_du[:] = approx.ravel()
    ctx = L.Context(0)
    ctx.set_points(pts)
    ctx.set_stencils(rowptr, cols)
    ctx.weights(L.OP_GRAD, 3, 3, 1)
    ctx.set_equations(L.EQ_EULER2D, [GAMMA])
    ctx.set_bcs([], [0], np.zeros(0, np.int32), None)
    ctx.set_sources([L.SRC_RV], [[1.0, 1.0, davg, 0.0]])
    if success_iter:
        ctx.set_rv_state(approx, success_iter)
    return semi, ctx


@pytest.mark.parametrize("warm", [False, True])
def test_ragged_rhs_fp64_and_fp32(oracle, gpu_lib, ragged, warm):
    from meshfree_gb300 import _lib as L
    pts, _rp, _ci, ops, _h = ragged
    u0 = ic_bumpy(pts)
    approx = None
    if warm:
        plain = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA).rhs(u0.copy(), 0.0)
        rng = np.random.default_rng(21)
        approx = np.ascontiguousarray(plain * (1 + 0.05 * rng.standard_normal(plain.shape)))
    semi, ctx = _pair(oracle, ragged, 2 if warm else 0, approx)
    du_ref, eps_ref = semi.rhs(u0.copy(), 0.0, want_eps=True)
    scale = cond_scale(ops, u0, fluxes=[flux_np(u0, 0), flux_np(u0, 1)], eps=eps_ref)
    du = np.empty_like(u0)
    ctx.rhs(du, u0.copy(), 0.0)
    err = np.abs(du - du_ref).max(axis=1) / scale
    assert np.all(err <= 1e-12), err
    ctx.set_precision(L.PREC_FP32)
    out = {}
    for mode in (L.GATHER_THREAD, L.GATHER_STAGED, L.GATHER_AUTO):
        ctx.set_option(L.OPT_GATHER, mode)
        d32 = np.empty_like(u0)
        ctx.rhs(d32, u0.copy(), 0.0)
        out[mode] = d32
    assert np.array_equal(out[L.GATHER_THREAD], out[L.GATHER_STAGED])
    assert np.array_equal(out[L.GATHER_THREAD], out[L.GATHER_AUTO])
    err32 = np.abs(out[L.GATHER_STAGED] - du_ref).max(axis=1) / scale
    assert np.all(err32 < 1e-5), err32
