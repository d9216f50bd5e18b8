"""K1 (KNN) and K2 (weights) on the GPU against the CPU oracle: bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ctx(points, period=None):
    from meshfree_gb300 import _lib as L
    ctx = L.Context(0)
    ctx.set_points(points, period)
    return ctx


def _clouds():
    from meshfree_gb300 import workloads as W
    out = {}
    pts, _, _ = W.advection_cloud(32)
    out["advection"] = (pts, None, 35)
    vp, per, _ = W.vortex_cloud(48)
    out["vortex_periodic"] = (vp, per, 35)
    g = np.arange(16) / 16.0
    out["grid_ties"] = (np.ascontiguousarray(np.stack(np.meshgrid(g, g), -1).reshape(-1, 2)), None, 21)
    g2 = (np.arange(12) + 0.5) / 12.0
    out["grid_ties_periodic"] = (np.ascontiguousarray(np.stack(np.meshgrid(g2, g2), -1).reshape(-1, 2)),
                                 (1.0, 1.0), 25)
    out["halton3d"] = (W.halton_points(3000, 3), None, 60)
    return out


CLOUDS = ["cyl", "advection", "vortex_periodic", "grid_ties", "grid_ties_periodic", "halton3d"]


def _get(name, cyl):
    if name == "cyl":
        return cyl["positions"], None, 20
    return _clouds()[name]


@pytest.mark.parametrize("name", CLOUDS)
def test_knn_bit_exact(oracle, gpu_lib, cyl, name):
    pts, per, k = _get(name, cyl)
    idx_o, dist_o, dmin_o, davg_o = oracle.knn(pts, k, period=per)
    ctx = _ctx(pts, per)
    idx_g, dist_g, dmin_g, davg_g = ctx.knn(k, want_dist=True)
    assert np.array_equal(idx_g, idx_o)
    assert np.array_equal(dist_g, dist_o)
    assert dmin_g == dmin_o and davg_g == davg_o


@pytest.mark.parametrize("name,rbf_pow,polydeg,order", [
    ("cyl", 3, 3, 1), ("cyl", 5, 3, 1), ("cyl", 3, 3, 2), ("cyl", 5, 3, 4),
    ("advection", 3, 3, 1), ("vortex_periodic", 3, 3, 1), ("halton3d", 3, 2, 1),
    ("halton3d", 3, 2, 2)])
def test_weights_bit_exact(oracle, gpu_lib, cyl, name, rbf_pow, polydeg, order):
    from meshfree_gb300 import _lib as L
    pts, per, k = _get(name, cyl)
    idx, _, _, _ = oracle.knn(pts, k, period=per)
    n = pts.shape[0]
    rowptr = np.arange(n + 1, dtype=np.int64) * k
    w_o, res_o = oracle.weights(pts, rowptr, idx.ravel(), rbf_pow=rbf_pow, polydeg=polydeg,
                                deriv_order=order, period=per, want_resid=True)
    ctx = _ctx(pts, per)
    ctx.set_stencils(rowptr, idx.ravel())
    w_g, res_g = ctx.weights(L.OP_GRAD, rbf_pow, polydeg, order, want_w=True, want_resid=True)
    assert np.array_equal(w_g, w_o)
    assert res_g < 1e-9


def test_weights_uneven_stencils_one_launch(oracle, gpu_lib):
    """Ragged stencils (interior 35, boundary band 40-60) in one launch."""
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    pts = W.halton_points(4000, 2)
    ks = W.halton_stencil_sizes(pts)
    idx, _, _, _ = oracle.knn(pts, int(ks.max()))
    rowptr = np.concatenate([[0], np.cumsum(ks)]).astype(np.int64)
    cols = np.concatenate([idx[i, :ks[i]] for i in range(pts.shape[0])]).astype(np.int32)
    w_o = oracle.weights(pts, rowptr, cols, rbf_pow=3, polydeg=3, deriv_order=1)
    ctx = _ctx(pts)
    ctx.set_stencils(rowptr, cols)
    w_g, _ = ctx.weights(L.OP_GRAD, 3, 3, 1, want_w=True)
    assert np.array_equal(w_g, w_o)


def test_knn_then_weights_then_rhs(oracle, gpu_lib, cyl):
    """Full GPU setup (KNN -> weights -> rhs!) equals the oracle built the same way."""
    from meshfree_gb300 import _lib as L
    from helpers import GAMMA, ic_bumpy
    pts = cyl["positions"]
    ctx = _ctx(pts)
    idx, _, dmin, davg = ctx.knn(20)
    ctx.weights(L.OP_GRAD, 3, 3, 1)
    ctx.set_equations(L.EQ_EULER2D, [GAMMA])
    u0 = ic_bumpy(pts)
    du = np.empty_like(u0)
    ctx.rhs(du, u0.copy(), 0.0)
    n = pts.shape[0]
    rowptr = np.arange(n + 1, dtype=np.int64) * 20
    w = oracle.weights(pts, rowptr, idx.ravel())
    ops = oracle.operators_from_stencils(n, rowptr, idx.ravel(), w)
    semi = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA)
    ref = semi.rhs(u0.copy(), 0.0)
    assert np.abs(du - ref).max() <= 1e-11 * np.abs(ref).max()
