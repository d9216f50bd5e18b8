"""Batched weights (mft_weights_batch): a 2D Halton cloud with uneven stencils (interior
k = 35, boundary band k in 40..60, degree 3) and a 3D Halton cloud (k in 60..90,
degree 2) solved together, size-bucketed, against the oracle's per-node solves: the
weights are bit-identical (same pivots and the same order of every operation)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ragged(oracle, pts, ks):
    """Each node's ks[i] nearest neighbours (centre first) as CSR rows."""
    idx, _, _, _ = oracle.knn(pts, int(ks.max()))
    rp = np.zeros(pts.shape[0] + 1, dtype=np.int64)
    rp[1:] = np.cumsum(ks)
    cols = np.concatenate([idx[i, :ks[i]] for i in range(pts.shape[0])]).astype(np.int32)
    return rp, cols


def test_batch_2d_3d_uneven_matches_oracle(oracle, gpu_lib):
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    p2 = W.halton_points(3000, 2, seed=11)
    k2 = W.halton_stencil_sizes(p2, seed=11, band=0.05)
    p3 = W.halton_points(700, 3, seed=12)
    k3 = np.random.default_rng(12).integers(60, 91, p3.shape[0])
    rp2, c2 = ragged(oracle, p2, k2)
    rp3, c3 = ragged(oracle, p3, k3)
    assert len(set(k2.tolist())) > 5 and len(set(k3.tolist())) > 5
    ctx = L.Context(0)
    (w2, w3), res = ctx.weights_batch([(p2, rp2, c2, 3, 3, 1), (p3, rp3, c3, 3, 2, 1)],
                                      want_resid=True)
    ref2 = oracle.weights(p2, rp2, c2, rbf_pow=3, polydeg=3, deriv_order=1)
    ref3 = oracle.weights(p3, rp3, c3, rbf_pow=3, polydeg=2, deriv_order=1)
    assert np.array_equal(w2.ravel(), np.asarray(ref2).ravel())
    assert np.array_equal(w3.ravel(), np.asarray(ref3).ravel())
    assert res < 1e-8
    ctx.close()


def test_batch_single_group_equals_context_weights(oracle, gpu_lib):
    """One group through the batch entry gives the context path's weights."""
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(24, seed=2)
    ctx = L.Context(0)
    ctx.set_points(pts)
    idx, _, _, _ = ctx.knn(35)
    w_ctx, _ = ctx.weights(L.OP_GRAD, 3, 3, 1, want_w=True)
    rp = np.arange(pts.shape[0] + 1, dtype=np.int64) * 35
    (w_b,), _ = ctx.weights_batch([(pts, rp, idx.ravel(), 3, 3, 1)])
    assert np.array_equal(np.asarray(w_ctx).ravel(), w_b.ravel())
    ctx.close()
