"""Status codes of the engine on invalid use (a context needs a device): every failure is
an MFT_ERR_* code with a message, nothing aborts, and the context stays usable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ctx():
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(16, seed=4)
    ctx = L.Context(0)
    ctx.set_points(pts, per)
    ctx.knn(20)
    ctx.weights(L.OP_GRAD, 3, 3, 1)
    ctx.set_equations(L.EQ_EULER2D, [1.4])
    ctx.set_bcs([], [0], np.zeros(0, np.int32), None)
    ctx.set_sources([], [])
    return L, W, ctx, pts


def _code(fn):
    from meshfree_gb300._lib import MFTError
    with pytest.raises(MFTError) as e:
        fn()
    return e.value.code


def test_invalid_arguments_return_status_codes(gpu_lib):
    L, W, ctx, pts = _ctx()
    u = W.isentropic_vortex(pts, 0.0)
    assert _code(lambda: ctx.set_sources([9], [[0, 0, 0, 0]])) == L.MFT_ERR_ARG
    assert _code(lambda: ctx.set_limiter([7], [0.1])) == L.MFT_ERR_ARG
    assert _code(lambda: ctx.set_limiter([0], [float("nan")])) == L.MFT_ERR_ARG
    assert _code(lambda: ctx.ssprk33(-1.0, 1)) in (L.MFT_ERR_ARG, L.MFT_ERR_STATE)
    assert _code(lambda: ctx.ssprk33_adjoint(u)) == L.MFT_ERR_STATE     # nothing recorded
    bad_rp = np.array([0, 3, 2], dtype=np.int64)
    assert _code(lambda: ctx.weights_batch([(pts[:2], bad_rp, np.zeros(3, np.int32), 3, 3, 1)])) \
        == L.MFT_ERR_ARG
    # the context still works after the refusals
    du = np.empty_like(u)
    ctx.rhs(du, u.copy(), 0.0)
    assert np.isfinite(du).all()
    ctx.close()


def test_unsupported_combinations(gpu_lib):
    L, W, ctx, pts = _ctx()
    u = W.isentropic_vortex(pts, 0.0)
    ctx.set_sources([L.SRC_IGR], [[0.01, 20.0, 0.0, 0.0]])
    assert _code(lambda: ctx.rhs_adjoint(u, u)) == L.MFT_ERR_UNSUPPORTED   # IGR: no adjoint
    ctx.set_sources([], [])
    ctx.set_equations(L.EQ_ADVECTION, [1.0, 0.5])
    assert _code(lambda: ctx.set_limiter([0], [0.1])) == L.MFT_ERR_UNSUPPORTED
    ctx.close()


def test_bounded_wait_reports_timeout_and_context_survives(gpu_lib):
    """The error path of the staged gathers' bounded mbarrier waits, without a fault: a
    warp waits on a barrier that nothing completes, gives up after 1000 polls and the
    host reads MFT_ERR_TIMEOUT from the device error word; the error word is cleared and
    the context keeps working."""
    L, W, ctx, pts = _ctx()
    assert ctx.selftest_bounded_wait(1000) == L.MFT_ERR_TIMEOUT
    assert ctx.selftest_bounded_wait(1) == L.MFT_ERR_TIMEOUT
    assert _code(lambda: ctx.check(ctx.lib.mft_selftest_bounded_wait(ctx.h, 0))) == L.MFT_ERR_ARG
    u = W.isentropic_vortex(pts, 0.0)
    du = np.empty_like(u)
    ctx.rhs(du, u.copy(), 0.0)
    assert np.isfinite(du).all()
    ctx.close()


def test_nonfinite_state_is_reported(gpu_lib):
    """A NaN in the state handed to rhs! (and to SSP-RK3 stepping, direct and graph
    replay) makes the call return MFT_ERR_NONFINITE: the stage epilogue flags NaN or
    infinite outputs in the device error word, which the host reads at the end of the
    call.  The outputs are still written, the word is cleared, and the context keeps
    working with a finite state."""
    L, W, ctx, pts = _ctx()
    u = W.isentropic_vortex(pts, 0.0)
    bad = u.copy()
    bad[0, 5] = float("nan")
    du = np.empty_like(u)
    assert _code(lambda: ctx.rhs(du, bad.copy(), 0.0)) == L.MFT_ERR_NONFINITE
    assert np.isnan(du).any()
    ctx.rhs(du, u.copy(), 0.0)
    assert np.isfinite(du).all()
    for graph in (False, True):
        ctx.set_state(bad, 0.0)
        assert _code(lambda: ctx.ssprk33(1e-3, 2, use_graph=graph)) == L.MFT_ERR_NONFINITE
        ctx.set_state(u, 0.0)
        ctx.ssprk33(1e-3, 2, use_graph=graph)
        assert np.isfinite(ctx.get_state()[0]).all()
    ctx.close()
