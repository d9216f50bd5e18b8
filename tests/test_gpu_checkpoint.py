"""Checkpoint / resume of the integrator state (mft_checkpoint_save / _load).

* A run split into two calls on one context, a run resumed in a fresh context from the
  image taken between them, and one uninterrupted call give the same state and time bit
  for bit: the 2D Euler vortex with residual viscosity + HistoryCallback (graph-replayed
  steps), in the FP64 form (both gather arithmetics) and the FP32-apply form, and the
  advection problem with a time-dependent Dirichlet inlet (direct steps).
* solve() with SaveCheckpointCallback, then solve(resume_from=...) to a later time,
  equals one solve() over the whole span.
* A truncated, corrupted or foreign image, or one of another problem size, is refused
  with MFT_ERR_ARG and leaves the context's state as it was.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _vortex(side=24, prec="fp64", arith="auto"):
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(side, seed=3)
    eq = M.CompressibleEulerEquations2D(1.4)
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision=prec, fp64_arith=arith))
    dom = M.PointCloudDomain(solver, pts, period=per)
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom))
    semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                          solver, source_terms=src)
    return M, semi, 0.2 * h


def _advection(side=24):
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, tags, h = W.advection_cloud(side)
    eq = M.LinearScalarAdvectionEquation2D((1.0, 0.5))
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300())
    dom = M.PointCloudDomain(solver, pts, {k: M.BoundaryData(*v) for k, v in tags.items()})
    bcs = {"inflow": M.BoundaryConditionDirichlet(lambda x, t, e: W.gaussian_bump(x, t).T),
           "outflow": M.BoundaryConditionDoNothing()}
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom))
    semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.gaussian_bump(x, t),
                                          solver, boundary_conditions=bcs, source_terms=src)
    return M, semi, 0.2 * h


def _start(semi, order=3):
    ctx = semi.domain.ctx
    ctx.set_state(semi.compute_coefficients(0.0), 0.0)
    ctx.history_init(order)
    return ctx


CASES = {
    "vortex_fp64_dw": lambda: _vortex(arith="dw"),
    "vortex_fp64_dfma": lambda: _vortex(arith="dfma"),
    "vortex_fp32": lambda: _vortex(prec="fp32"),
    "advection_dirichlet": lambda: _advection(),
}


@pytest.mark.parametrize("case", list(CASES))
def test_resume_is_bit_identical(gpu_lib, case):
    make = CASES[case]
    # one call of 12 steps
    M, semi, dt = make()
    ctx = _start(semi)
    ctx.ssprk33(dt, 12)
    u_one, t_one = ctx.get_state()
    ctx.close()
    # 5 + 7 steps on one context, the image taken in between
    M, semi, dt = make()
    ctx = _start(semi)
    ctx.ssprk33(dt, 5)
    image = ctx.checkpoint()
    ctx.ssprk33(dt, 7)
    u_split, t_split = ctx.get_state()
    ctx.close()
    # a fresh context set up the same way, resumed from the image
    M, semi, dt = make()
    ctx = semi.domain.ctx
    ctx.restore(image)
    ctx.ssprk33(dt, 7)
    u_res, t_res = ctx.get_state()
    ctx.close()
    assert t_split == t_one and t_res == t_one
    assert np.array_equal(u_split, u_one)
    assert np.array_equal(u_res, u_one)


def test_solve_with_checkpoint_callback_and_resume(gpu_lib, tmp_path):
    path = tmp_path / "run.ckpt"
    M, semi, dt = _vortex()
    ode = M.semidiscretize(semi, (0.0, 16 * dt))
    ref = M.solve(ode, M.SSPRK33(), dt=dt, callback=M.HistoryCallback(approx_order=3))
    semi.domain.ctx.close()

    M, semi, dt = _vortex()
    ode = M.semidiscretize(semi, (0.0, 8 * dt))
    first = M.solve(ode, M.SSPRK33(), dt=dt,
                    callback=[M.HistoryCallback(approx_order=3),
                              M.SaveCheckpointCallback(3, str(path))])
    semi.domain.ctx.close()
    assert first.nsteps == 8 and path.exists()

    M, semi, dt = _vortex()
    ode = M.semidiscretize(semi, (0.0, 16 * dt))
    sol = M.solve(ode, M.SSPRK33(), dt=dt, callback=M.HistoryCallback(approx_order=3),
                  resume_from=str(path))
    semi.domain.ctx.close()
    assert sol.nsteps == 8
    assert sol.t == ref.t
    assert np.array_equal(sol.u, ref.u)


def test_bad_images_are_refused(gpu_lib):
    from meshfree_gb300 import _lib as L
    M, semi, dt = _vortex()
    ctx = _start(semi)
    ctx.ssprk33(dt, 2)
    image = ctx.checkpoint()
    u_before, t_before = ctx.get_state()
    bad = [image[:-1],                                   # truncated
           image[:200] + bytes([image[200] ^ 1]) + image[201:],   # one bit flipped
           b"NOTACKPT" + image[8:],                      # foreign
           b""]
    for b in bad:
        with pytest.raises(L.MFTError) as e:
            ctx.restore(b)
        assert e.value.code == L.MFT_ERR_ARG
    u_after, t_after = ctx.get_state()
    assert t_after == t_before and np.array_equal(u_after, u_before)
    ctx.close()
    # another problem size
    M, semi2, _ = _vortex(side=20)
    ctx2 = _start(semi2)
    with pytest.raises(L.MFTError) as e:
        ctx2.restore(image)
    assert e.value.code == L.MFT_ERR_ARG
    ctx2.close()
