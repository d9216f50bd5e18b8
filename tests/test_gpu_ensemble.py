"""Ensembles: independent vortex problems of different sizes advanced in one context
(one graph per step) give the same states as each problem run on its own."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _semi(M, W, solver, domain):
    eq = M.CompressibleEulerEquations2D(1.4)
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, domain))
    return M.SemidiscretizationHyperbolic(domain, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                          solver, source_terms=src)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_ensemble_matches_members_run_alone(gpu_lib, prec):
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    sides = [20, 33, 24, 41, 28]
    clouds = [W.vortex_cloud(s, seed=100 + s) for s in sides]
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision=prec))
    ens = M.PointCloudEnsemble(solver, [c[0] for c in clouds], period=(10.0, 10.0))
    semi = _semi(M, W, solver, ens)
    dt = 0.1 * min(c[2] for c in clouds)
    nsteps = 7
    ode = M.semidiscretize(semi, (0.0, nsteps * dt))
    sol = M.solve(ode, M.SSPRK33(), dt=dt, callback=M.HistoryCallback(3))
    for m, (pts, per, h) in enumerate(clouds):
        dom = M.PointCloudDomain(solver, pts, period=per)
        assert np.array_equal(dom.pd.neighbors + ens.offsets[m], ens.pd.neighbors[
            ens.offsets[m]:ens.offsets[m + 1]])
        assert dom.pd.dx_avg == ens.dx_avg[m]
        s1 = _semi(M, W, solver, dom)
        o1 = M.semidiscretize(s1, (0.0, nsteps * dt))
        ref = M.solve(o1, M.SSPRK33(), dt=dt, callback=M.HistoryCallback(3)).u
        got = ens.member(sol.u, m)
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < (1e-11 if prec == "fp64" else 1e-5), (m, err)
