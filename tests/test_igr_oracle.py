"""The oracle's IGR source (src/sources/IGR.jl:17-239): it changes only the momentum
rows of du, by -Dx sigma and -Dy sigma, and sigma is the conjugate-gradient solution of
(rho^-1 - alpha (Dx rho^-1 Dx + Dy rho^-1 Dy)) sigma = alpha (tr(Du)^2 + tr(Du^2))
(CPU only)."""
import numpy as np

from helpers import stencil_ops


def _vortex(oracle):
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(32, seed=3)
    idx, _, _, _ = oracle.knn(pts, 35, period=per)
    ops, _ = stencil_ops(oracle, pts, idx, period=per)
    return pts, ops, h, W.isentropic_vortex(pts, 0.0)


def test_igr_changes_momentum_rows_only(oracle):
    pts, ops, h, u = _vortex(oracle)
    s = oracle.Semi(pts, ops, eq="euler", gamma=1.4, sources=[oracle.SRC_IGR], igr_alpha=h * h)
    s0 = oracle.Semi(pts, ops, eq="euler", gamma=1.4)
    du = s.rhs(u.copy(), 0.0)
    du0 = s0.rhs(u.copy(), 0.0)
    assert np.array_equal(du[0], du0[0]) and np.array_equal(du[3], du0[3])
    Dx, Dy = ops[0].to_scipy(), ops[1].to_scipy()
    sig = s.igr_sigma
    assert np.allclose(du[1] - du0[1], -(Dx @ sig), rtol=0, atol=1e-12 * np.abs(du0).max())
    assert np.allclose(du[2] - du0[2], -(Dy @ sig), rtol=0, atol=1e-12 * np.abs(du0).max())


def test_igr_sigma_solves_the_regularisation_system(oracle):
    pts, ops, h, u = _vortex(oracle)
    a = h * h
    s = oracle.Semi(pts, ops, eq="euler", gamma=1.4, sources=[oracle.SRC_IGR], igr_alpha=a)
    s.rhs(u.copy(), 0.0)
    sig = s.igr_sigma
    Dx, Dy = ops[0].to_scipy(), ops[1].to_scipy()
    rinv = 1.0 / u[0]
    v1, v2 = u[1] / u[0], u[2] / u[0]
    tr = Dx @ u[0] + Dy @ v1            # tr(Du) as the reference forms it
    b = a * (tr * tr + (Dx @ v1) ** 2 + 2 * (Dy @ v1) * (Dx @ v2) + (Dy @ v2) ** 2)
    A = rinv * sig - a * (Dx @ (rinv * (Dx @ sig)) + Dy @ (rinv * (Dy @ sig)))
    assert np.linalg.norm(A - b) / np.linalg.norm(b) < 1e-4
