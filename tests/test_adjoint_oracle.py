"""The oracle's adjoint of rhs! and of the SSP-RK3 trajectory, checked against
centred finite differences of the oracle's own rhs! (CPU only).

Dot-product form: <lam, (f(u + e v) - f(u - e v)) / 2e> must equal
<J(u)^T lam, v> to 1e-7 relative (central-difference truncation ~e^2, rounding
~1e-16/e), on the reference fixture cyl_0_05 with its strong BCs (Dirichlet inlet,
slip walls) and on a periodic vortex cloud."""
import numpy as np
import pytest

from helpers import GAMMA, cyl_bcs, ic_bumpy, ic_gradient, stencil_ops

FD_EPS = 1e-6
TOL_RHS = 1e-7
TOL_TRAJ = 1e-6


@pytest.fixture(scope="module")
def cyl_ops(oracle, cyl):
    pts = cyl["positions"]
    ops, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=3)
    lap_parts, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=3, order=2)
    lap = oracle.csr_add(lap_parts)
    fly_parts, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=5, order=4)
    return dict(ops=ops, H_tom=oracle.ata(lap), H_fly=oracle.csr_add(fly_parts))


def cyl_semi(oracle, cyl, cyl_ops, eq="euler", hv=None):
    pts = cyl["positions"]
    dx_min = float(cyl["dx"][0])
    H, g, src = None, 0.0, []
    if hv == "tominec":
        H, g, src = cyl_ops["H_tom"], 1.0 * dx_min ** 4.5, [oracle.SRC_HV_TOMINEC]
    elif hv == "flyer":
        H, g, src = cyl_ops["H_fly"], 0.1 * dx_min ** 4, [oracle.SRC_HV_FLYER]
    if eq == "euler":
        bcs = cyl_bcs(cyl, lambda x, t: ic_gradient(x, t).T)
    else:
        bcs = [(oracle.BC_DIRICHLET, cyl["bidx_1"], cyl["bnrm_1"],
                lambda x, t: np.exp(-((x[:, 0] - 0.3) ** 2 + x[:, 1] ** 2))[:, None]),
               (oracle.BC_DO_NOTHING, cyl["bidx_2"], cyl["bnrm_2"], None)]
    return oracle.Semi(pts, cyl_ops["ops"], eq=eq, gamma=GAMMA, adv=(1.0, 0.5), bcs=bcs,
                       sources=src, hv=H, hv_gamma=g)


def vortex_semi(oracle, side=16):
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(side, seed=11)
    idx, _, _, _ = oracle.knn(pts, 20, period=per)
    ops, _ = stencil_ops(oracle, pts, idx, period=per)
    return oracle.Semi(pts, ops, eq="euler", gamma=GAMMA), pts, h


def fd_jvp(semi, u, v, t=0.0):
    up = u + FD_EPS * v
    um = u - FD_EPS * v
    return (semi.rhs(up, t) - semi.rhs(um, t)) / (2.0 * FD_EPS)


def dot_check(semi, u, seed):
    g = np.random.default_rng(seed)
    lam = g.standard_normal(u.shape)
    v = g.standard_normal(u.shape) * np.abs(u).max(axis=1, keepdims=True)
    lhs = float(np.sum(lam * fd_jvp(semi, u, v)))
    adj = semi.rhs_adjoint(u, lam)
    rhs = float(np.sum(adj * v))
    return abs(lhs - rhs) / max(abs(lhs), abs(rhs)), adj


@pytest.mark.parametrize("hv", [None, "tominec", "flyer"])
def test_rhs_adjoint_euler_cyl_matches_fd(oracle, cyl, cyl_ops, hv):
    semi = cyl_semi(oracle, cyl, cyl_ops, hv=hv)
    u = ic_bumpy(cyl["positions"])
    err, adj = dot_check(semi, u, 1)
    assert err < TOL_RHS, err
    assert np.isfinite(adj).all()


def test_rhs_adjoint_advection_cyl_matches_fd(oracle, cyl, cyl_ops):
    semi = cyl_semi(oracle, cyl, cyl_ops, eq="advection", hv="tominec")
    x = cyl["positions"]
    u = np.ascontiguousarray(np.sin(2 * x[:, 0] + x[:, 1])[None, :])
    err, _ = dot_check(semi, u, 2)
    assert err < TOL_RHS, err


def test_rhs_adjoint_vortex_matches_fd(oracle):
    from meshfree_gb300 import workloads as W
    semi, pts, _ = vortex_semi(oracle)
    u = W.isentropic_vortex(pts, 0.0)
    err, _ = dot_check(semi, u, 3)
    assert err < TOL_RHS, err


def test_rhs_adjoint_rejects_residual_viscosity(oracle, cyl, cyl_ops):
    pts = cyl["positions"]
    semi = oracle.Semi(pts, cyl_ops["ops"], eq="euler", gamma=GAMMA, sources=[oracle.SRC_RV],
                       h=float(cyl["dx"][1]))
    u = ic_bumpy(pts)
    with pytest.raises(RuntimeError):
        semi.rhs_adjoint(u, u)


def misfit(u, target):
    d = u[0] - target
    return 0.5 * float(d @ d)


@pytest.mark.parametrize("case", ["vortex", "cyl"])
def test_trajectory_adjoint_matches_fd(oracle, cyl, cyl_ops, case):
    """Gradient of J = 0.5 |rho(T) - rho*|^2 w.r.t. u0 after 6 SSP-RK3 steps."""
    from meshfree_gb300 import workloads as W
    if case == "vortex":
        semi, pts, h = vortex_semi(oracle)
        u0 = W.isentropic_vortex(pts, 0.0)
    else:
        semi = cyl_semi(oracle, cyl, cyl_ops, hv="tominec")
        pts = cyl["positions"]
        h = float(cyl["dx"][0])
        u0 = ic_bumpy(pts)
    dt, nsteps = 0.1 * h, 6
    g = np.random.default_rng(7)
    target = u0[0] * (1.0 + 0.01 * g.standard_normal(u0.shape[1]))
    uT, _, rec = oracle.ssprk33_record(semi, u0, 0.0, dt, nsteps)
    # the recording integrator is the plain ssprk33
    ref, _ = oracle.ssprk33(semi, u0, 0.0, dt, nsteps)
    assert np.array_equal(uT, ref)
    lamT = np.zeros_like(uT)
    lamT[0] = uT[0] - target
    grad = oracle.ssprk33_adjoint(semi, rec, dt, lamT)
    v = g.standard_normal(u0.shape) * np.abs(u0).max(axis=1, keepdims=True)
    e = 1e-6
    jp = misfit(oracle.ssprk33(semi, u0 + e * v, 0.0, dt, nsteps)[0], target)
    jm = misfit(oracle.ssprk33(semi, u0 - e * v, 0.0, dt, nsteps)[0], target)
    fd = (jp - jm) / (2 * e)
    ad = float(np.sum(grad * v))
    assert abs(fd - ad) / abs(ad) < TOL_TRAJ, (fd, ad)
