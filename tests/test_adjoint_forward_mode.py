"""The oracle's adjoint of rhs! against forward-mode derivatives of rhs! (CPU only).

Forward mode here is the complex step through a numpy restatement of the oracle's rhs!
(tests/helpers.py: rhs_complex), the counterpart of checking the adjoint against
ForwardDiff through the reference rhs! at small N.  Unlike centred differences it has
no truncation or cancellation error, so the checks hold to rounding:
  * the restatement's real part equals the oracle's rhs! (1e-13 of max |du|);
  * <lam, J v> = <J^T lam, v> to 1e-12 relative on the reference fixture cyl_0_05
    (Dirichlet inlet, outlet, three slip walls) with no / Tominec / Flyer
    hyperviscosity, for the advection equation, and on a periodic vortex;
  * at N = 64 the full Jacobian (one complex-step column per unknown) gives J^T lam
    equal to the oracle's adjoint to 1e-12 of the product's scale;
  * the reverse sweep over a recorded SSP-RK3 trajectory matches the forward-mode
    derivative of the whole trajectory, <lam_T, (du_T/du_0) v> = <lam_0, v>, to 1e-12."""
import numpy as np
import pytest

from helpers import (GAMMA, cyl_bcs, ic_bumpy, ic_gradient, jacobian_complex, jvp_complex,
                     rhs_complex, ssprk33_complex, stencil_ops, trajectory_jvp_complex)

TOL = 1e-12


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


def vortex_semi(oracle, side):
    from meshfree_gb300 import workloads as W
    pts, per, _h = W.vortex_cloud(side, seed=11)
    idx, _, _, _ = oracle.knn(pts, 20, period=per)
    ops, _ = stencil_ops(oracle, pts, idx, period=per)
    return oracle.Semi(pts, ops, eq="euler", gamma=GAMMA), pts


def dot_err(semi, u, seed):
    g = np.random.default_rng(seed)
    lam = g.standard_normal(u.shape)
    v = g.standard_normal(u.shape) * np.abs(u).max(axis=1, keepdims=True)
    lhs = float(np.sum(lam * jvp_complex(semi, u, v)))
    rhs = float(np.sum(semi.rhs_adjoint(u, lam) * v))
    return abs(lhs - rhs) / max(abs(lhs), abs(rhs))


@pytest.mark.parametrize("hv", [None, "tominec", "flyer"])
def test_restatement_equals_oracle_rhs(oracle, cyl, cyl_ops, hv):
    semi = cyl_semi(oracle, cyl, cyl_ops, hv=hv)
    u = ic_bumpy(cyl["positions"])
    ref = semi.rhs(u.copy(), 0.0)
    got = rhs_complex(semi, u)
    assert np.abs(got.imag).max() == 0.0
    assert np.abs(got.real - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("hv", [None, "tominec", "flyer"])
def test_adjoint_matches_forward_mode_euler_cyl(oracle, cyl, cyl_ops, hv):
    semi = cyl_semi(oracle, cyl, cyl_ops, hv=hv)
    u = ic_bumpy(cyl["positions"])
    for seed in (1, 2):
        err = dot_err(semi, u, seed)
        assert err < TOL, err


def test_adjoint_matches_forward_mode_advection_cyl(oracle, cyl, cyl_ops):
    semi = cyl_semi(oracle, cyl, cyl_ops, eq="advection", hv="tominec")
    x = cyl["positions"]
    u = np.ascontiguousarray(np.sin(2 * x[:, 0] + x[:, 1])[None, :])
    assert np.abs(rhs_complex(semi, u).real - semi.rhs(u.copy(), 0.0)).max() <= \
        1e-13 * np.abs(semi.rhs(u.copy(), 0.0)).max()
    err = dot_err(semi, u, 3)
    assert err < TOL, err


def test_adjoint_matches_forward_mode_vortex(oracle):
    from meshfree_gb300 import workloads as W
    semi, pts = vortex_semi(oracle, 16)
    u = W.isentropic_vortex(pts, 0.0)
    err = dot_err(semi, u, 4)
    assert err < TOL, err


def test_full_jacobian_transpose_small(oracle):
    """N = 64 (8 x 8 vortex cloud, 256 unknowns): J^T lam from the dense complex-step
    Jacobian equals the oracle's adjoint entry by entry."""
    from meshfree_gb300 import workloads as W
    semi, pts = vortex_semi(oracle, 8)
    u = W.isentropic_vortex(pts, 0.0)
    J = jacobian_complex(semi, u)
    g = np.random.default_rng(5)
    for _ in range(3):
        lam = g.standard_normal(u.shape)
        ref = (J.T @ lam.ravel()).reshape(u.shape)
        adj = semi.rhs_adjoint(u, lam)
        scale = (np.abs(J).T @ np.abs(lam).ravel()).max()
        assert np.abs(adj - ref).max() <= TOL * scale


@pytest.mark.parametrize("case", ["cyl", "vortex"])
def test_trajectory_adjoint_matches_forward_mode(oracle, cyl, cyl_ops, case):
    from meshfree_gb300 import workloads as W
    if case == "cyl":
        semi = cyl_semi(oracle, cyl, cyl_ops, hv="tominec")
        u0 = ic_bumpy(cyl["positions"])
        dt = 0.1 * float(cyl["dx"][0])
    else:
        semi, pts = vortex_semi(oracle, 16)
        u0 = W.isentropic_vortex(pts, 0.0)
        dt = 0.02
    nsteps = 6
    uT, _, rec = oracle.ssprk33_record(semi, u0, 0.0, dt, nsteps)
    assert np.abs(ssprk33_complex(semi, u0, 0.0, dt, nsteps).real - uT).max() <= \
        1e-12 * np.abs(uT).max()
    g = np.random.default_rng(8)
    lamT = g.standard_normal(u0.shape)
    v = g.standard_normal(u0.shape) * np.abs(u0).max(axis=1, keepdims=True)
    lam0 = oracle.ssprk33_adjoint(semi, rec, dt, lamT)
    lhs = float(np.sum(lamT * trajectory_jvp_complex(semi, u0, v, dt, nsteps)))
    rhs = float(np.sum(lam0 * v))
    assert abs(lhs - rhs) / abs(rhs) < TOL, (lhs, rhs)


@pytest.mark.parametrize("src,si", [("upwind", 0), ("rv", 0), ("rv", 3)])
def test_restatement_with_viscosity_equals_oracle_rhs(oracle, cyl, cyl_ops, src, si):
    """The complex-step restatement with a viscosity source (every selection taken on
    the real parts) has the oracle's rhs! as its real part."""
    pts = cyl["positions"]
    kind = oracle.SRC_RV if src == "rv" else oracle.SRC_UPWIND
    bcs = cyl_bcs(cyl, lambda x, t: ic_gradient(x, t).T)
    semi = oracle.Semi(pts, cyl_ops["ops"], eq="euler", gamma=GAMMA, bcs=bcs, sources=(kind,),
                       c_rv=1.0, c_uw=1.0, h=float(cyl["dx"][1]))
    u = ic_bumpy(pts)
    if si:
        plain = oracle.Semi(pts, cyl_ops["ops"], eq="euler", gamma=GAMMA, bcs=bcs)
        du = plain.rhs(u.copy(), 0.0)
        semi.approx_du[:] = (du * (1 + 0.05 * np.random.default_rng(5).standard_normal(
            du.shape))).ravel()
        semi.s.success_iter = si
    ref = semi.rhs(u.copy(), 0.0)
    got = rhs_complex(semi, u)
    assert np.abs(got.imag).max() == 0.0
    assert np.abs(got.real - ref).max() <= 1e-13 * np.abs(ref).max()
