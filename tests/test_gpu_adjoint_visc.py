"""Adjoint of rhs! with the viscosity sources (residual viscosity, upwind viscosity) on the
GPU against forward-mode derivatives (the complex step through the numpy restatement of
the oracle's rhs!, tests/helpers.py), every selection of the viscosity frozen as the
forward evaluation takes it (min(eps_rv, eps_uw), the maximum over variables, the row of
ode_maximum, |.|): the derivative away from selection ties.

* <lam, J v> = <J^T lam, v> on the reference fixture cyl_0_05 (Dirichlet inlet, outlet,
  slip walls) for the upwind source, the residual source before the history has points
  (success_iter 0: eps = eps_uw) and with a history estimate (success_iter > 0), with
  Tominec hyperviscosity after it, in both gather arithmetics; and for advection;
* N = 64 (8 x 8 periodic vortex): J^T lam entry by entry against the dense complex-step
  Jacobian with the residual viscosity active;
* a 4-step SSP-RK3 trajectory with the residual viscosity (its history estimate held
  fixed, as the recording holds it): the reverse sweep against the forward-mode
  derivative of the whole trajectory.
The restatement's real part equals the oracle's rhs! (checked first, 1e-13)."""
import numpy as np
import pytest

from helpers import (GAMMA, cyl_bcs, ic_bumpy, ic_gradient, jacobian_complex, jvp_complex,
                     load_ops_into, rhs_complex, ssprk33_complex, stencil_ops,
                     trajectory_jvp_complex)

pytestmark = pytest.mark.gpu

TOL = 1e-11


@pytest.fixture(scope="module")
def cyl_ops(oracle, cyl):
    pts = cyl["positions"]
    ops, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=3)
    lap_parts, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=3, order=2)
    lap = oracle.csr_add(lap_parts)
    return dict(ops=ops, lap=lap, H=oracle.ata(lap))


def _pair(oracle, gpu_lib, cyl, cyl_ops, srcs, eq="euler", si=0, arith="auto"):
    """The oracle semidiscretization (for the complex step) and a GPU context with the
    same operators, BCs, sources and residual-viscosity state."""
    from meshfree_gb300 import _lib as L
    pts = cyl["positions"]
    n = pts.shape[0]
    dx_min, dx_avg = float(cyl["dx"][0]), float(cyl["dx"][1])
    ok = {"rv": oracle.SRC_RV, "upwind": oracle.SRC_UPWIND, "tominec": oracle.SRC_HV_TOMINEC}
    gk = {"rv": L.SRC_RV, "upwind": L.SRC_UPWIND, "tominec": L.SRC_HV_TOMINEC}
    hv_gamma = 1.0 * dx_min ** 4.5 if "tominec" in srcs else 0.0
    if eq == "euler":
        bcs = cyl_bcs(cyl, lambda x, t: ic_gradient(x, t).T)
        u0 = ic_bumpy(pts)
    else:
        bcs = [(oracle.BC_DIRICHLET, cyl["bidx_1"], cyl["bnrm_1"],
                lambda x, t: np.exp(-((x[:, 0] - 0.3) ** 2 + x[:, 1] ** 2))[:, None]),
               (oracle.BC_DO_NOTHING, cyl["bidx_2"], cyl["bnrm_2"], None)]
        u0 = np.ascontiguousarray(np.exp(-((pts[:, 0] - 0.5) ** 2 + (pts[:, 1] - 0.4) ** 2)
                                         / 0.1)[None, :])
    semi = oracle.Semi(pts, cyl_ops["ops"], eq=eq, gamma=GAMMA, adv=(1.0, 0.5), bcs=bcs,
                       sources=[ok[s] for s in srcs], c_rv=1.0, c_uw=1.0, h=dx_avg,
                       hv=cyl_ops["H"] if "tominec" in srcs else None, hv_gamma=hv_gamma)
    V = u0.shape[0]
    approx = np.zeros((V, n))
    if si:
        plain = oracle.Semi(pts, cyl_ops["ops"], eq=eq, gamma=GAMMA, adv=(1.0, 0.5), bcs=bcs)
        du = plain.rhs(u0.copy(), 0.0)
        rng = np.random.default_rng(5)
        approx = np.ascontiguousarray(du * (1 + 0.05 * rng.standard_normal(du.shape)))
        semi.approx_du[:] = approx.ravel()
        semi.s.success_iter = si
    ctx = L.Context(0)
    ctx.set_option(L.OPT_FP64_ARITH, {"auto": L.ARITH_AUTO, "dw": L.ARITH_DW,
                                      "dfma": L.ARITH_DFMA}[arith])
    ctx.set_points(pts)
    load_ops_into(ctx, cyl_ops["ops"], lap=cyl_ops["lap"] if "tominec" in srcs else None)
    ctx.set_equations(L.EQ_EULER2D if eq == "euler" else L.EQ_ADVECTION,
                      [GAMMA] if eq == "euler" else [1.0, 0.5])
    kinds = [b[0] for b in bcs]
    ptr = np.cumsum([0] + [len(b[1]) for b in bcs])
    ctx.set_bcs(kinds, ptr, np.concatenate([b[1] for b in bcs]),
                np.concatenate([b[2] for b in bcs]))
    ctx.set_dirichlet_values(semi.dirichlet_values(0.0))
    params = []
    for s in srcs:
        params.append([1.0, 1.0, dx_avg, 0] if s == "rv" else
                      ([1.0, dx_avg, 0, 0] if s == "upwind" else [hv_gamma, 0, 0, 0]))
    ctx.set_sources([gk[s] for s in srcs], params)
    ctx.set_rv_state(approx, si)
    return semi, ctx, u0


def _dot_err(semi, ctx, u, seed):
    g = np.random.default_rng(seed)
    lam = g.standard_normal(u.shape)
    v = g.standard_normal(u.shape) * np.abs(u).max(axis=1, keepdims=True)
    lhs = float(np.sum(lam * jvp_complex(semi, u, v)))
    rhs = float(np.sum(ctx.rhs_adjoint(lam, u, 0.0) * v))
    return abs(lhs - rhs) / max(abs(lhs), abs(rhs))


CASES = {
    "upwind": (["upwind"], 0),
    "rv_cold": (["rv"], 0),
    "rv": (["rv"], 3),
    "rv_tominec": (["rv", "tominec"], 3),
}


@pytest.mark.parametrize("arith", ["dw", "dfma"])
@pytest.mark.parametrize("case", list(CASES))
def test_visc_adjoint_matches_forward_mode(oracle, gpu_lib, cyl, cyl_ops, case, arith):
    srcs, si = CASES[case]
    semi, ctx, u = _pair(oracle, gpu_lib, cyl, cyl_ops, srcs, si=si, arith=arith)
    ref = semi.rhs(u.copy(), 0.0)
    assert np.abs(rhs_complex(semi, u).real - ref).max() <= 1e-13 * np.abs(ref).max()
    for seed in (1, 2):
        err = _dot_err(semi, ctx, u, seed)
        assert err < TOL, err
    ctx.close()


def test_visc_adjoint_advection(oracle, gpu_lib, cyl, cyl_ops):
    semi, ctx, u = _pair(oracle, gpu_lib, cyl, cyl_ops, ["rv"], eq="advection", si=2)
    err = _dot_err(semi, ctx, u, 3)
    assert err < TOL, err
    ctx.close()


def _vortex_pair(oracle, side, si):
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    pts, per, _h = W.vortex_cloud(side, seed=11)
    idx, _, _, davg = oracle.knn(pts, 20, period=per)
    ops, _ = stencil_ops(oracle, pts, idx, period=per)
    semi = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA, sources=(oracle.SRC_RV,), h=davg)
    u = W.isentropic_vortex(pts, 0.0)
    plain = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA)
    du = plain.rhs(u.copy(), 0.0)
    rng = np.random.default_rng(7)
    approx = np.ascontiguousarray(du * (1 + 0.1 * rng.standard_normal(du.shape)))
    semi.approx_du[:] = approx.ravel()
    semi.s.success_iter = si
    ctx = L.Context(0)
    ctx.set_points(pts, per)
    load_ops_into(ctx, ops)
    ctx.set_equations(L.EQ_EULER2D, [GAMMA])
    ctx.set_sources([L.SRC_RV], [[1.0, 1.0, davg, 0]])
    ctx.set_rv_state(approx, si)
    return semi, ctx, u


def test_visc_adjoint_full_jacobian_small(oracle, gpu_lib):
    semi, ctx, u = _vortex_pair(oracle, 8, 2)
    J = jacobian_complex(semi, u)
    g = np.random.default_rng(5)
    for _ in range(3):
        lam = g.standard_normal(u.shape)
        ref = (J.T @ lam.ravel()).reshape(u.shape)
        adj = ctx.rhs_adjoint(lam, u, 0.0)
        scale = (np.abs(J).T @ np.abs(lam).ravel()).max()
        assert np.abs(adj - ref).max() <= 1e-12 * scale
    ctx.close()


def test_visc_trajectory_adjoint_matches_forward_mode(oracle, gpu_lib):
    semi, ctx, u0 = _vortex_pair(oracle, 12, 3)
    dt, nsteps = 0.02, 4
    ctx.set_state(u0, 0.0)
    ctx.ssprk33_record(dt, nsteps, 0)
    uT = ctx.get_state()[0]
    assert np.abs(ssprk33_complex(semi, u0, 0.0, dt, nsteps).real - uT).max() <= \
        1e-12 * np.abs(uT).max()
    g = np.random.default_rng(8)
    lamT = g.standard_normal(u0.shape)
    v = g.standard_normal(u0.shape) * np.abs(u0).max(axis=1, keepdims=True)
    lam0 = ctx.ssprk33_adjoint(lamT)
    lhs = float(np.sum(lamT * trajectory_jvp_complex(semi, u0, v, dt, nsteps)))
    rhs = float(np.sum(lam0 * v))
    assert abs(lhs - rhs) / abs(rhs) < TOL, (lhs, rhs)
    ctx.close()
