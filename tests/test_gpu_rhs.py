"""GPU parity of rhs! (FP64 form) against the CPU oracle on identical inputs.

The operators are produced by the oracle and handed to the GPU through the 1-based
CSC entry point (mft_load_csc), as the reference's SparseMatrixCSC would be.
Tolerance (FP64): per variable, max_i |du_gpu - du_ref| <= 1e-12 * max_i s_i with
the condition scale s = |D||F| + sum_d |D_d|'(|eps| |D_d||u|) + gamma |lap|'|lap||u|
(+ gamma |H||u|); states mutated by strong BCs must agree bit for bit.  The Euler cases
run with both arithmetics of the FP64 form's gathers: double-word FP32 ("dw", the
default) and FP64 fused multiply-adds ("dfma"), under the same tolerance.
"""
import numpy as np
import pytest

from helpers import (GAMMA, cond_scale, cyl_bcs, flux_np, ic_bumpy, ic_gradient, load_ops_into,
                     stencil_ops)

pytestmark = pytest.mark.gpu

TOL = 1e-12

CASES = {
    "plain": [],
    "upwind": ["upwind"],
    "rv": ["rv"],
    "tominec": ["tominec"],
    "rv_tominec": ["rv", "tominec"],
    "tominec_rv": ["tominec", "rv"],
    "flyer": ["flyer"],
    "rv_flyer": ["rv", "flyer"],
    "flyer_rv": ["flyer", "rv"],
}


@pytest.fixture(scope="module")
def cyl_ops(oracle, cyl):
    pts = cyl["positions"]
    ops, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=3)
    lap_parts, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=3, order=2)
    lap = oracle.csr_add(lap_parts)
    H_tom = oracle.ata(lap)
    fly_parts, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=5, order=4)
    H_fly = oracle.csr_add(fly_parts)
    return dict(ops=ops, lap=lap, H_tom=H_tom, H_fly=H_fly)


ARITH = ["dw", "dfma"]


def _setup(oracle, gpu_lib, cyl, cyl_ops, case, eq="euler", success_iter=0, approx_du=None,
           arith="auto"):
    from meshfree_gb300 import _lib as L
    pts = cyl["positions"]
    n = pts.shape[0]
    srcs = CASES[case]
    ok = {"rv": oracle.SRC_RV, "upwind": oracle.SRC_UPWIND, "tominec": oracle.SRC_HV_TOMINEC,
          "flyer": oracle.SRC_HV_FLYER}
    gk = {"rv": L.SRC_RV, "upwind": L.SRC_UPWIND, "tominec": L.SRC_HV_TOMINEC,
          "flyer": L.SRC_HV_FLYER}
    dx_min, dx_avg = float(cyl["dx"][0]), float(cyl["dx"][1])
    hv_gamma = 0.0
    hv = None
    if "tominec" in srcs:
        hv_gamma, hv = 1.0 * dx_min ** 4.5, cyl_ops["H_tom"]
    if "flyer" in srcs:
        hv_gamma, hv = 0.1 * dx_min ** 4, cyl_ops["H_fly"]
    V = 4 if eq == "euler" else 1
    if eq == "euler":
        bcs = cyl_bcs(cyl, lambda x, t: ic_gradient(x, t).T)
    else:
        bcs = [(oracle.BC_DIRICHLET, cyl["bidx_1"], cyl["bnrm_1"],
                lambda x, t: np.exp(-((x[:, 0] - 0.3) ** 2 + x[:, 1] ** 2))[:, None]),
               (oracle.BC_DO_NOTHING, cyl["bidx_2"], cyl["bnrm_2"], None)]
    semi = oracle.Semi(pts, cyl_ops["ops"], eq=eq, gamma=GAMMA, adv=(1.0, 0.5), bcs=bcs,
                       sources=[ok[s] for s in srcs], c_rv=1.0, c_uw=1.0, h=dx_avg, hv=hv,
                       hv_gamma=hv_gamma)
    semi.s.success_iter = success_iter
    if approx_du is not None:
        semi.approx_du[:] = approx_du.ravel()
    ctx = L.Context(0)
    ctx.set_option(L.OPT_FP64_ARITH, {"auto": L.ARITH_AUTO, "dw": L.ARITH_DW,
                                      "dfma": L.ARITH_DFMA}[arith])
    ctx.set_points(pts)
    load_ops_into(ctx, cyl_ops["ops"],
                  lap=cyl_ops["lap"] if "tominec" in srcs else None,
                  hv=cyl_ops["H_fly"] if "flyer" in srcs else None)
    ctx.set_equations(L.EQ_EULER2D if eq == "euler" else L.EQ_ADVECTION,
                      [GAMMA] if eq == "euler" else [1.0, 0.5])
    kinds = [b[0] for b in bcs]
    ptr = np.cumsum([0] + [len(b[1]) for b in bcs])
    ctx.set_bcs(kinds, ptr, np.concatenate([b[1] for b in bcs]),
                np.concatenate([b[2] for b in bcs]))
    ctx.set_dirichlet_values(semi.dirichlet_values(0.0))
    params = []
    for s in srcs:
        if s == "rv":
            params.append([1.0, 1.0, dx_avg, 0])
        elif s == "upwind":
            params.append([1.0, dx_avg, 0, 0])
        else:
            params.append([hv_gamma, 0, 0, 0])
    ctx.set_sources([gk[s] for s in srcs], params)
    if success_iter or approx_du is not None:
        ctx.set_rv_state(approx_du if approx_du is not None else np.zeros((V, n)), success_iter)
    return semi, ctx, hv, hv_gamma


def _check(semi, ctx, u0, ops, srcs, hv, hv_gamma, eq="euler", lap_op=None):
    u_ref = u0.copy()
    du_ref, eps_ref, (_mean, norms) = semi.rhs(u_ref, 0.0, want_eps=True, diag=True)
    u_gpu = u0.copy()
    du_gpu = np.empty_like(u0)
    ctx.rhs(du_gpu, u_gpu, 0.0)
    assert np.array_equal(u_gpu, u_ref), "strong-BC mutation of u differs"
    fl = [flux_np(u_ref, 0), flux_np(u_ref, 1)] if eq == "euler" else [
        1.0 * u_ref, 0.5 * u_ref]
    visc = any(s in ("rv", "upwind") for s in srcs)
    scale = cond_scale(ops, u_ref, fluxes=fl, eps=eps_ref if visc else None,
                       lap=lap_op if "tominec" in srcs else None, hv_gamma=hv_gamma,
                       hvop=hv if (hv is not None and "flyer" in srcs) else None)
    err = np.abs(du_gpu - du_ref).max(axis=1) / scale
    assert np.all(err <= TOL), (err, scale)
    if visc:
        eps_gpu = ctx.viscosity()
        # The residual viscosity 0.5 c_rv h^2 max_v |approx_du - du_partial|_v / n_v
        # inherits the partial du's tolerance: |d eps| <= 0.5 c_rv h^2 max_v TOL s_v / n_v
        # (s_v the condition scale), on top of 1e-9 of eps for the FP64 formula itself.
        tol = 1e-9 * np.abs(eps_ref)
        if "rv" in srcs and semi.s.success_iter:
            tol = tol + 0.5 * semi.s.c_rv * semi.s.h ** 2 * np.max(TOL * scale / norms)
        assert np.all(np.abs(eps_gpu - eps_ref) <= tol)
    return err


@pytest.mark.parametrize("arith", ARITH)
@pytest.mark.parametrize("case", list(CASES))
def test_rhs_euler_matches_oracle(oracle, gpu_lib, cyl, cyl_ops, case, arith):
    pts = cyl["positions"]
    u0 = ic_bumpy(pts)
    semi, ctx, hv, g = _setup(oracle, gpu_lib, cyl, cyl_ops, case, arith=arith)
    _check(semi, ctx, u0, cyl_ops["ops"], CASES[case], hv, g, lap_op=cyl_ops["lap"])


@pytest.mark.parametrize("arith", ARITH)
@pytest.mark.parametrize("case", ["rv", "rv_tominec", "tominec_rv", "flyer_rv"])
def test_rhs_residual_viscosity_active(oracle, gpu_lib, cyl, cyl_ops, case, arith):
    """success_iter > 0: eps = min(eps_rv, eps_uw) from a history estimate."""
    pts = cyl["positions"]
    u0 = ic_bumpy(pts)
    semi0, _ctx0, _, _ = _setup(oracle, gpu_lib, cyl, cyl_ops, "plain")
    du_plain = semi0.rhs(u0.copy(), 0.0)
    rng = np.random.default_rng(5)
    approx = np.ascontiguousarray(du_plain * (1 + 0.05 * rng.standard_normal(du_plain.shape)))
    semi, ctx, hv, g = _setup(oracle, gpu_lib, cyl, cyl_ops, case, success_iter=3,
                              approx_du=approx, arith=arith)
    _check(semi, ctx, u0, cyl_ops["ops"], CASES[case], hv, g, lap_op=cyl_ops["lap"])


@pytest.mark.parametrize("scale", [1e-4, 1e-2, 0.05, 0.5, 5.0])
def test_viscosity_selection_matches_oracle(oracle, gpu_lib, cyl, cyl_ops, scale):
    """eps = min(eps_rv, eps_uw) node by node: residual estimates from far below to far
    above the upwind viscosity, and resting nodes (zero momentum, where the bound on
    eps_uw from the speed alone is zero).  The kernel decides eps_rv < eps_uw without
    forming eps_uw where that bound proves it.  Where the oracle takes eps_uw the GPU
    must too (1e-14: same formula up to an ulp); where it takes eps_rv the GPU value must
    be the smaller one and match to 1e-11 / scale (the residual |approx_du - du| is
    ~scale * max|du|, so the rhs! rounding, ~1e-13 of max|du|, cancels into it);
    near-ties (1e-6) are skipped."""
    pts = cyl["positions"]
    n = pts.shape[0]
    u0 = ic_bumpy(pts)
    rng = np.random.default_rng(12)
    rest = rng.choice(n, 40, replace=False)
    u0[1:3, rest] = 0.0
    semi0, _ctx0, _, _ = _setup(oracle, gpu_lib, cyl, cyl_ops, "plain")
    du_plain = semi0.rhs(u0.copy(), 0.0)
    approx = np.ascontiguousarray(du_plain + scale * np.abs(du_plain).max(axis=1, keepdims=True)
                                  * rng.standard_normal(du_plain.shape))
    semi, ctx, _hv, _g = _setup(oracle, gpu_lib, cyl, cyl_ops, "rv", success_iter=2,
                                approx_du=approx)
    semi_uw, _c, _, _ = _setup(oracle, gpu_lib, cyl, cyl_ops, "upwind")
    _du_ref, eps_ref = semi.rhs(u0.copy(), 0.0, want_eps=True)
    _du_uw, eps_uw = semi_uw.rhs(u0.copy(), 0.0, want_eps=True)
    du = np.empty_like(u0)
    ctx.rhs(du, u0.copy(), 0.0)
    eps_gpu = ctx.viscosity()
    took_uw = eps_ref == eps_uw
    tie = np.abs(eps_ref - eps_uw) <= 1e-6 * eps_uw
    a, b = took_uw & ~tie, ~took_uw & ~tie
    assert np.allclose(eps_gpu[a], eps_uw[a], rtol=1e-14, atol=0)
    assert np.all(eps_gpu[b] < eps_uw[b])
    assert np.allclose(eps_gpu[b], eps_ref[b], rtol=1e-11 / scale, atol=0)
    assert b.sum() > 0 or scale >= 5.0


@pytest.mark.parametrize("case", ["plain", "rv", "upwind", "tominec", "rv_tominec"])
def test_rhs_advection_matches_oracle(oracle, gpu_lib, cyl, cyl_ops, case):
    pts = cyl["positions"]
    u0 = np.ascontiguousarray(np.exp(-((pts[:, 0] - 0.5) ** 2 + (pts[:, 1] - 0.4) ** 2) / 0.1)[None, :])
    semi, ctx, hv, g = _setup(oracle, gpu_lib, cyl, cyl_ops, case, eq="advection")
    _check(semi, ctx, u0, cyl_ops["ops"], CASES[case], hv, g, eq="advection",
           lap_op=cyl_ops["lap"])


def test_rhs_divergence_identity_on_gpu(oracle, gpu_lib, cyl, cyl_ops):
    """divergence_test.jl's identity through the GPU rhs! (no BCs, no sources)."""
    from meshfree_gb300 import _lib as L
    pts = cyl["positions"]
    u0 = ic_gradient(pts)
    ctx = L.Context(0)
    ctx.set_points(pts)
    load_ops_into(ctx, cyl_ops["ops"])
    ctx.set_equations(L.EQ_EULER2D, [GAMMA])
    du = np.empty_like(u0)
    ctx.rhs(du, u0.copy(), 0.0)
    Dx, Dy = cyl_ops["ops"][0].to_scipy(), cyl_ops["ops"][1].to_scipy()
    ref = np.stack([-(Dx @ flux_np(u0, 0)[v]) - Dy @ flux_np(u0, 1)[v] for v in range(4)])
    from helpers import isapprox
    assert isapprox(du, ref)


def test_rhs_device_pointers(oracle, gpu_lib, cyl, cyl_ops):
    torch = pytest.importorskip("torch")
    semi, ctx, hv, g = _setup(oracle, gpu_lib, cyl, cyl_ops, "rv")
    u0 = ic_bumpy(cyl["positions"])
    du_h = np.empty_like(u0)
    uh = u0.copy()
    ctx.rhs(du_h, uh, 0.0)
    ud = torch.from_numpy(u0.copy()).cuda()
    dud = torch.empty_like(ud)
    torch.cuda.synchronize()
    ctx.rhs_device(dud.data_ptr(), ud.data_ptr(), 0.0)
    assert np.array_equal(dud.cpu().numpy(), du_h)
    assert np.array_equal(ud.cpu().numpy(), uh)


def test_errors_are_status_codes(gpu_lib):
    from meshfree_gb300 import _lib as L
    ctx = L.Context(0)
    with pytest.raises(L.MFTError) as e:
        ctx.rhs(np.zeros((4, 3)), np.zeros((4, 3)), 0.0)
    assert e.value.code == L.MFT_ERR_STATE
    ctx.set_points(np.random.default_rng(0).uniform(size=(50, 2)))
    with pytest.raises(L.MFTError) as e:
        ctx.knn(51)
    assert e.value.code == L.MFT_ERR_ARG
    with pytest.raises(L.MFTError) as e:
        ctx.load_csc(L.OP_GRAD, 0, np.zeros(51, np.int64), np.zeros(0, np.int64), np.zeros(0))
    assert e.value.code == L.MFT_ERR_ARG
