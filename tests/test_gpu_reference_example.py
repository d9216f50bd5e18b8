"""The reference's own example set-up (rbfsolver_test.jl): the Medusa cylinder cloud
(test/data/cyl_0_05), 2D Euler with Trixi's initial_condition_constant, Dirichlet inlet,
do-nothing outlet, slip walls elsewhere, SourceTerms(hv = Tominec (c = 1), rv = residual
viscosity (c = 1)), HistoryCallback(approx_order = 3).  The example integrates with
adaptive SSPRK43; here both sides take the same fixed SSP-RK3 steps.  GPU trajectory vs
the oracle's: 1e-11 relative after 5 steps; after 25 steps of the start-up transient,
within 10x of the oracle's own response to a 1e-15 perturbation of u0."""
import numpy as np
import pytest

from helpers import GAMMA, cyl_bcs, load_ops_into, stencil_ops

pytestmark = pytest.mark.gpu

U_CONST = np.array([1.0, 0.1, -0.2, 10.0])  # Trixi initial_condition_constant (2D Euler)


def test_cylinder_example_trajectory(oracle, gpu_lib, cyl):
    from meshfree_gb300 import _lib as L
    pts = cyl["positions"]
    n = pts.shape[0]
    ops, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=3)
    lap_parts, _ = stencil_ops(oracle, pts, cyl["knn"], rbf_pow=3, order=2)
    lap = oracle.csr_add(lap_parts)
    H = oracle.ata(lap)
    dx_min, dx_avg = float(cyl["dx"][0]), float(cyl["dx"][1])
    gamma_hv = 1.0 * dx_min ** 4.5
    const = lambda x, t: np.tile(U_CONST, (x.shape[0], 1))
    bcs = cyl_bcs(cyl, const)
    semi = oracle.Semi(pts, ops, eq="euler", gamma=GAMMA, bcs=bcs,
                       sources=[oracle.SRC_HV_TOMINEC, oracle.SRC_RV], c_rv=1.0, c_uw=1.0,
                       h=dx_avg, hv=H, hv_gamma=gamma_hv)
    ctx = L.Context(0)
    ctx.set_points(pts)
    load_ops_into(ctx, ops, lap=lap)
    ctx.set_equations(L.EQ_EULER2D, [GAMMA])
    ptr = np.cumsum([0] + [len(b[1]) for b in bcs])
    ctx.set_bcs([b[0] for b in bcs], ptr, np.concatenate([b[1] for b in bcs]),
                np.concatenate([b[2] for b in bcs]))
    ctx.set_dirichlet_values(semi.dirichlet_values(0.0))
    ctx.set_sources([L.SRC_HV_TOMINEC, L.SRC_RV], [[gamma_hv, 0, 0, 0], [1.0, 1.0, dx_avg, 0]])
    u0 = np.ascontiguousarray(np.tile(U_CONST[:, None], (1, n)))
    dt = 0.05 * dx_avg

    def oracle_run(u, nsteps):
        return oracle.ssprk33(semi, u, 0.0, dt, nsteps, history=oracle.History(semi, 3))[0]

    def gpu_run(nsteps):
        ctx.history_init(3)
        ctx.set_state(u0, 0.0)
        ctx.ssprk33(dt, nsteps, use_graph=True)
        return ctx.get_state()[0]

    # before the residual viscosity switches on strongly: rounding-level agreement
    ref5 = oracle_run(u0, 5)
    assert np.abs(gpu_run(5) - ref5).max() / np.abs(ref5).max() < 1e-11
    # the start-up transient then amplifies rounding differences (a 1e-15 perturbation of
    # u0 grows to ~3e-8 in the oracle itself after 25 steps): the GPU must stay within
    # 10x of the oracle's own sensitivity
    ref = oracle_run(u0, 25)
    noise = np.random.default_rng(0).uniform(-1.0, 1.0, u0.shape)
    pert = oracle_run(np.ascontiguousarray(u0 * (1.0 + 1e-15 * noise)), 25)
    sens = np.abs(pert - ref).max() / np.abs(ref).max()
    got = gpu_run(25)
    assert np.isfinite(got).all()
    assert np.abs(ref - u0).max() > 1e-6          # the walls set the flow in motion
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err <= 10.0 * max(sens, 1e-13), (err, sens)
    ctx.close()
