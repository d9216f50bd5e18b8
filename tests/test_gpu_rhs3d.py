"""rhs! on 3D point clouds against the oracle: CompressibleEulerEquations3D on a periodic
jittered cube (both gather arithmetics: double-word and FP64 FMAs) and 3D scalar advection
with a time-dependent Dirichlet inflow (the plain flux divergence of calc_fluxes! over
D_x, D_y, D_z, rbfsolver.jl:247-265, with the strong BCs).  GPU KNN and weights (PHS r^3 + degree 2, k = 30) bit-identical to the oracle's; one
rhs! within 1e-12 of the condition scale; SSP-RK3 trajectories within 1e-10.  The
combinations the reference writes only for 2D Euler (viscosity sources, slip walls) and
the FP32 form and adjoint are refused with MFT_ERR_UNSUPPORTED."""
import numpy as np
import pytest

from helpers import GAMMA, cond_scale, flux3d_np, stencil_ops

pytestmark = pytest.mark.gpu

SIDE, K, DEG = 10, 30, 2
PER = (1.0, 1.0, 1.0)


@pytest.fixture(scope="module")
def cube(oracle):
    from meshfree_gb300 import workloads as W
    pts, h = W.jittered_grid3(SIDE, seed=7)
    idx, _, _, _ = oracle.knn(pts, K, period=PER)
    ops, w = stencil_ops(oracle, pts, idx, polydeg=DEG, period=PER)
    return pts, h, idx, ops, w


def _euler_semi(pts, prec="fp64", sources=None, arith="auto"):
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    basis = M.PointCloudBasis(M.Point3D(), DEG, nv=K)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision=prec, fp64_arith=arith))
    dom = M.PointCloudDomain(solver, pts, period=PER)
    eq = M.CompressibleEulerEquations3D(GAMMA)
    semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.euler3d_wave(x), solver,
                                          source_terms=sources)
    return M, dom, semi


@pytest.mark.parametrize("arith", ["dw", "dfma"])
def test_euler3d_rhs_and_steps_match_oracle(oracle, gpu_lib, cube, arith):
    from meshfree_gb300 import workloads as W
    pts, h, idx, ops, _w = cube
    M, dom, semi = _euler_semi(pts, arith=arith)
    assert np.array_equal(dom.pd.neighbors, idx)
    osemi = oracle.Semi(pts, ops, eq="euler3d", gamma=GAMMA)
    u0 = W.euler3d_wave(pts)
    ref = osemi.rhs(u0.copy(), 0.0)
    du = np.empty_like(u0)
    dom.ctx.rhs(du, u0.copy(), 0.0)
    scale = cond_scale(ops, u0, fluxes=[flux3d_np(u0, d) for d in range(3)])
    err = np.abs(du - ref).max(axis=1) / scale
    assert np.all(err <= 1e-12), err
    dt, nsteps = 0.1 * h, 8
    ode = M.semidiscretize(semi, (0.0, nsteps * dt))
    sol = M.solve(ode, M.SSPRK33(), dt=dt)
    u_ref, t_ref = oracle.ssprk33(osemi, ode.u0, 0.0, dt, nsteps)
    assert abs(sol.t - t_ref) <= 1e-14
    rel = np.abs(sol.u - u_ref).max(axis=1) / np.abs(u_ref).max(axis=1)
    assert np.all(rel < 1e-10), rel
    dom.ctx.close()


def test_advection3d_dirichlet_matches_oracle(oracle, gpu_lib, cube):
    import meshfree_gb300 as M
    pts, h, idx, ops, _w = cube
    a = (1.0, 0.5, -0.25)
    inflow = np.where(pts[:, 0] < 0.1)[0]
    normals = np.tile([-1.0, 0.0, 0.0], (inflow.size, 1))
    g = lambda x, t: np.exp(-np.sum((x - 0.5 - np.array(a) * t) ** 2, axis=1) / 0.05)
    basis = M.PointCloudBasis(M.Point3D(), DEG, nv=K)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300())
    dom = M.PointCloudDomain(solver, pts, {"inflow": M.BoundaryData(inflow, normals)}, period=PER)
    eq = M.LinearScalarAdvectionEquation3D(a)
    semi = M.SemidiscretizationHyperbolic(
        dom, eq, lambda x, t, e: g(x, t)[None, :], solver,
        boundary_conditions={"inflow": M.BoundaryConditionDirichlet(lambda x, t, e: g(x, t)[:, None])})
    osemi = oracle.Semi(pts, ops, eq="advection", adv=a,
                        bcs=[(oracle.BC_DIRICHLET, inflow.astype(np.int32), normals,
                              lambda x, t: g(x, t)[:, None])])
    u0 = semi.compute_coefficients(0.0)
    ref_u = u0.copy()
    ref = osemi.rhs(ref_u, 0.0)
    gu = u0.copy()
    du = np.empty_like(u0)
    dom.ctx.rhs(du, gu, 0.0)
    assert np.array_equal(gu, ref_u)
    scale = cond_scale(ops, ref_u, fluxes=[a[d] * ref_u for d in range(3)])
    err = np.abs(du - ref).max(axis=1) / scale
    assert np.all(err <= 1e-12), err
    dt, nsteps = 0.1 * h, 6
    ode = M.semidiscretize(semi, (0.0, nsteps * dt))
    sol = M.solve(ode, M.SSPRK33(), dt=dt)
    u_ref, _ = oracle.ssprk33(osemi, ode.u0, 0.0, dt, nsteps)
    rel = np.abs(sol.u - u_ref).max() / np.abs(u_ref).max()
    assert rel < 1e-10, rel
    dom.ctx.close()


def test_3d_unsupported_combinations(oracle, gpu_lib, cube):
    import meshfree_gb300 as M
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    pts, h, idx, ops, _w = cube
    u0 = W.euler3d_wave(pts)
    du = np.empty_like(u0)
    # viscosity source (written for CompressibleEulerEquations2D in the reference)
    M_, dom, semi = _euler_semi(pts)
    dom.ctx.set_sources([L.SRC_RV], [[1.0, 1.0, h, 0]])
    with pytest.raises(L.MFTError) as e:
        dom.ctx.rhs(du, u0.copy(), 0.0)
    assert e.value.code == L.MFT_ERR_UNSUPPORTED
    dom.ctx.close()
    # slip wall
    M_, dom, semi = _euler_semi(pts)
    wall = np.arange(5, dtype=np.int32)
    dom.ctx.set_bcs([L.BC_SLIP_WALL], [0, 5], wall, np.tile([1.0, 0.0, 0.0], (5, 1)))
    with pytest.raises(L.MFTError) as e:
        dom.ctx.rhs(du, u0.copy(), 0.0)
    assert e.value.code == L.MFT_ERR_UNSUPPORTED
    dom.ctx.close()
    # FP32 form and adjoint
    M_, dom, semi = _euler_semi(pts, prec="fp32")
    with pytest.raises(L.MFTError) as e:
        dom.ctx.rhs(du, u0.copy(), 0.0)
    assert e.value.code == L.MFT_ERR_UNSUPPORTED
    dom.ctx.close()
    M_, dom, semi = _euler_semi(pts)
    with pytest.raises(L.MFTError) as e:
        dom.ctx.rhs_adjoint(u0, u0, 0.0)
    assert e.value.code == L.MFT_ERR_UNSUPPORTED
    dom.ctx.close()


def test_euler3d_staged_gather_equals_direct(gpu_lib):
    """The double-word 3D gather with each 128-row group's neighbour records staged in
    shared memory equals the direct gather bit for bit: a shuffled 14^3 cube in Morton row
    order (every group staged) and in node order (groups of random nodes: none staged),
    both with the rows' entries in ascending-column order, so that each node's sum runs in
    the same order."""
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    pts, h = W.jittered_grid3(14, seed=11)
    rng = np.random.default_rng(2)
    pts = np.ascontiguousarray(pts[rng.permutation(pts.shape[0])])
    u0 = W.euler3d_wave(pts)
    out = {}
    for order in (1, 0):
        M, dom, semi = _euler_semi(pts, arith="dw")
        ctx = dom.ctx
        ctx.set_option(L.OPT_ENTRY_ORDER, 0)
        ctx.set_option(L.OPT_LAYOUT_ORDER, order)
        du = np.empty_like(u0)
        ctx.rhs(du, u0.copy(), 0.0)
        out[order] = (du, ctx.get_option(L.OPT_HALO_STAGED_FWD), ctx.get_option(L.OPT_HALO_GROUPS))
        ctx.close()
    assert out[1][1] == out[1][2] > 0
    assert out[0][1] == 0
    assert np.array_equal(out[1][0], out[0][0])
