"""The oracle's rhs! for 3D point clouds: CompressibleEulerEquations3D (5 variables) and
scalar advection in 3D, with the plain flux divergence of calc_fluxes!
(src/solvers/pointcloudsolver/rbfsolver.jl:247-265, dimension-generic over the operators
D_x, D_y, D_z of compute_flux_operator, compute_operators.jl:500-546) and strong
Dirichlet / do-nothing BCs.  The reference's viscosity sources and slip walls are written
for CompressibleEulerEquations2D only (hyperviscosity.jl:246-329, PointCloudBCs.jl:15-21);
the oracle refuses them in 3D.

* calc_fluxes! == -Dx fx - Dy fy - Dz fz (the divergence identity of
  test/divergence_test.jl:63-82, in 3D);
* a constant state is steady (the weights reproduce constants);
* Dirichlet rows: u set to the boundary values, du zero;
* sources or slip walls with 3D Euler are refused."""
import numpy as np
import pytest

from helpers import GAMMA, flux3d_np, isapprox, stencil_ops


@pytest.fixture(scope="module")
def cube(oracle):
    from meshfree_gb300 import workloads as W
    pts, h = W.jittered_grid3(10, seed=7)
    idx, _, _, _ = oracle.knn(pts, 30, period=(1.0, 1.0, 1.0))
    ops, _ = stencil_ops(oracle, pts, idx, polydeg=2, period=(1.0, 1.0, 1.0))
    return pts, ops, h


def test_euler3d_divergence_identity(oracle, cube):
    from meshfree_gb300 import workloads as W
    pts, ops, _h = cube
    semi = oracle.Semi(pts, ops, eq="euler3d", gamma=GAMMA)
    u = W.euler3d_wave(pts)
    du = semi.rhs(u.copy(), 0.0)
    D = [o.to_scipy() for o in ops]
    ref = np.stack([-sum(D[d] @ flux3d_np(u, d)[v] for d in range(3)) for v in range(5)])
    assert isapprox(du, ref, rtol=1e-13)
    assert np.abs(du).max() > 0.1


def test_euler3d_constant_state_is_steady(oracle, cube):
    pts, ops, _h = cube
    semi = oracle.Semi(pts, ops, eq="euler3d", gamma=GAMMA)
    u = np.tile(np.array([1.2, 0.3, -0.1, 0.2, 2.5])[:, None], (1, pts.shape[0]))
    du = semi.rhs(np.ascontiguousarray(u), 0.0)
    assert np.abs(du).max() < 1e-9


def test_advection3d_dirichlet(oracle, cube):
    pts, ops, _h = cube
    inflow = np.where(pts[:, 0] < 0.1)[0].astype(np.int32)
    g = lambda x, t: np.exp(-np.sum((x - 0.5) ** 2, axis=1))[:, None]
    semi = oracle.Semi(pts, ops, eq="advection", adv=(1.0, 0.5, -0.25),
                       bcs=[(oracle.BC_DIRICHLET, inflow, np.tile([-1.0, 0, 0], (inflow.size, 1)), g)])
    u = np.ascontiguousarray(np.sin(2 * np.pi * pts[:, 0]) * np.cos(2 * np.pi * pts[:, 2]))[None, :]
    uu = u.copy()
    du = semi.rhs(uu, 0.0)
    assert np.array_equal(uu[0, inflow], g(pts[inflow], 0.0)[:, 0])
    assert np.all(du[0, inflow] == 0.0)
    D = [o.to_scipy() for o in ops]
    a = (1.0, 0.5, -0.25)
    ref = -sum(D[d] @ (a[d] * uu[0]) for d in range(3))
    ref[inflow] = 0.0
    assert isapprox(du[0], ref, rtol=1e-13)


def test_euler3d_refuses_sources_and_slip_walls(oracle, cube):
    from meshfree_gb300 import workloads as W
    pts, ops, h = cube
    u = W.euler3d_wave(pts)
    semi = oracle.Semi(pts, ops, eq="euler3d", gamma=GAMMA, sources=(oracle.SRC_RV,), h=h)
    with pytest.raises(RuntimeError):
        semi.rhs(u.copy(), 0.0)
    wall = np.arange(5, dtype=np.int32)
    semi = oracle.Semi(pts, ops, eq="euler3d", gamma=GAMMA,
                       bcs=[(oracle.BC_SLIP_WALL, wall, np.tile([1.0, 0, 0], (5, 1)), None)])
    with pytest.raises(RuntimeError):
        semi.rhs(u.copy(), 0.0)
