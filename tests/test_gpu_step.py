"""SSP-RK3 + HistoryCallback trajectories on the GPU against the CPU oracle, the
FP32-apply form against the FP64 form, and the host-buffer entry point."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _advection_problem(n_side, prec="fp64"):
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, tags, h = W.advection_cloud(n_side)
    eq = M.LinearScalarAdvectionEquation2D((1.0, 0.5))
    basis = M.PointCloudBasis(M.Point2D(), 3, approximation_type=M.RBF(M.PolyharmonicSpline(3)),
                              nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision=prec))
    domain = M.PointCloudDomain(solver, pts, {k: M.BoundaryData(*v) for k, v in tags.items()})
    ic = lambda x, t, e: W.gaussian_bump(x, t)
    bcs = {"inflow": M.BoundaryConditionDirichlet(lambda x, t, e: W.gaussian_bump(x, t).T),
           "outflow": M.BoundaryConditionDoNothing()}
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, domain, c_rv=1.0, c_uw=1.0))
    semi = M.SemidiscretizationHyperbolic(domain, eq, ic, solver, boundary_conditions=bcs,
                                          source_terms=src)
    return semi, domain, pts, tags, h


def _oracle_advection(oracle, pts, tags, domain, nv=35):
    from meshfree_gb300 import workloads as W
    n = pts.shape[0]
    idx, _, dmin, davg = oracle.knn(pts, nv)
    assert np.array_equal(idx, domain.pd.neighbors)
    rowptr = np.arange(n + 1, dtype=np.int64) * nv
    w = oracle.weights(pts, rowptr, idx.ravel())
    ops = oracle.operators_from_stencils(n, rowptr, idx.ravel(), w)
    bcs = [(oracle.BC_DIRICHLET, tags["inflow"][0], tags["inflow"][1],
            lambda x, t: W.gaussian_bump(x, t).T),
           (oracle.BC_DO_NOTHING, tags["outflow"][0], tags["outflow"][1], None)]
    return oracle.Semi(pts, ops, eq="advection", adv=(1.0, 0.5), bcs=bcs,
                       sources=(oracle.SRC_RV,), c_rv=1.0, c_uw=1.0, h=davg)


@pytest.mark.parametrize("n_side", [32, 31])
def test_advection_rv_trajectory_matches_oracle(oracle, gpu_lib, n_side):
    """n_side 31 gives 1085 nodes: an odd number of history values, whose last one the
    history kernels take singly."""
    import meshfree_gb300 as M
    semi, domain, pts, tags, h = _advection_problem(n_side)
    dt, nsteps = 0.2 * h, 30
    ode = M.semidiscretize(semi, (0.0, nsteps * dt))
    sol = M.solve(ode, M.SSPRK33(), dt=dt, callback=M.HistoryCallback(approx_order=3))
    osemi = _oracle_advection(oracle, pts, tags, domain)
    hist = oracle.History(osemi, 3)
    u_ref, t_ref = oracle.ssprk33(osemi, ode.u0, 0.0, dt, nsteps, history=hist)
    assert sol.nsteps == nsteps
    assert abs(sol.t - t_ref) <= 1e-14
    err = np.abs(sol.u - u_ref).max() / np.abs(u_ref).max()
    assert err < 1e-10, err


def test_advection_64_200_steps_matches_oracle(oracle, gpu_lib):
    """The reference's CPU-runnable case: 64x64 jittered nodes + exact inflow, PHS r^3,
    degree 3, k=35, residual viscosity, SSP-RK3 dt=0.2h for 200 steps."""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    semi, domain, pts, tags, h = _advection_problem(64)
    dt, nsteps = 0.2 * h, 200
    ode = M.semidiscretize(semi, (0.0, nsteps * dt))
    sol = M.solve(ode, M.SSPRK33(), dt=dt, callback=M.HistoryCallback(approx_order=3))
    osemi = _oracle_advection(oracle, pts, tags, domain)
    hist = oracle.History(osemi, 3)
    u_ref, t_ref = oracle.ssprk33(osemi, ode.u0, 0.0, dt, nsteps, history=hist)
    assert sol.nsteps == nsteps
    err = np.abs(sol.u - u_ref).max() / np.abs(u_ref).max()
    assert err < 1e-10, err
    exact = W.gaussian_bump(pts, t_ref)
    # bump width 0.05 = 3.2 h: residual viscosity smears it to ~11 % L2 error at t = 0.625
    assert np.linalg.norm(sol.u - exact) / np.linalg.norm(exact) < 0.2


def test_vortex_rv_trajectory_matches_oracle(oracle, gpu_lib):
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(32)
    eq = M.CompressibleEulerEquations2D(1.4)
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis)
    domain = M.PointCloudDomain(solver, pts, period=per)
    ic = lambda x, t, e: W.isentropic_vortex(x, t)
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, domain))
    semi = M.SemidiscretizationHyperbolic(domain, eq, ic, solver, source_terms=src)
    dt, nsteps = 0.1 * h, 12
    ode = M.semidiscretize(semi, (0.0, nsteps * dt))
    sol = M.solve(ode, M.SSPRK33(), dt=dt, callback=M.HistoryCallback(approx_order=3))
    n = pts.shape[0]
    idx, _, _, davg = oracle.knn(pts, 35, period=per)
    rowptr = np.arange(n + 1, dtype=np.int64) * 35
    w = oracle.weights(pts, rowptr, idx.ravel(), period=per)
    ops = oracle.operators_from_stencils(n, rowptr, idx.ravel(), w)
    osemi = oracle.Semi(pts, ops, eq="euler", gamma=1.4, sources=(oracle.SRC_RV,), h=davg)
    u_ref, _ = oracle.ssprk33(osemi, ode.u0, 0.0, dt, nsteps, history=oracle.History(osemi, 3))
    err = np.abs(sol.u - u_ref).max(axis=1) / np.abs(u_ref).max(axis=1)
    assert np.all(err < 1e-10), err


def test_fp32_apply_error_vs_fp64(gpu_lib):
    """FP32 weights/states/sums in the apply; error of density vs the FP64 form."""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(64)
    res = {}
    for prec in ("fp64", "fp32"):
        eq = M.CompressibleEulerEquations2D(1.4)
        basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
        solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision=prec))
        domain = M.PointCloudDomain(solver, pts, period=per)
        src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, domain))
        semi = M.SemidiscretizationHyperbolic(domain, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                              solver, source_terms=src)
        ode = M.semidiscretize(semi, (0.0, 20 * 0.1 * h))
        res[prec] = M.solve(ode, M.SSPRK33(), dt=0.1 * h, callback=M.HistoryCallback(3)).u
    r64, r32 = res["fp64"][0], res["fp32"][0]
    l2 = np.linalg.norm(r32 - r64) / np.linalg.norm(r64)
    assert l2 < 1e-5, l2


@pytest.mark.parametrize("n_side", [24, 31])
def test_host_entry_point_equals_device_steps(gpu_lib, n_side):
    """mft_ssprk33_host step by step (state handed back each time) equals device
    stepping, and reuses the pending first stage when handed its own state back."""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    semi, domain, pts, tags, h = _advection_problem(n_side)
    ctx = domain.ctx
    u0 = semi.compute_coefficients(0.0)
    dt = 0.2 * h
    ctx.history_init(3)
    ctx.set_state(u0, 0.0)
    ctx.ssprk33(dt, 3)
    u_dev, t_dev = ctx.get_state()
    ctx.history_init(3)
    u = u0.copy()
    t = 0.0
    for _ in range(3):
        t = ctx.ssprk33_host(u, t, dt, 1)
    assert t == t_dev
    assert np.array_equal(u, u_dev)


def test_host_entry_point_pinned_and_pageable_agree(gpu_lib):
    """Pinned caller arrays (read and written in place by the layout kernels) and pageable
    ones (staged copies) give the same states as device stepping, bit for bit (vortex with
    residual viscosity: graph-replayed steps)."""
    torch = pytest.importorskip("torch")
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(40)
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision="fp64"))
    dom = M.PointCloudDomain(solver, pts, period=per)
    eq = M.CompressibleEulerEquations2D(1.4)
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom))
    semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                          solver, source_terms=src)
    ctx = dom.ctx
    u0 = semi.compute_coefficients(0.0)
    dt = 0.2 * h
    ctx.history_init(3)
    ctx.set_state(u0, 0.0)
    ctx.ssprk33(dt, 4)
    u_dev, _ = ctx.get_state()
    results = []
    for pinned in (True, False):
        if pinned:
            buf = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True)
            u = buf.numpy()
            u[:] = u0
        else:
            u = u0.copy()
        ctx.history_init(3)
        t = 0.0
        for _ in range(4):
            t = ctx.ssprk33_host(u, t, dt, 1)
        results.append(np.array(u, copy=True))
    assert np.array_equal(results[0], u_dev)
    assert np.array_equal(results[1], u_dev)


@pytest.mark.parametrize("pinned", [True, False])
def test_host_entry_point_reruns_when_caller_changed_state(gpu_lib, pinned):
    """The caller edits its state between host calls (same time): the steps that ran
    speculatively on the held state are discarded and rerun from the caller's state,
    with the HistoryCallback bookkeeping and approx_du restored; the result equals
    device stepping from the edited state bit for bit (vortex, residual viscosity,
    history of order 3)."""
    torch = pytest.importorskip("torch")
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(40)
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision="fp64"))
    dom = M.PointCloudDomain(solver, pts, period=per)
    eq = M.CompressibleEulerEquations2D(1.4)
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom))
    semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                          solver, source_terms=src)
    ctx = dom.ctx
    u0 = semi.compute_coefficients(0.0)
    dt = 0.2 * h
    # reference: device stepping, the state replaced after three steps
    ctx.history_init(3)
    ctx.set_state(u0, 0.0)
    ctx.ssprk33(dt, 3)
    u3, t3 = ctx.get_state()
    u_edit = u3.copy()
    u_edit[0, 17] *= 1.001
    u_edit[3, 301] *= 0.999
    ctx.set_state(u_edit, t3)
    ctx.ssprk33(dt, 2)
    u_ref, t_ref = ctx.get_state()
    # host stepping with the same edit between calls
    if pinned:
        u = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True).numpy()
        u[:] = u0
    else:
        u = u0.copy()
    ctx.history_init(3)
    t = 0.0
    for _ in range(3):
        t = ctx.ssprk33_host(u, t, dt, 1)
    assert np.array_equal(u, u3) and t == t3
    u[0, 17] *= 1.001
    u[3, 301] *= 0.999
    assert np.array_equal(u, u_edit)
    for _ in range(2):
        t = ctx.ssprk33_host(u, t, dt, 1)
    assert t == t_ref
    assert np.array_equal(u, u_ref)


def test_graph_steps_equal_direct_steps(gpu_lib):
    """Steps replayed from the captured per-step CUDA graphs (device step table for the
    history weights) equal directly launched steps bit for bit, across odd batch sizes
    that swap the state buffers and a change of dt."""
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(40)
    res = []
    for use_graph in (False, True):
        eq = M.CompressibleEulerEquations2D(1.4)
        basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
        solver = M.PointCloudSolver(basis)
        domain = M.PointCloudDomain(solver, pts, period=per)
        src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, domain))
        semi = M.SemidiscretizationHyperbolic(domain, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                              solver, source_terms=src)
        ctx = domain.ctx
        ctx.history_init(3)
        ctx.set_state(semi.compute_coefficients(0.0), 0.0)
        for nsteps, dt in ((3, 0.1 * h), (2, 0.1 * h), (5, 0.1 * h), (1, 0.05 * h), (4, 0.05 * h)):
            ctx.ssprk33(dt, nsteps, use_graph=use_graph)
        res.append(ctx.get_state())
    assert res[0][1] == res[1][1]
    assert np.array_equal(res[0][0], res[1][0])


def test_graph_steps_equal_direct_steps_odd_count(gpu_lib):
    """Scalar advection on 1085 nodes (an odd number of history values): graph-replayed
    and directly launched steps agree bit for bit, the history ring filling up over the
    first steps (1 to 4 history points)."""
    res = []
    for use_graph in (False, True):
        semi, domain, pts, tags, h = _advection_problem(31)
        ctx = domain.ctx
        ctx.history_init(3)
        ctx.set_state(semi.compute_coefficients(0.0), 0.0)
        for nsteps in (1, 1, 1, 3, 2):
            ctx.ssprk33(0.2 * h, nsteps, use_graph=use_graph)
        res.append(ctx.get_state())
    assert res[0][1] == res[1][1]
    assert np.array_equal(res[0][0], res[1][0])


class _Rows:
    """Per-variable arrays handed to the host entry point as separate rows."""

    def __init__(self, rows):
        self.rows = rows
        self.shape = (len(rows), rows[0].shape[0])

    def __iter__(self):
        return iter(self.rows)


def test_host_entry_point_odd_node_count_pinned_layouts(gpu_lib):
    """An odd node count (39 x 39 vortex, 1,521 nodes) through pinned caller arrays: four
    separately allocated rows (16-byte aligned: the two-nodes-per-thread layout kernels,
    the last node taken singly) and one 2D array (its odd rows start 8 bytes off: the
    one-node-per-thread kernels) give device stepping's states bit for bit."""
    torch = pytest.importorskip("torch")
    import meshfree_gb300 as M
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(39)
    n = pts.shape[0]
    assert n % 2 == 1
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision="fp64"))
    dom = M.PointCloudDomain(solver, pts, period=per)
    eq = M.CompressibleEulerEquations2D(1.4)
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom))
    semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                          solver, source_terms=src)
    ctx = dom.ctx
    u0 = semi.compute_coefficients(0.0)
    dt = 0.2 * h
    ctx.history_init(3)
    ctx.set_state(u0, 0.0)
    ctx.ssprk33(dt, 3)
    u_dev, t_dev = ctx.get_state()
    rows = [torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for _ in range(4)]
    for v in range(4):
        rows[v][:] = u0[v]
    assert all(r.ctypes.data % 16 == 0 for r in rows)
    whole = torch.empty((4, n), dtype=torch.float64, pin_memory=True).numpy()
    whole[:] = u0
    assert whole[1].ctypes.data % 16 == 8
    for u in (_Rows(rows), whole):
        ctx.history_init(3)
        t = 0.0
        for _ in range(3):
            t = ctx.ssprk33_host(u, t, dt, 1)
        assert t == t_dev
        got = np.stack([np.array(r, copy=True) for r in u])
        assert np.array_equal(got, u_dev)


@pytest.mark.parametrize("mode", ["graph", "direct", "limited"])
def test_host_entry_point_several_steps_per_call(gpu_lib, mode):
    """Pinned caller arrays with three SSP-RK3 steps per host call (graph-replayed steps,
    directly launched steps while profiling, and a stage limiter on density and pressure
    after every stage): two calls equal six device steps bit for bit (vortex with residual
    viscosity and history)."""
    torch = pytest.importorskip("torch")
    import meshfree_gb300 as M
    from meshfree_gb300 import _lib as L
    from meshfree_gb300 import workloads as W
    pts, per, h = W.vortex_cloud(40)
    basis = M.PointCloudBasis(M.Point2D(), 3, nv=35)
    solver = M.PointCloudSolver(basis, M.RBFFDEngineGB300(precision="fp64"))
    dom = M.PointCloudDomain(solver, pts, period=per)
    eq = M.CompressibleEulerEquations2D(1.4)
    src = M.SourceTerms(rv=M.SourceResidualViscosityTominec(solver, eq, dom))
    semi = M.SemidiscretizationHyperbolic(dom, eq, lambda x, t, e: W.isentropic_vortex(x, t),
                                          solver, source_terms=src)
    ctx = dom.ctx
    if mode == "limited":
        ctx.set_limiter([L.LIM_DENSITY, L.LIM_PRESSURE], [0.05, 0.05])
    u0 = semi.compute_coefficients(0.0)
    dt = 0.2 * h
    ctx.history_init(3)
    ctx.set_state(u0, 0.0)
    ctx.ssprk33(dt, 6, use_graph=(mode != "direct"))
    u_dev, t_dev = ctx.get_state()
    u = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True).numpy()
    u[:] = u0
    ctx.history_init(3)
    if mode == "direct":
        ctx.profile(True)  # profiled steps are launched directly
    t = 0.0
    for _ in range(2):
        t = ctx.ssprk33_host(u, t, dt, 3)
    if mode == "direct":
        ctx.profile(False)
    assert t == t_dev
    assert np.array_equal(u, u_dev)
    ctx.close()
