"""Shared set-up for parity tests: the same inputs for the CPU oracle and the GPU."""
from __future__ import annotations

import numpy as np

GAMMA = 1.4


def ic_gradient(x, t=0.0):
    """initial_condition_gradient of test/divergence_test.jl:28-38 (conserved vars)."""
    s = 0.1 * x[:, 0] + 0.1 * x[:, 1]
    return np.ascontiguousarray(np.stack([1.4 + s, 4.1 + s, 0.0 + s, 8.8 + s]))


def ic_bumpy(x, seed=3):
    """Smooth non-trivial Euler state (positive density / pressure)."""
    g = np.random.Generator(np.random.PCG64(seed))
    a = g.uniform(0.5, 1.5, 6)
    rho = 1.0 + 0.2 * np.sin(a[0] * 3 * x[:, 0]) * np.cos(a[1] * 2 * x[:, 1])
    u = 0.5 + 0.3 * np.cos(a[2] * 2 * x[:, 0] + x[:, 1])
    v = -0.2 + 0.3 * np.sin(a[3] * 2 * x[:, 1] - x[:, 0])
    p = 1.0 + 0.1 * np.cos(a[4] * x[:, 0] * x[:, 1])
    e = p / (GAMMA - 1.0) + 0.5 * rho * (u * u + v * v)
    return np.ascontiguousarray(np.stack([rho, rho * u, rho * v, e]))


def cyl_bcs(cyl, dirichlet_fn):
    """Reference test BCs (divergence_test.jl:40-44) in NamedTuple order:
    inlet Dirichlet, outlet DoNothing, top / bottom / cyl slip walls.
    Boundary groups: inlet 1, outlet 2, bottom 3, top 4, cyl 5."""
    from oracle.oracle import BC_DIRICHLET, BC_DO_NOTHING, BC_SLIP_WALL
    return [
        (BC_DIRICHLET, cyl["bidx_1"], cyl["bnrm_1"], dirichlet_fn),
        (BC_DO_NOTHING, cyl["bidx_2"], cyl["bnrm_2"], None),
        (BC_SLIP_WALL, cyl["bidx_4"], cyl["bnrm_4"], None),
        (BC_SLIP_WALL, cyl["bidx_3"], cyl["bnrm_3"], None),
        (BC_SLIP_WALL, cyl["bidx_5"], cyl["bnrm_5"], None),
    ]


def stencil_ops(oracle, points, idx, rbf_pow=3, polydeg=3, order=1, period=None):
    n, k = idx.shape
    rowptr = np.arange(n + 1, dtype=np.int64) * k
    w = oracle.weights(points, rowptr, idx.ravel(), rbf_pow=rbf_pow, polydeg=polydeg,
                       deriv_order=order, period=period)
    return oracle.operators_from_stencils(n, rowptr, idx.ravel(), w), w


def load_ops_into(ctx, ops, lap=None, hv=None):
    """Loads oracle CSR/CSC operators into a GPU context through the 1-based CSC
    entry point, as a Julia caller would pass SparseMatrixCSC arrays."""
    from meshfree_gb300 import _lib as L
    for d, o in enumerate(ops):
        ctx.load_csc(L.OP_GRAD, d, o.cp + 1, o.ri.astype(np.int64) + 1, o.valt)
    if lap is not None:
        ctx.load_csc(L.OP_LAP, 0, lap.cp + 1, lap.ri.astype(np.int64) + 1, lap.valt)
    if hv is not None:
        ctx.load_csc(L.OP_HV, 0, hv.cp + 1, hv.ri.astype(np.int64) + 1, hv.valt)


def isapprox(a, b, rtol=np.sqrt(np.finfo(float).eps)):
    """Julia's isapprox for arrays: norm(a-b) <= rtol * max(norm(a), norm(b))."""
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return np.linalg.norm(a - b) <= rtol * max(np.linalg.norm(a), np.linalg.norm(b))


def flux_np(u, d, gamma=GAMMA):
    rho, m1, m2, e = u
    v1, v2 = m1 / rho, m2 / rho
    p = (gamma - 1.0) * (e - 0.5 * (m1 * v1 + m2 * v2))
    if d == 0:
        return np.stack([m1, m1 * v1 + p, m1 * v2, (e + p) * v1])
    return np.stack([m2, m2 * v1, m2 * v2 + p, (e + p) * v2])


def flux3d_np(u, d, gamma=GAMMA):
    """CompressibleEulerEquations3D flux in direction d (textbook form)."""
    rho, m1, m2, m3, e = u
    v = [m1 / rho, m2 / rho, m3 / rho]
    m = [m1, m2, m3]
    p = (gamma - 1.0) * (e - 0.5 * (m1 * v[0] + m2 * v[1] + m3 * v[2]))
    f = [m[d]] + [m[d] * v[k] + (p if k == d else 0.0) for k in range(3)] + [(e + p) * v[d]]
    return np.stack(f)


def cond_scale(ops, u, fluxes=None, eps=None, lap=None, hv_gamma=0.0, hvop=None):
    """Per-variable condition scale  |D||F| + sum_d |D_d|'(|eps| |D_d||u|)
    + gamma |lap|'|lap||u| (+ gamma |H||u|), max over nodes."""
    A = [abs(o.to_scipy()) for o in ops]
    V = u.shape[0]
    out = np.zeros(V)
    for v in range(V):
        s = np.zeros(u.shape[1])
        if fluxes is not None:
            for d, a in enumerate(A):
                s += a @ np.abs(fluxes[d][v])
        if eps is not None:
            for a in A:
                s += a.T @ (np.abs(eps) * (a @ np.abs(u[v])))
        if lap is not None:
            la = abs(lap.to_scipy())
            s += hv_gamma * (la.T @ (la @ np.abs(u[v])))
        if hvop is not None:
            s += hv_gamma * (abs(hvop.to_scipy()) @ np.abs(u[v]))
        out[v] = s.max()
    return out


# --------------------------------------------------------------------------------------
# Forward-mode derivative of rhs! by the complex step: the counterpart of ForwardDiff
# through the reference rhs!.  rhs_complex restates the oracle's rhs! (mfto_rhs in
# oracle/mft_oracle.c: strong BC pass, flux divergence, hyperviscosity, second BC pass;
# rbfsolver.jl:397-428, PointCloudBCs.jl:49-115) in numpy so that it runs on complex
# states; for the real-analytic map u -> du,  J v = Im rhs(u + i h v) / h  with h = 1e-30
# has no truncation and no cancellation error.

CS_STEP = 1e-30


def _bc_pass_complex(semi, dirichlet, du, u):
    from oracle.oracle import BC_DIRICHLET, BC_SLIP_WALL
    for b, (kind, ii, normals, _fn) in enumerate(semi.bcs):
        ii = np.asarray(ii, dtype=np.int64)
        if kind == BC_DIRICHLET:
            du[:, ii] = 0.0
            u[:, ii] = dirichlet[semi.bc_ptr[b]:semi.bc_ptr[b + 1]].T
        elif kind == BC_SLIP_WALL and semi.nvars == 4:
            nr = np.asarray(normals, dtype=np.float64).reshape(ii.size, semi.dim)
            nn = np.sqrt(nr[:, 0] ** 2 + nr[:, 1] ** 2)
            n1, n2 = nr[:, 0] / nn, nr[:, 1] / nn
            vn = u[1, ii] * n1 + u[2, ii] * n2
            s1, s2 = u[1, ii] - vn * n1, u[2, ii] - vn * n2
            du[1, ii] = 0.0
            du[2, ii] = 0.0
            u[1, ii] = s1
            u[2, ii] = s2


JL_EPS = 2.220446049250313e-16


def _cabs(z):
    """|x| continued to complex arguments as sign(Re z) z: the derivative of |x| away
    from x = 0 (its branch frozen by the real part)."""
    return np.where(z.real < 0, -z, z)


def _visc_complex(semi, kind, du, u):
    """The viscosity source (update_upwind_visc!, update_residual_visc!, update_visc!
    and its application, hyperviscosity.jl:246-409; the oracle's visc_source) on complex
    states, every selection (the min in update_visc!, the maximum over variables, the
    lexicographic ode_maximum, |.|) decided by the real parts as the real evaluation
    decides it.  du holds the partial du the source reads; the source is added to it."""
    from oracle.oracle import SRC_RV
    s = semi.s
    n, V = semi.n, semi.nvars
    h = s.h
    if V == 4:
        rho, m1, m2, en = u
        v1, v2 = m1 / rho, m2 / rho
        p = (s.gamma - 1.0) * (en - 0.5 * (m1 * v1 + m2 * v2))
        speed = np.sqrt(v1 * v1 + v2 * v2)
        bad = (p.real < 0.0) | (rho.real < 0.0)
        c = np.where(bad, 0.0, np.sqrt(np.where(bad, 1.0, s.gamma * p / rho)))
        eps_uw = s.c_uw * 0.5 * h * (speed + c)
    else:
        a2 = sum(s.adv[d] * s.adv[d] for d in range(semi.dim))
        eps_uw = np.full(n, s.c_uw * 0.5 * h * np.sqrt(a2), dtype=np.complex128)
    eps = eps_uw
    if kind == SRC_RV and s.success_iter != 0:
        denom = float(n * V) if s.mean_mode == 0 else float(n)
        mean = np.array([u[v].sum() / denom for v in range(V)])
        loc = _cabs(u - mean[:, None])
        if s.max_mode == 0:
            keys = loc.real.T
            best = 0
            for i in range(1, n):           # max(a, b) = isless(b, a) ? a : b; ties: later
                if not tuple(keys[i]) < tuple(keys[best]):
                    best = i
            nrm = loc[:, best].copy()
        else:
            nrm = np.array([loc[v, np.flatnonzero(loc[v].real == loc[v].real.max())[-1]]
                            for v in range(V)])
        nrm = np.where(nrm.real == 0.0, JL_EPS, nrm)
        ad = semi.approx_du.reshape(V, n)
        q = _cabs(ad - du) / nrm[:, None]
        mr = q[0].copy()
        for v in range(1, V):               # jl_max: ties take the later argument
            mr = np.where(q[v].real >= mr.real, q[v], mr)
        eps_rv = 0.5 * s.c_rv * (h * h) * mr
        take_uw = eps_uw.real < eps_rv.real
        eps = np.where(take_uw, eps_uw, eps_rv)
    for j, op in enumerate(semi.ops):
        A = op.to_scipy()
        for v in range(V):
            du[v] -= A.T @ (eps * (A @ u[v]))
    return du


def rhs_complex(semi, u, t=0.0, return_state=False):
    """rhs!(u, t) of an oracle Semi without the IGR source, for real or complex u
    (nvars, n); u is not mutated.  With return_state, also the state as the BC pass
    leaves it (rhs! mutates u at boundary nodes).  Viscosity sources freeze their
    selections at the real parts (derivatives away from selection ties)."""
    from oracle.oracle import SRC_HV_FLYER, SRC_HV_TOMINEC, SRC_RV, SRC_UPWIND
    u = np.array(u, dtype=np.complex128)
    du = np.zeros_like(u)
    dv = semi.dirichlet_values(t)
    _bc_pass_complex(semi, dv, du, u)
    for d, op in enumerate(semi.ops):
        A = op.to_scipy()
        if semi.nvars == 4:
            f = flux_np(u, d, semi.s.gamma)
        else:
            f = semi.s.adv[d] * u
        for v in range(semi.nvars):
            du[v] -= A @ f[v]
    srcs = [int(k) for k in semi.src[:semi.s.n_src]]
    for k in srcs:
        if k in (SRC_RV, SRC_UPWIND):
            du = _visc_complex(semi, k, du, u)
            continue
        assert k in (SRC_HV_TOMINEC, SRC_HV_FLYER), "IGR source: no derivative"
        H = semi.hv.to_scipy()
        for v in range(semi.nvars):
            du[v] -= semi.s.hv_gamma * (H @ u[v])
    _bc_pass_complex(semi, dv, du, u)
    return (du, u) if return_state else du


def ssprk33_complex(semi, u0, t0, dt, nsteps):
    """The oracle's ssprk33_record trajectory (Shu-Osher SSP-RK3; every rhs! projects its
    argument by the BC pass; the final FSAL evaluation projects u_T) on complex states."""
    u = np.array(u0, dtype=np.complex128)
    t = t0
    for step in range(nsteps):
        k, u = rhs_complex(semi, u, t, return_state=True)
        un = u
        u1 = un + dt * k
        k1, u1 = rhs_complex(semi, u1, t + dt, return_state=True)
        u2 = (3.0 * un + u1 + dt * k1) / 4.0
        k2, u2 = rhs_complex(semi, u2, t + 0.5 * dt, return_state=True)
        u = (un + 2.0 * u2 + 2.0 * dt * k2) / 3.0
        t = t0 + (step + 1) * dt
    _, u = rhs_complex(semi, u, t, return_state=True)
    return u


def trajectory_jvp_complex(semi, u0, v, dt, nsteps, t0=0.0):
    """d u_T / d u0 applied to v by the complex step."""
    uc = np.asarray(u0) + 1j * CS_STEP * np.asarray(v)
    return ssprk33_complex(semi, uc, t0, dt, nsteps).imag / CS_STEP


def jvp_complex(semi, u, v, t=0.0):
    """J(u) v by the complex step."""
    return rhs_complex(semi, np.asarray(u) + 1j * CS_STEP * np.asarray(v), t).imag / CS_STEP


def jacobian_complex(semi, u, t=0.0):
    """Dense Jacobian d vec(du) / d vec(u) (row-major (nvars, n) vectorisation), one
    complex-step column per unknown; small problems only."""
    V, n = u.shape
    J = np.empty((V * n, V * n))
    e = np.zeros((V, n))
    for q in range(V * n):
        e.flat[q] = 1.0
        J[:, q] = jvp_complex(semi, u, e, t).ravel()
        e.flat[q] = 0.0
    return J
