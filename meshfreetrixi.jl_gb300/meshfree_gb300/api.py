"""Host-side mirror of the reference's point-cloud API over libmeshfree_gb300.so.

Names, arguments and behaviour follow MeshfreeTrixi.jl and the Trixi.jl calls it
is used with (PointCloudBasis, PointCloudSolver, PointCloudDomain,
SemidiscretizationHyperbolic, semidiscretize, rhs!, the source types, the
HistoryCallback and an SSPRK33 integrator).  Arrays follow the StructArray
layout: a state is an (nvars, n) float64 array, one row per conserved variable.
Node indices are 0-based.  Every numerical step runs in the CUDA library.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Callable

import numpy as np

from . import _lib as L
from .medusa import read_medusa_file

# ------------------------------------------------------------------ basis
# src/domains/PointCloudDomain/geometry_primatives.jl:1-209


class Point1D:
    ndims = 1


class Point2D:
    ndims = 2


class Point3D:
    ndims = 3


@dataclass(frozen=True)
class PolyharmonicSpline:
    """phi(r) = r^Nrbf (geometry_primatives.jl:110-114, 212-237)."""
    Nrbf: int = 3


@dataclass(frozen=True)
class RBF:
    rbf_type: PolyharmonicSpline = field(default_factory=PolyharmonicSpline)

    @property
    def Nrbf(self):
        return self.rbf_type.Nrbf


@dataclass(frozen=True)
class RefPointData:
    """element_type, approximation_type, N (polynomial degree), nv (stencil size)
    (geometry_primatives.jl:27-35)."""
    element_type: object
    approximation_type: RBF
    N: int
    nv: int

    @property
    def ndims(self):
        return self.element_type.ndims


def PointCloudBasis(element_type, polydeg, approximation_type=None, nv=None):
    """types.jl:83-86; nv defaults to max(2*binomial(N+d, d), (10,15,20)[d])
    (geometry_primatives.jl:183-184)."""
    at = approximation_type if approximation_type is not None else RBF()
    d = element_type.ndims
    if nv is None:
        nv = max(2 * math.comb(polydeg + d, d), (10, 15, 20)[d - 1])
    return RefPointData(element_type, at, int(polydeg), int(nv))


# ------------------------------------------------------------------ solver
# src/solvers/rbfsolver.jl:8-71, src/solvers/pointcloudsolver/types.jl:49-74


@dataclass
class RBFFDEngineGB300:
    """The GB300 engine (the reference's RBFFDEngineCUDA slot).  precision is
    "fp64" (FP64 weights, states and sums) or "fp32" (FP32 apply, FP64 RK).
    fp64_arith: how the FP64 form's gathers form their sums of products -- "auto"
    (= "dw"), "dw" (double-word FP32 arithmetic, 2D Euler) or "dfma" (FP64 FMAs)."""
    device: int = 0
    precision: str = "fp64"
    fp64_arith: str = "auto"


@dataclass
class RBFSolver:
    basis: RefPointData
    engine: RBFFDEngineGB300


def PointCloudSolver(basis, engine=None):
    return RBFSolver(basis, engine if engine is not None else RBFFDEngineGB300())


# ------------------------------------------------------------------ domain
# src/domains/PointCloudDomain/*.jl


@dataclass
class PointData:
    """geometry_primatives.jl:300-339: neighbours (n, nv) sorted by distance, self
    first; dx_min / dx_avg: min and mean nearest-neighbour distance."""
    points: np.ndarray
    neighbors: np.ndarray
    num_points: int
    num_neighbors: int
    dx_min: float
    dx_avg: float


@dataclass
class BoundaryData:
    idx: np.ndarray
    normals: np.ndarray


class PointCloudDomain:
    """Point cloud with GPU-built stencils and boundary tags.  Holds the engine
    context that the semidiscretization on this domain uses."""

    def __init__(self, solver, points, boundary_tags=None, period=None):
        basis = solver.basis
        pts = np.ascontiguousarray(points, dtype=np.float64)
        assert pts.ndim == 2 and pts.shape[1] == basis.ndims
        self.solver = solver
        self.period = None if period is None else tuple(float(p) for p in period)
        self.ctx = L.Context(solver.engine.device)
        self.ctx.set_points(pts, self.period)
        idx, _dist, dmin, davg = self.ctx.knn(basis.nv)
        self.pd = PointData(pts, idx, pts.shape[0], basis.nv, dmin, davg)
        self.boundary_tags = dict(boundary_tags or {})
        self.loaded = {}

    @property
    def ndims(self):
        return self.pd.points.shape[1]

    def operator(self, op, rbf_pow, polydeg, deriv_order):
        """Computes (once) the weights of operator slot `op` on the GPU."""
        key = (op, rbf_pow, polydeg, deriv_order)
        if self.loaded.get(op) != key:
            self.ctx.weights(op, rbf_pow, polydeg, deriv_order)
            self.loaded[op] = key


class PointCloudEnsemble(PointCloudDomain):
    """Independent point clouds advanced together in one engine context (one set of
    kernels and one graph per step for all members).  Member m owns nodes
    offsets[m]:offsets[m+1]; stencils are built per member (GPU KNN) and never cross
    members; the residual-viscosity normalisation and dx_avg are per member."""

    def __init__(self, solver, member_points, period=None):
        basis = solver.basis
        self.solver = solver
        self.period = None if period is None else tuple(float(p) for p in period)
        k = basis.nv
        idx_all, pts_all, dmins, davgs, offs = [], [], [], [], [0]
        tmp = L.Context(solver.engine.device)
        for pts in member_points:
            pts = np.ascontiguousarray(pts, dtype=np.float64)
            tmp.set_points(pts, self.period)
            idx, _d, dmin, davg = tmp.knn(k)
            idx_all.append(idx.astype(np.int64) + offs[-1])
            pts_all.append(pts)
            dmins.append(dmin)
            davgs.append(davg)
            offs.append(offs[-1] + pts.shape[0])
        tmp.close()
        points = np.ascontiguousarray(np.concatenate(pts_all))
        neighbors = np.ascontiguousarray(np.concatenate(idx_all).astype(np.int32))
        self.offsets = np.asarray(offs, dtype=np.int64)
        self.dx_min = np.asarray(dmins)
        self.dx_avg = np.asarray(davgs)
        self.ctx = L.Context(solver.engine.device)
        self.ctx.set_points(points, self.period)
        n = points.shape[0]
        self.ctx.set_stencils(np.arange(n + 1, dtype=np.int64) * k, neighbors.ravel())
        self.ctx.set_segments(self.offsets, self.dx_avg)
        self.pd = PointData(points, neighbors, n, k, float(self.dx_min.min()),
                            float(self.dx_avg.mean()))
        self.boundary_tags = {}
        self.loaded = {}

    @property
    def members(self):
        return len(self.offsets) - 1

    def member(self, u, m):
        """Member m's slice of an (nvars, n) ensemble state."""
        return u[:, self.offsets[m]:self.offsets[m + 1]]


def PointCloudDomain_from_medusa(solver, casename, boundary_names):
    """PointCloudDomain(solver, casename, Dict(:inlet => 1, ...)) (types.jl:133-145,
    SerialPointCloud.jl:45-54)."""
    pos, _interior, b_idx, b_nrm, _normals, _types = read_medusa_file(casename)
    tags = {name: BoundaryData(b_idx[i - 1], b_nrm[i - 1]) for name, i in boundary_names.items()}
    return PointCloudDomain(solver, pos, tags)


# ------------------------------------------------------------------ equations


@dataclass
class CompressibleEulerEquations2D:
    gamma: float = 1.4
    nvariables = 4
    kind = L.EQ_EULER2D

    def params(self):
        return [self.gamma]

    def cons2prim(self, u):
        rho, m1, m2, e = u
        v1, v2 = m1 / rho, m2 / rho
        p = (self.gamma - 1.0) * (e - 0.5 * (m1 * v1 + m2 * v2))
        return np.stack([rho, v1, v2, p])

    def prim2cons(self, w):
        rho, v1, v2, p = w
        return np.stack([rho, rho * v1, rho * v2, p / (self.gamma - 1.0) + 0.5 * rho * (v1 * v1 + v2 * v2)])


@dataclass
class CompressibleEulerEquations3D:
    """Trixi's CompressibleEulerEquations3D (rho, rho v1, rho v2, rho v3, E).  On 3D clouds
    the engine evaluates the plain flux divergence with Dirichlet / do-nothing BCs (the
    reference's viscosity sources and slip walls are 2D-only)."""
    gamma: float = 1.4
    nvariables = 5
    kind = L.EQ_EULER3D

    def params(self):
        return [self.gamma]

    def cons2prim(self, u):
        rho, m1, m2, m3, e = u
        v1, v2, v3 = m1 / rho, m2 / rho, m3 / rho
        p = (self.gamma - 1.0) * (e - 0.5 * (m1 * v1 + m2 * v2 + m3 * v3))
        return np.stack([rho, v1, v2, v3, p])

    def prim2cons(self, w):
        rho, v1, v2, v3, p = w
        return np.stack([rho, rho * v1, rho * v2, rho * v3,
                         p / (self.gamma - 1.0) + 0.5 * rho * (v1 * v1 + v2 * v2 + v3 * v3)])


@dataclass
class LinearScalarAdvectionEquation2D:
    advection_velocity: tuple = (1.0, 0.5)
    nvariables = 1
    kind = L.EQ_ADVECTION

    def params(self):
        return list(self.advection_velocity)


@dataclass
class LinearScalarAdvectionEquation3D:
    advection_velocity: tuple = (1.0, 0.5, 0.25)
    nvariables = 1
    kind = L.EQ_ADVECTION

    def params(self):
        return list(self.advection_velocity)


# ------------------------------------------------------------------ boundary conditions
# src/equations/PointCloudBCs.jl


@dataclass
class BoundaryConditionDirichlet:
    """boundary_value_function(x (m, d), t, equations) -> (m, nvars) array."""
    boundary_value_function: Callable
    kind = L.BC_DIRICHLET


class BoundaryConditionSlipWall:
    kind = L.BC_SLIP_WALL


class BoundaryConditionDoNothing:
    kind = L.BC_DO_NOTHING


boundary_condition_slip_wall = BoundaryConditionSlipWall()


# ------------------------------------------------------------------ sources
# src/sources/generic_sources.jl, src/sources/hyperviscosity.jl


class SourceTerms(dict):
    """SourceTerms(; kwargs...): an ordered name -> source mapping."""

    def __init__(self, **kw):
        super().__init__(kw)


@dataclass
class SourceResidualViscosityTominec:
    solver: RBFSolver
    equations: object
    domain: PointCloudDomain
    c_rv: float = 1.0
    c_uw: float = 1.0
    polydeg: int = 4
    norm_mode: int = 0  # 0: reference ode_mean/ode_maximum; 1: per-component

    def spec(self):
        return L.SRC_RV, [self.c_rv, self.c_uw, self.domain.pd.dx_avg, self.norm_mode]


@dataclass
class SourceUpwindViscosityTominec:
    solver: RBFSolver
    equations: object
    domain: PointCloudDomain
    c: float = 1.0
    c_uw: float = 1.0
    polydeg: int = 4

    def spec(self):
        return L.SRC_UPWIND, [self.c_uw, self.domain.pd.dx_avg, 0.0, 0.0]


@dataclass
class SourceHyperviscosityTominec:
    """gamma = c * dx_min^4.5; operator lap' * lap, lap = Dxx + Dyy (:101-119)."""
    solver: RBFSolver
    equations: object
    domain: PointCloudDomain
    c: float = 1.0

    @property
    def gamma(self):
        return self.c * self.domain.pd.dx_min ** 4.5

    def prepare(self):
        b = self.solver.basis
        self.domain.operator(L.OP_LAP, b.approximation_type.Nrbf, b.N, 2)

    def spec(self):
        return L.SRC_HV_TOMINEC, [self.gamma, 0.0, 0.0, 0.0]


@dataclass
class SourceIGR:
    """SourceIGR(solver, equations, domain; alpha) (src/sources/IGR.jl:17-32): information
    geometric regularisation; sigma from a conjugate-gradient solve (at most `maxiter`
    iterations) of (rho^-1 - alpha (Dx rho^-1 Dx + Dy rho^-1 Dy)) sigma =
    alpha (tr(Du)^2 + tr(Du^2)), then du[rho v] -= (Dx sigma, Dy sigma)."""
    solver: RBFSolver
    equations: object
    domain: PointCloudDomain
    alpha: float = 1.0
    maxiter: int = 20

    def spec(self):
        return L.SRC_IGR, [self.alpha, float(self.maxiter), 0.0, 0.0]


@dataclass
class SourceHyperviscosityFlyer:
    """gamma = c * dx_min^(2k); operator sum_d D_d^(2k) (:34-50)."""
    solver: RBFSolver
    equations: object
    domain: PointCloudDomain
    k: int = 2
    c: float = 1.0

    @property
    def gamma(self):
        return self.c * self.domain.pd.dx_min ** (2 * self.k)

    def prepare(self):
        b = self.solver.basis
        self.domain.operator(L.OP_HV, b.approximation_type.Nrbf, b.N, 2 * self.k)

    def spec(self):
        return L.SRC_HV_FLYER, [self.gamma, 0.0, 0.0, 0.0]


# ------------------------------------------------------------------ semidiscretization


class SemidiscretizationHyperbolic:
    """Trixi's SemidiscretizationHyperbolic specialised to point clouds: the cache
    (Trixi.create_cache, rbfsolver.jl:130-165) lives in the engine context."""

    def __init__(self, domain, equations, initial_condition, solver, boundary_conditions=None,
                 source_terms=None):
        self.domain, self.equations, self.solver = domain, equations, solver
        self.initial_condition = initial_condition
        self.boundary_conditions = dict(boundary_conditions or {})
        self.source_terms = source_terms if source_terms is not None else SourceTerms()
        b = solver.basis
        ctx = domain.ctx
        domain.operator(L.OP_GRAD, b.approximation_type.Nrbf, b.N, 1)
        ctx.set_equations(equations.kind, equations.params())
        ctx.set_precision(L.PREC_FP32 if solver.engine.precision == "fp32" else L.PREC_FP64)
        ctx.set_option(L.OPT_FP64_ARITH, {"auto": L.ARITH_AUTO, "dw": L.ARITH_DW,
                                          "dfma": L.ARITH_DFMA}[solver.engine.fp64_arith])
        kinds, ptr, idx, nrm = [], [0], [], []
        self._dirichlet = []
        for name, bc in self.boundary_conditions.items():
            tag = domain.boundary_tags[name]
            ii = np.asarray(tag.idx, dtype=np.int32)
            kinds.append(bc.kind)
            idx.append(ii)
            nrm.append(np.asarray(tag.normals, dtype=np.float64).reshape(ii.size, -1))
            if bc.kind == L.BC_DIRICHLET:
                self._dirichlet.append((slice(ptr[-1], ptr[-1] + ii.size), ii, bc))
            ptr.append(ptr[-1] + ii.size)
        self._nb = ptr[-1]
        if kinds:
            ctx.set_bcs(kinds, ptr, np.concatenate(idx), np.concatenate(nrm))
        else:
            ctx.set_bcs([], [0], np.zeros(0, np.int32), None)
        if self._dirichlet:
            ctx.set_dirichlet_callback(self.dirichlet_values)
        else:
            ctx.set_dirichlet_callback(None)
        skinds, spars = [], []
        for src in self.source_terms.values():
            if hasattr(src, "prepare"):
                src.prepare()
            k, p = src.spec()
            skinds.append(k)
            spars.append(p)
        ctx.set_sources(skinds, spars)

    def dirichlet_values(self, t):
        V = self.equations.nvariables
        out = np.zeros((self._nb, V))
        for sl, ii, bc in self._dirichlet:
            x = self.domain.pd.points[ii]
            out[sl] = np.asarray(bc.boundary_value_function(x, t, self.equations)).reshape(-1, V)
        return out

    def compute_coefficients(self, t):
        """u = initial_condition(x, t, equations) at every node (rbfsolver.jl:174-185)."""
        u = self.initial_condition(self.domain.pd.points, t, self.equations)
        return np.ascontiguousarray(np.asarray(u, dtype=np.float64).reshape(self.equations.nvariables, -1))


@dataclass
class ODEProblem:
    u0: np.ndarray
    tspan: tuple
    p: SemidiscretizationHyperbolic


def semidiscretize(semi, tspan):
    return ODEProblem(semi.compute_coefficients(tspan[0]), tuple(tspan), semi)


def rhs_(du, u, semi, t):
    """Trixi's rhs!(du_ode, u_ode, semi, t) (rbfsolver.jl:397-428) on the GPU.
    du, u: (nvars, n) float64 C-contiguous; u is mutated at boundary nodes."""
    semi.domain.ctx.rhs(du, u, t)
    return None


def rhs_adjoint_(out, lam, u, semi, t):
    """Pullback of rhs!: out = (d rhs!(u, t)/du)^T lam on the GPU (mft_rhs_adjoint);
    the reference has no counterpart (it differentiates rhs! with ForwardDiff duals).
    u is not mutated."""
    out[...] = semi.domain.ctx.rhs_adjoint(lam, u, t)
    return None


# ------------------------------------------------------------------ time integration


@dataclass
class HistoryCallback:
    """HistoryCallback(; approx_order) (src/callbacks_step/history.jl:43-49)."""
    approx_order: int


@dataclass
class SaveCheckpointCallback:
    """Writes the integrator state (t, u, the pending first stage, the history ring) to
    `path` every `interval` steps and at the end of solve, overwriting the file
    (mft_checkpoint_save).  solve(..., resume_from=path) continues from such a file bit
    for bit.  The reference has no restart files (save_solution_vtk.jl writes output)."""
    interval: int
    path: str


def save_checkpoint(semi, path):
    """The device integrator state of semi's context into the file at path."""
    data = semi.domain.ctx.checkpoint()
    tmp = str(path) + ".tmp"
    with open(tmp, "wb") as f:
        f.write(data)
    os.replace(tmp, path)


def load_checkpoint(semi, path):
    """Loads a file written by save_checkpoint into semi's context (same problem set-up)."""
    with open(path, "rb") as f:
        semi.domain.ctx.restore(f.read())


class SSPRK33:
    """Shu-Osher SSP-RK3 with first-same-as-last stage reuse; SSPRK33(stage_limiter!)
    applies the limiter after every stage, as OrdinaryDiffEq does."""

    def __init__(self, stage_limiter=None):
        self.stage_limiter = stage_limiter


def density(u, equations=None):
    """Trixi.density (the first conserved variable)."""
    return u[0]


def pressure(u, equations):
    """Trixi.pressure for CompressibleEulerEquations2D."""
    return (equations.gamma - 1.0) * (u[3] - 0.5 * (u[1] * u[1] + u[2] * u[2]) / u[0])


class PositivityPreservingLimiterZhangShu:
    """PositivityPreservingLimiterZhangShu(; thresholds, variables)
    (src/callbacks_stage/positivity_zhang_shu.jl:22-31); variables are `density` and
    `pressure`, applied in the given order.  Calling it on (u, semi) limits u in place
    (limiter_zhang_shu!, positivity_zhang_shu_point2d.jl:22-82) on the GPU."""

    def __init__(self, thresholds, variables):
        if len(thresholds) != len(variables):
            raise ValueError("one threshold per variable")
        kinds = {density: L.LIM_DENSITY, pressure: L.LIM_PRESSURE}
        self.thresholds = tuple(float(x) for x in thresholds)
        self.variables = tuple(variables)
        self.kinds = [kinds[v] for v in self.variables]

    def configure(self, ctx):
        ctx.set_limiter(self.kinds, self.thresholds)

    def __call__(self, u, semi):
        ctx = semi.domain.ctx
        self.configure(ctx)
        u = np.ascontiguousarray(u, dtype=np.float64)
        ctx.limit(u)
        return u


@dataclass
class ODESolution:
    u: np.ndarray
    t: float
    nsteps: int


def solve(ode, alg=None, dt=None, callback=None, save_everystep=False, resume_from=None):
    """Fixed-step SSPRK33 on the device from tspan[0] to tspan[1]; with resume_from (a
    file of SaveCheckpointCallback / save_checkpoint) from the state and time held there
    to tspan[1]."""
    assert dt is not None and dt > 0
    semi = ode.p
    ctx = semi.domain.ctx
    t0, t1 = ode.tspan
    cbs = callback if isinstance(callback, (list, tuple)) else ([callback] if callback else [])
    lim = getattr(alg, "stage_limiter", None)
    if lim is not None:
        lim.configure(ctx)
    else:
        ctx.set_limiter([], [])
    if resume_from is not None:
        load_checkpoint(semi, resume_from)
        t0 = ctx.get_state()[1]
    else:
        ctx.set_state(ode.u0, t0)
        for cb in cbs:
            if isinstance(cb, HistoryCallback):
                ctx.history_init(cb.approx_order)
    ckpt = [cb for cb in cbs if isinstance(cb, SaveCheckpointCallback)]
    nfull = max(int(math.floor((t1 - t0) / dt + 1e-9)), 0)
    if ckpt:
        every = max(int(ckpt[0].interval), 1)
        done = 0
        while done < nfull:
            k = min(every, nfull - done)
            ctx.ssprk33(dt, k)
            done += k
            save_checkpoint(semi, ckpt[0].path)
    else:
        ctx.ssprk33(dt, nfull)
    steps = nfull
    rest = (t1 - t0) - nfull * dt
    if rest > 1e-12 * dt:
        ctx.ssprk33(rest, 1)
        steps += 1
    u, t = ctx.get_state()
    return ODESolution(u, t, steps)


def solve_adjoint(ode, dt, dJdu, checkpoint_every=-1):
    """Gradient of an objective of the final state w.r.t. the initial state: SSP-RK3
    from tspan[0] to tspan[1] in steps of dt (which must divide the span), recorded
    with a checkpoint every `checkpoint_every` steps (0 keeps every stage state; -1, the
    default, keeps every stage state when they fit in half of the free device memory and
    checkpoints otherwise), then the reverse sweep from dJdu(u(T)).  Returns
    (ODESolution, dJ/du0)."""
    semi = ode.p
    ctx = semi.domain.ctx
    t0, t1 = ode.tspan
    nsteps = int(round((t1 - t0) / dt))
    if nsteps < 1 or abs(nsteps * dt - (t1 - t0)) > 1e-9 * max(abs(t1 - t0), dt):
        raise ValueError("dt must divide tspan into a whole number of steps")
    ctx.set_state(ode.u0, t0)
    ctx.ssprk33_record(dt, nsteps, checkpoint_every)
    u, t = ctx.get_state()
    lam = np.ascontiguousarray(dJdu(u), dtype=np.float64)
    return ODESolution(u, t, nsteps), ctx.ssprk33_adjoint(lam)
