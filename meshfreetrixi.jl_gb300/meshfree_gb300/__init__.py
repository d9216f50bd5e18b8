"""meshfree_gb300: GB300 (sm_103a) engine for the RBF-FD semidiscretization of
MeshfreeTrixi.jl, with a host API that mirrors the reference's point-cloud API."""
from ._lib import Context, MFTError, load  # noqa: F401
from .api import (  # noqa: F401
    RBF, BoundaryConditionDirichlet, BoundaryConditionDoNothing, BoundaryData,
    CompressibleEulerEquations2D, CompressibleEulerEquations3D, HistoryCallback,
    LinearScalarAdvectionEquation2D, LinearScalarAdvectionEquation3D, ODEProblem,
    Point1D, Point2D, Point3D, PointCloudBasis, PositivityPreservingLimiterZhangShu, density, pressure, PointCloudDomain, PointCloudDomain_from_medusa,
    PointCloudEnsemble, PointCloudSolver, PointData, PolyharmonicSpline, RBFFDEngineGB300, RBFSolver, RefPointData,
    SemidiscretizationHyperbolic, SourceHyperviscosityFlyer, SourceHyperviscosityTominec, SourceIGR,
    SaveCheckpointCallback, SourceResidualViscosityTominec, SourceTerms,
    SourceUpwindViscosityTominec, SSPRK33, boundary_condition_slip_wall, load_checkpoint, rhs_,
    rhs_adjoint_, save_checkpoint, semidiscretize, solve, solve_adjoint)
from .medusa import read_medusa_file  # noqa: F401
