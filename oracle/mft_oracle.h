/*
 * mft_oracle.h -- CPU restatement of the MeshfreeTrixi.jl RBF-FD semidiscretization
 * hot path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the
 * CPU-baseline leg of the benchmark call it as the checker.  The product library
 * (libmeshfree_gb300.so) never links or calls it.
 *
 * Pinning status (what this restatement is checked against):
 *   - reference known-answer test  test/history_test.jl:4-32       -> pinned
 *   - reference identity           test/divergence_test.jl:63-82   -> pinned
 *   - reference identity           test/upwind_viscosity_test.jl:66-78 -> pinned
 *   - saddle-point solve vs LAPACK dsytrf/dsytrs (the routine behind the
 *     reference's `Symmetric \`, compute_operators.jl:435), via scipy -> pinned
 *   - weights: polynomial reproduction on the reference fixture
 *     test/data/cyl_0_05_* (2154 nodes)                              -> pinned
 *   - whole rhs!/SSPRK trajectories against the Julia reference itself:
 *     parity unpinned (no Julia toolchain exists to run the reference).
 *
 * Arithmetic conventions: this file is compiled with -ffp-contract=off so every
 * a*b+c rounds twice, like Julia code outside @muladd (SparseArrays, Distances);
 * explicit fma() calls restate fused operations (the Bunch-Kaufman updates, as
 * optimised BLAS kernels perform them, and @muladd expressions of the limiter).
 */
#ifndef MFT_ORACLE_H
#define MFT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Julia's pairwise reduction (Base.mapreduce_impl, block size 1024) of a strided
 * double sequence: used for sum(u) in ode_mean and mean(dists) in PointData. */
double mfto_pairwise_sum(const double* x, int64_t n, int64_t stride);

/* A1  PointData(points, basis)  geometry_primatives.jl:322-339.
 * Exact k nearest neighbours of every node (self included), ordered by
 * (squared distance, node index).  d2 = (dx*dx) + (dy*dy) [+ (dz*dz)], no FMA,
 * as Distances.jl's Euclidean reduction.  `period` (dim entries) selects a
 * periodic minimum-image metric (extension; the reference has none), else NULL.
 * dists (optional) receives sqrt(d2).  dx_min = min nearest-neighbour distance,
 * dx_avg = pairwise mean of nearest-neighbour distances.  Returns 0 or <0. */
int mfto_knn(int dim, int64_t n, const double* x, const double* period, int k,
             int32_t* idx, double* dists, double* dx_min, double* dx_avg, int nthreads);

/* A2-A5  compute_flux_operator  compute_operators.jl:409-453 (first derivatives,
 * deriv_order = 1) and :549-594 (pure deriv_order-th derivatives).
 * Stencil of node e is stencil[rowptr[e] .. rowptr[e+1]), centre first.
 * Output w[(rowptr[e]+j)*dim + d] = weight of stencil node j for d/dx_d^order.
 * resid (optional, per node): max_col ||M w - b||_inf / ||b||_inf.
 * Returns 0, or -(e+1) for the first node whose factorisation met an exactly
 * singular pivot (weights of that node are then NaN). */
int mfto_weights(int dim, int64_t n, const double* x, const double* period,
                 const int64_t* rowptr, const int32_t* stencil, int rbf_pow, int polydeg,
                 int deriv_order, double* w, double* resid, int nthreads);

/* mfto_weights restricted to the listed rows (nrows node indices in rows); only
 * those rows' entries of w are written. */
int mfto_weights_rows(int dim, int64_t n, const double* x, const double* period,
                      const int64_t* rowptr, const int32_t* stencil, int rbf_pow, int polydeg,
                      int deriv_order, double* w, int nthreads, int64_t nrows,
                      const int64_t* rows);

/* Node e's saddle-point system as mfto_weights builds it: full symmetric M
 * (n x n), rhs b (n x dim), both column-major, and the axis scales s (dim).
 * Returns n = k + number of monomials. */
int mfto_saddle_system(int dim, const double* x, const double* period, const int64_t* rowptr,
                       const int32_t* stencil, int rbf_pow, int polydeg, int deriv_order,
                       int64_t e, double* m_out, double* b_out, double* s_out);

/* Bunch-Kaufman LDL^T (upper) factor + solve of one dense symmetric system,
 * column-major a[n*n] (upper triangle read, overwritten), b[n*nrhs] overwritten.
 * Restates the LAPACK dsytf2/dsytrs algorithm used by `Symmetric \`.
 * Returns 0, or k>0 when D(k,k) is exactly zero. */
int mfto_bk_solve(int n, double* a, int nrhs, double* b);

/* Equation kinds and boundary-condition kinds. */
enum { MFTO_EQ_EULER2D = 0, MFTO_EQ_ADVECTION = 1, MFTO_EQ_EULER3D = 2 };
enum { MFTO_BC_DIRICHLET = 0, MFTO_BC_SLIP_WALL = 1, MFTO_BC_DO_NOTHING = 2 };
enum { MFTO_SRC_RV = 0, MFTO_SRC_UPWIND = 1, MFTO_SRC_HV_TOMINEC = 2, MFTO_SRC_HV_FLYER = 3,
       MFTO_SRC_IGR = 4 };

/* Compressed sparse rows with ascending columns (CSR), plus the same operator
 * stored by columns (CSC) for transposed products. */
typedef struct {
  int64_t n;
  const int64_t* rp;  /* n+1 */
  const int32_t* ci;  /* nnz, ascending within a row */
  const double* val;  /* nnz */
  const int64_t* cp;  /* n+1   (CSC) */
  const int32_t* ri;  /* nnz, ascending within a column */
  const double* valt; /* nnz   values D[ri, col] */
} mfto_csr;

typedef struct {
  int dim, nvars, eq;
  double gamma;
  double adv[3];
  int64_t n;
  mfto_csr dop[3];       /* D_x, D_y (, D_z) */
  /* boundary conditions in NamedTuple order */
  int n_bc;
  const int* bc_kind;
  const int64_t* bc_ptr; /* n_bc+1 offsets into bc_idx */
  const int32_t* bc_idx;
  const double* bc_normal; /* (bc_ptr[n_bc]) x dim */
  /* sources in NamedTuple order */
  int n_src;
  const int* src_kind;
  /* residual / upwind viscosity parameters */
  double c_rv, c_uw, h;
  int success_iter;
  const double* approx_du; /* nvars x n (SoA) */
  int mean_mode;           /* 0: sum/(n*nvars) as Trixi recursive_length; 1: sum/n per component */
  int max_mode;            /* 0: lexicographic maximum (Base.isless on vectors); 1: per component */
  /* hyperviscosity: materialised operator H (CSR only) and its scale */
  mfto_csr hv;
  double hv_gamma;
  /* information geometric regularisation (SourceIGR): alpha and CG iteration cap */
  double igr_alpha;
  int igr_maxiter;
  double* igr_sigma; /* optional n output: sigma of the last evaluation */
} mfto_semi;

/* Diagnostics of the last residual-viscosity evaluation (optional output). */
typedef struct {
  double mean[8];
  double norms[8];
} mfto_rv_diag;

/* A7  Trixi.rhs!  rbfsolver.jl:397-428.  u, du: nvars pointers to length-n
 * arrays (StructArray SoA).  u is mutated at boundary nodes (strong BCs).
 * dirichlet (optional) holds the boundary value g(x,t) for every node listed
 * under a Dirichlet BC, nvars values per listed node in bc_idx order.
 * eps_out (optional) receives the viscosity of the last RV/upwind source. */
int mfto_rhs(const mfto_semi* s, double t, const double* dirichlet, double* const* du,
             double* const* u, double* eps_out, mfto_rv_diag* diag, int nthreads);

/* Adjoint of rhs! at state u (extension: the reference differentiates rhs! with
 * ForwardDiff duals).  out = (d rhs!(u)/du)^T lam for the flux divergence
 * (calc_fluxes!, rbfsolver.jl:247-265), the strong BCs (bc_pass above: Dirichlet
 * rows/values constant, slip-wall momentum projection) and the hyperviscosity
 * sources (du -= gamma*H*u).  u and lam are nvars pointers of length n; u is not
 * mutated.  Returns -1 when a residual/upwind viscosity source is present (its
 * viscosity is a maximum over the field and has no adjoint here). */
int mfto_rhs_adjoint(const mfto_semi* s, const double* const* u, const double* const* lam,
                     double* const* out, int nthreads);
/* Zhang-Shu positivity limiter on a point cloud, one variable pass of
 * limiter_zhang_shu! (src/callbacks_stage/positivity_zhang_shu_point2d.jl:22-82):
 * per node e, value_min = min over e's stencil of variable(u); where
 * value_min < threshold, u_mean = (sum over the stencil of u) / stencil size,
 * theta = (variable(u_mean) - threshold) / (variable(u_mean) - value_min) and the new
 * state is muladd(theta, u[e], (1 - theta) u_mean), applied after all nodes are
 * computed (a zero result leaves the node unchanged, as the reference's test does).
 * variable: 0 density, 1 pressure (Euler, gamma).  Stencils in the given order
 * (rowptr, cols).  u: nvars pointers, mutated.  Returns the number of limited nodes.
 * The reference divides by the global neighbour count; it equals the stencil size
 * for the uniform stencils it supports. */
int64_t mfto_limiter_zhang_shu(int64_t n, int nvars, double gamma, const int64_t* rowptr,
                               const int32_t* cols, int variable, double threshold,
                               double* const* u);
/* Pieces of rhs! exposed for the reference's own identity tests. */
int mfto_calc_fluxes(const mfto_semi* s, double* const* du, double* const* u, int nthreads);
/* y += alpha * A x (SparseArrays 5-arg mul!, CSC column scatter == ascending CSR rows) */
void mfto_spmv_accum(const mfto_csr* a, double alpha, const double* x, double* y, int nthreads);
/* y = A x (3-arg mul!) */
void mfto_spmv(const mfto_csr* a, const double* x, double* y, int nthreads);
/* y += alpha * A' x (mul! with an Adjoint of CSC) */
void mfto_spmv_t_accum(const mfto_csr* a, double alpha, const double* x, double* y, int nthreads);

/* H = A' * A as SparseArrays spmatmul forms it (per entry: ascending k, product
 * then add).  Two-call protocol: with hcol == NULL only hrp (n+1) is filled;
 * the second call fills hci/hval.  Columns ascending within a row. */
int mfto_ata(const mfto_csr* a, int64_t* hrp, int32_t* hci, double* hval, int nthreads);
void mfto_csr_to_csc(int64_t n, const int64_t* rp, const int32_t* ci, const double* val,
                     int64_t* cp, int32_t* ri, double* valt);

/* A16  time_deriv_weights!  history.jl:131-152:  w = scale * (A' \ b). */
int mfto_time_deriv_weights(int m, const double* t, double* w);

#ifdef __cplusplus
}
#endif
#endif
