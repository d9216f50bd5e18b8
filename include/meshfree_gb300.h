/*
 * meshfree_gb300.h -- C ABI of libmeshfree_gb300.so, the GB300 (sm_103a) engine for
 * the RBF-FD semidiscretization hot path of MeshfreeTrixi.jl.
 *
 * The reference selects its compute backend through the engine field of
 * RBFSolver{Basis,Engine} (src/solvers/rbfsolver.jl:68-71), chosen with
 * PointCloudSolver(basis; engine=...) (src/solvers/pointcloudsolver/types.jl:71-74).
 * Its CUDA engine is an empty stub (RBFFDEngineCUDA, src/solvers/rbfsolver.jl:60-61).
 * A Julia engine type `RBFFDEngineGB300 <: AbstractRBFEngine` binds the entry points
 * below with ccall; each entry point names the reference function it replaces.
 *
 * Conventions
 *  - Every function returns mft_status (0 = MFT_OK).  Nothing aborts, throws across
 *    the ABI or traps on the device.  mft_last_error() describes the last failure.
 *  - Host arrays are read during the call only; nothing is retained.
 *  - Node indices are 0-based int32 unless a function says otherwise (mft_load_csc
 *    takes the reference's 1-based Int64 CSC arrays as they are).
 *  - State arrays follow the reference's StructArray layout: nvars separate arrays of
 *    length n (one per conserved variable), passed as an array of nvars pointers.
 *  - One context = one CUDA stream on one device; a context is not re-entrant.
 */
#ifndef MESHFREE_GB300_H
#define MESHFREE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mft_ctx mft_ctx;
typedef int mft_status;

enum {
  MFT_OK = 0,
  MFT_ERR_ARG = 1,         /* invalid argument or inconsistent sizes */
  MFT_ERR_CUDA = 2,        /* CUDA runtime error (message in mft_last_error) */
  MFT_ERR_STATE = 3,       /* call out of order (e.g. rhs before operators) */
  MFT_ERR_SINGULAR = 4,    /* a local saddle-point system had an exactly zero pivot */
  MFT_ERR_NONFINITE = 5,   /* a du or stage value became NaN/Inf (outputs still written) */
  MFT_ERR_TIMEOUT = 6,     /* a bounded device wait gave up */
  MFT_ERR_UNSUPPORTED = 7, /* configuration not provided by this engine */
  MFT_ERR_NOMEM = 8        /* device or host allocation failed */
};

/* Equation kinds (Trixi equation types used with point clouds). */
enum { MFT_EQ_EULER2D = 0, MFT_EQ_ADVECTION = 1, MFT_EQ_EULER3D = 2 };

/* Boundary-condition kinds (src/equations/PointCloudBCs.jl). */
enum { MFT_BC_DIRICHLET = 0, MFT_BC_SLIP_WALL = 1, MFT_BC_DO_NOTHING = 2 };

/* Source kinds (src/sources/hyperviscosity.jl). */
enum { MFT_SRC_RV = 0, MFT_SRC_UPWIND = 1, MFT_SRC_HV_TOMINEC = 2, MFT_SRC_HV_FLYER = 3,
       MFT_SRC_IGR = 4 };

/* Operator slots. MFT_OP_GRAD holds D_1..D_dim (compute_flux_operator(solver, domain));
 * MFT_OP_LAP holds sum_d D_d^(2) (Tominec HV builds lap'*lap from it);
 * MFT_OP_HV holds a ready hyperviscosity operator sum_d D_d^(2k) (Flyer HV). */
enum { MFT_OP_GRAD = 0, MFT_OP_LAP = 1, MFT_OP_HV = 2 };

/* Arithmetic of the operator apply.  FP64: FP64 weights and states, sums accurate to
 * FP64 (double-word FP32 or FP64 fused multiply-adds, see MFT_OPT_FP64_ARITH).
 * FP32: weights generated in FP64 and stored FP32, FP32 states and sums in the apply;
 * the state stays FP64 and the SSP-RK stage combination is evaluated in FP64 (the FP64
 * state carries the low-order part that a compensated FP32 state would keep, so no
 * separate compensation term is formed). */
enum { MFT_PREC_FP64 = 0, MFT_PREC_FP32 = 1 };

/* ---------------------------------------------------------------- context */

/* Creates a context on CUDA device `device`.  flags: reserved, pass 0. */
mft_status mft_ctx_create(mft_ctx** ctx, int device, int flags);
mft_status mft_ctx_destroy(mft_ctx* ctx);
/* Text of the last error on this context (never NULL; "" if none). */
const char* mft_last_error(const mft_ctx* ctx);
mft_status mft_version(int* major, int* minor, int* patch);
/* Blocks until all work queued on the context stream has finished. */
mft_status mft_sync(mft_ctx* ctx);

/* ---------------------------------------------------------------- geometry */

/* Node coordinates, n x dim row-major (the reference's Vector{SVector{dim}}).
 * period: dim box lengths for a periodic (minimum-image) metric, or NULL.
 * Replaces the point input of PointData (src/domains/PointCloudDomain/
 * geometry_primatives.jl:322-339).  Resets stencils and operators. */
mft_status mft_set_points(mft_ctx* ctx, int dim, int64_t n, const double* xyz,
                          const double* period);

/* Exact k nearest neighbours of every node (self first), ordered by (squared
 * distance, node index), computed on the GPU; they become the context stencils.
 * Replaces KDTree + knn(tree, points, nv, true) and the dx_min / dx_avg statistics
 * of PointData (geometry_primatives.jl:327-334).  out_idx (n*k, host) and
 * out_dist (n*k, host) may be NULL. */
mft_status mft_knn(mft_ctx* ctx, int k, int32_t* out_idx, double* out_dist, double* out_dx_min,
                   double* out_dx_avg);

/* Ragged stencils given by the caller (centre first): rowptr[n+1], cols[rowptr[n]].
 * Replaces domain.pd.neighbors.  Stencil sizes may differ per node. */
mft_status mft_set_stencils(mft_ctx* ctx, const int64_t* rowptr, const int32_t* cols);

/* ---------------------------------------------------------------- weights */

/* Batched FP64 polyharmonic-spline (r^rbf_pow) + polynomial (total degree polydeg)
 * saddle-point solves, one per node, for pure derivatives of order deriv_order along
 * every axis, in one persistent launch bucketed by stencil size.  Replaces
 * compute_flux_operator(solver, domain) (compute_operators.jl:409-453, deriv_order 1)
 * and compute_flux_operator(solver, domain, k) (:549-594).  The result is stored in
 * operator slot `op`: MFT_OP_GRAD takes the dim components as they are, MFT_OP_LAP and
 * MFT_OP_HV take their sum over axes (as `sum(...)` at hyperviscosity.jl:44,111).
 * out_w (host, rowptr[n]*dim, [slot][axis]) may be NULL; out_max_resid receives
 * max over nodes of ||M w - b||_inf / ||b||_inf when not NULL. */
mft_status mft_weights(mft_ctx* ctx, int op, int rbf_pow, int polydeg, int deriv_order,
                       double* out_w, double* out_max_resid);

/* One group of a weight batch: `n` stencils over the group's own point cloud (host
 * arrays: xyz n*dim, rowptr n+1 starting at 0, cols rowptr[n] with the centre first,
 * w rowptr[n]*dim out in stencil order [slot][axis]); PHS r^rbf_pow with polynomials of
 * degree polydeg, derivatives of order deriv_order along each axis. */
typedef struct {
  int dim;
  int64_t n;
  const double* xyz;
  const int64_t* rowptr;
  const int32_t* cols;
  int rbf_pow, polydeg, deriv_order;
  double* w;
} mft_weight_group;

/* Weights of up to two groups (e.g. a 2D and a 3D cloud, uneven stencil sizes) solved
 * together in one persistent launch, largest systems first; per-node solves as
 * compute_flux_operator (compute_operators.jl:409-453, :549-594) performs them, with
 * the same arithmetic as mft_weights.  max_resid (optional): max over nodes of
 * ||M w - b||_inf / ||b||_inf.  The context only provides the stream and device. */
mft_status mft_weights_batch(mft_ctx* ctx, int ngroups, const mft_weight_group* groups,
                             double* max_resid);

/* Allocation-free weights (no counterpart in the reference).  For callers that cannot
 * allocate device memory during the solve -- code running inside a stream-ordered pool
 * it does not own, or a host whose allocator must not be bypassed by cudaMalloc (which
 * also synchronises the device).  Same numbers as mft_weights(MFT_OP_GRAD ...) on the
 * same stencils, without a context: every input and output is caller-owned device
 * memory (xyz n*dim, rowptr n+1, cols rowptr[n] with centre first, w rowptr[n]*dim in
 * stencil order [slot][axis]); period is a host array of dim lengths or NULL; stream
 * may be 0.  kmax: the caller's bound on the stencil size; kmax + number of monomials
 * must be <= 161 (shared-memory limit), else MFT_ERR_ARG with the reason in err.  The
 * device arrays are checked on the device before any coordinate is read: a stencil
 * longer than kmax, an empty stencil, a row outside [0, rowptr[n]) or a column outside
 * 0..n-1 is skipped, its weights (where its row lies inside cols) are set to NaN, and
 * the call returns MFT_ERR_ARG; the other stencils are solved.  The only global
 * scratch is a 32-byte static device array per GPU; its address is looked up on the
 * first call on each device (make that call before any stream capture; a
 * cudaDeviceReset after it is not supported), and it is reset at the start of every
 * call.  Calls that overlap on the GPU (other streams, other host threads) share that
 * array and race.  Blocks until the solve finished.  err (may be NULL) receives a
 * message of at most err_len bytes. */
mft_status mft_weights_noalloc(int dim, int64_t n, const double* xyz, const double* period,
                               const int64_t* rowptr, const int32_t* cols, int kmax,
                               int rbf_pow, int polydeg, int deriv_order, double* w,
                               void* stream, char* err, int err_len);

/* Loads one component of an operator from the reference's SparseMatrixCSC arrays
 * (1-based colptr[n+1], rowval[nnz], nzval[nnz]), e.g.
 * semi.cache.rbf_differentiation_matrices[comp+1] (rbfsolver.jl:139).  All loaded
 * operators must share one sparsity pattern. */
mft_status mft_load_csc(mft_ctx* ctx, int op, int comp, int64_t n, const int64_t* colptr,
                        const int64_t* rowval, const double* nzval);

/* ---------------------------------------------------------------- physics */

/* kind MFT_EQ_EULER2D: params[0] = gamma (CompressibleEulerEquations2D, 2D clouds);
 * kind MFT_EQ_EULER3D: params[0] = gamma (CompressibleEulerEquations3D, 3D clouds, 5
 * variables);  kind MFT_EQ_ADVECTION: params[0..dim-1] = advection velocity
 * (LinearScalarAdvectionEquation2D / 3D).  On 3D clouds rhs! is the plain flux divergence
 * (calc_fluxes! over D_x, D_y, D_z, rbfsolver.jl:247-265) with Dirichlet and do-nothing
 * BCs, in the FP64 form (FP64 fused multiply-adds): the reference's viscosity sources,
 * slip walls, positivity limiter and IGR are written for the 2D Euler equations, and an
 * rhs! on a 3D cloud with any of them returns MFT_ERR_UNSUPPORTED, as does the adjoint. */
mft_status mft_set_equations(mft_ctx* ctx, int kind, const double* params);

/* Boundary conditions in the order of the reference's NamedTuple
 * (calc_boundary_flux!, rbfsolver.jl:277-318): kinds[n_bc], node lists
 * idx[ptr[b]..ptr[b+1]), outward normals normals[ptr[n_bc]*dim] (slip walls). */
mft_status mft_set_bcs(mft_ctx* ctx, int n_bc, const int* kinds, const int64_t* ptr,
                       const int32_t* idx, const double* normals);

/* Boundary values g(x, t) for the Dirichlet-listed nodes (ptr order, nvars each),
 * used by every following rhs evaluation until replaced
 * (BoundaryConditionDirichlet, PointCloudBCs.jl:49-63). */
mft_status mft_set_dirichlet_values(mft_ctx* ctx, const double* values);

/* Host callback that fills Dirichlet values for time t (same layout as above); when
 * set, the time integrator calls it before every stage instead of using fixed values. */
typedef void (*mft_dirichlet_fn)(double t, int64_t n_nodes, int nvars, double* values,
                                 void* user);
mft_status mft_set_dirichlet_callback(mft_ctx* ctx, mft_dirichlet_fn fn, void* user);

/* Sources in the order of SourceTerms (calc_sources!, rbfsolver.jl:388-395).
 * params: 4 doubles per source.
 *   MFT_SRC_RV      {c_rv, c_uw, h = dx_avg, mean_mode}  SourceResidualViscosityTominec
 *   MFT_SRC_UPWIND  {c_uw, h = dx_avg, 0, 0}             SourceUpwindViscosityTominec
 *   MFT_SRC_HV_TOMINEC {gamma = c*dx_min^4.5, 0, 0, 0}   SourceHyperviscosityTominec
 *   MFT_SRC_HV_FLYER   {gamma = c*dx_min^(2k), 0, 0, 0}  SourceHyperviscosityFlyer
 *   MFT_SRC_IGR     {alpha, max CG iterations (20), 0, 0}  SourceIGR (src/sources/IGR.jl):
 *                   (rho^-1 - alpha (Dx rho^-1 Dx + Dy rho^-1 Dy)) sigma =
 *                   alpha (tr(Du)^2 + tr(Du^2)) by conjugate gradients from 0 (relative
 *                   tolerance sqrt(eps)), then du[rho v] -= (Dx sigma, Dy sigma); 2D Euler
 * mean_mode 0: ode_mean divides by n*nvars (Trixi recursive_length); 1: by n. */
mft_status mft_set_sources(mft_ctx* ctx, int n_src, const int* kinds, const double* params);

mft_status mft_set_precision(mft_ctx* ctx, int precision);

/* Ensembles: the context holds nseg independent point clouds back to back; member m owns
 * nodes [offsets[m], offsets[m+1]) (offsets[0] = 0, offsets[nseg] = n) and its stencils
 * must stay inside the member.  The residual-viscosity normalisation (ode_mean /
 * ode_maximum, src/auxiliary/mpi.jl:40-81) is then taken per member, and h[m] is the
 * member's dx_avg (replacing the source's h).  nseg = 0 returns to one problem. */
mft_status mft_set_segments(mft_ctx* ctx, int nseg, const int64_t* offsets, const double* h);

/* Engine options.  MFT_OPT_GATHER selects the mapping of the FP32 operator gathers:
 * MFT_GATHER_THREAD (one node per thread, direct loads), MFT_GATHER_STAGED (one warp
 * per 32-node slice with the slice's indices and weights streamed into shared memory by
 * bulk copies), MFT_GATHER_HALO (one node per thread, each group of 256 (or 128)
 * layout rows staging its distinct neighbour records in shared memory first), or
 * MFT_GATHER_AUTO (default: the autotuner times the three on the live inputs). */
enum { MFT_OPT_GATHER = 0, MFT_OPT_TUNED_FWD = 1, MFT_OPT_TUNED_REV = 2,
       MFT_OPT_FP64_ARITH = 3, MFT_OPT_LAYOUT_ORDER = 4, MFT_OPT_DW_VARIANT = 5,
       MFT_OPT_HALO_STAGED_FWD = 6, MFT_OPT_HALO_STAGED_REV = 7, MFT_OPT_HALO_GROUPS = 8,
       MFT_OPT_IGR_ITERS = 9, MFT_OPT_ADJ_EVERY = 10, MFT_OPT_HALO_ROWS = 11,
       MFT_OPT_ENTRY_ORDER = 12, MFT_OPT_BANK_FWD = 13, MFT_OPT_BANK_REV = 14,
       MFT_OPT_FUSE_FLUX = 15, MFT_OPT_FLUX_FUSED = 16 };
/* MFT_OPT_FUSE_FLUX (default 1): in the double-word form, when every row group is staged
 * and the forward gather's variant is 7, 11 or 12, that gather forms each staged
 * neighbour's state and flux pairs from the FP64 state while staging, and the separate
 * flux kernel (which writes those pairs for every node) is skipped; 0 always runs it.  The
 * results are the same bits either way.  Read-only MFT_OPT_FLUX_FUSED: 1 when the last
 * evaluation formed the pairs in the gather. */
/* MFT_OPT_ENTRY_ORDER: order of the entries inside the rows of the staged row groups
 * (which is the order each row's sum runs in, for every gather variant of that layout):
 * 1 (default) spreads the shared-memory reads of the 8 lanes of each quarter-warp over
 * the bank groups, slot by slot; 0 keeps the structure's (ascending-column) order.  The
 * layouts are rebuilt on change; sums differ between the two in the last bits only.
 * Read-only MFT_OPT_BANK_FWD / _REV: for the staged forward / transpose gathers' layout,
 * the mean number of serialised shared-memory accesses per quarter-warp record load
 * (1000 = conflict-free), counted on the host when the layout is built; 0 before. */
/* MFT_OPT_HALO_ROWS: layout rows per staged group (= threads per block of the staged
 * gathers): 0 (default) picks 256, or 128 on 3D clouds and when 256-row groups would give
 * every SM fewer than four; 128 or 256 fixes it (the layouts are rebuilt).  Read back: the size in use
 * (0 when no staged layout is built). */
/* Read-only MFT_OPT_IGR_ITERS: conjugate-gradient iterations of the last IGR solve
 * (-1 before the first).  Read-only MFT_OPT_ADJ_EVERY: the checkpoint interval of the last
 * mft_ssprk33_record (0: every stage state stored). */
/* Read-only (mft_get_option): MFT_OPT_HALO_GROUPS = row groups of the staged layouts
 * (MFT_OPT_HALO_ROWS layout rows each), MFT_OPT_HALO_STAGED_FWD / _REV = how many of them
 * have their neighbour records staged in shared memory by the staged gathers (the others
 * gather directly); 0 before the first evaluation in the double-word (2D or 3D Euler) or
 * FP32 2D Euler form. */
/* MFT_OPT_DW_VARIANT: kernel variant of the double-word gathers -- 0 one stencil entry
 * per loop iteration, 1 two entries per iteration with registers capped at six blocks per
 * SM, 2 two entries uncapped, 3 software-pipelined (indices two entries ahead, weights and
 * neighbour records one ahead), 4 and 5 = 1 and 2 with each warp's streamed index and
 * weight arrays prefetched into L2 eight slots ahead (one bulk prefetch per array),
 * 6 and 7 = 0 and 2 with the distinct neighbour records of each group of 256 (or 128)
 * layout rows staged in shared memory by coalesced asynchronous copies and read from there (16-bit
 * positions instead of the 32-bit indices; a group with more than 640 distinct
 * neighbours gathers directly; registers capped at three blocks per SM), 8 = 7 capped at
 * four blocks per SM, 9 and 11 = staged with four and three entries per iteration, 10 = 7
 * with the streamed position and weight arrays prefetched into L2 as in 4, 12 = 7 with L2
 * eviction-priority hints (streamed arrays evict-first, the intermediates the transpose
 * gather reads back evict-last);
 * -1 (default) lets the autotuner time them at the first launch of each configuration.
 * Every variant forms the same sums in the same order (bit-identical results).
 * MFT_OPT_TUNED_FWD / MFT_OPT_TUNED_REV then report the variant in use. */
/* MFT_OPT_LAYOUT_ORDER: 1 (default) assigns the operator rows to threads along a Morton
 * curve of the node coordinates, so that a warp's 32 rows are a compact patch whose
 * neighbours overlap; 0 keeps node order.  Results are identical either way (every row
 * keeps its own summation order); only the memory locality of the gathers changes. */
enum { MFT_GATHER_AUTO = 0, MFT_GATHER_THREAD = 1, MFT_GATHER_STAGED = 2, MFT_GATHER_HALO = 3 };
/* MFT_OPT_FP64_ARITH: how the FP64 form's operator gathers form their sums of products.
 * MFT_ARITH_DFMA: FP64 fused multiply-adds.  MFT_ARITH_DW: double-word FP32 arithmetic
 * (weights, fluxes and neighbour states as unevaluated float pairs h + l, error-free
 * products and sums on the FP32 pipe, ~48-bit significands; per-node values, the
 * viscosity and the stage combination stay FP64); 2D Euler only, other equations use
 * DFMA.  MFT_ARITH_AUTO (default) = MFT_ARITH_DW.  mft_get_option returns the setting. */
enum { MFT_ARITH_AUTO = 0, MFT_ARITH_DFMA = 1, MFT_ARITH_DW = 2 };
mft_status mft_set_option(mft_ctx* ctx, int option, int value);
/* Reads an option; MFT_OPT_TUNED_FWD / MFT_OPT_TUNED_REV return the mapping the
 * autotuner chose for the most recent forward / transpose gather launch: FP32 form
 * 0 = one node per thread, 4 or 8 = staged with that many slots per bulk copy; FP64
 * form with double-word gathers: the kernel variant 0..5; -1 = not tuned yet. */
mft_status mft_get_option(mft_ctx* ctx, int option, int* value);

/* Self-test of the bounded-wait error path (no fault involved): one warp waits on a
 * shared-memory mbarrier that nothing completes, gives up after `polls` polls (1 ..
 * 1,000,000), records MFT_ERR_TIMEOUT in the device error word and returns; the host
 * reads the word as every staged gather's caller does.  Returns MFT_ERR_TIMEOUT (the
 * expected outcome) with the context still usable. */
mft_status mft_selftest_bounded_wait(mft_ctx* ctx, int polls);

/* Arithmetic-rate probe (no counterpart in the reference): the FMA throughput of the
 * context's GPU, kind 0 = FP64 fused multiply-adds, 1 = FP32 ones, per second (many
 * independent chains on every SM, best of three timed launches).  It is the
 * denominator of the FP64-issue roofline that the benchmark reports. */
mft_status mft_measure_fma_rate(mft_ctx* ctx, int kind, double* per_second);

/* ---------------------------------------------------------------- rhs! */

/* du = rhs!(u, t) with host StructArray-style arrays (nvars pointers of length n).
 * u is mutated at boundary nodes as the reference's strong BCs do.  Replaces
 * Trixi.rhs!(du, u, t, domain, equations, ic, bcs, sources, solver, cache)
 * (rbfsolver.jl:397-428), calc_fluxes! (:247-265) and the source functors. */
mft_status mft_rhs(mft_ctx* ctx, double* const* du, double* const* u, int nvars, double t);

/* Same on device memory owned by the caller: u and du are nvars x n (SoA) FP64. */
mft_status mft_rhs_device(mft_ctx* ctx, double* du, double* u, double t);

/* ---------------------------------------------------------------- time integration */

/* Device-resident state: upload / download (host SoA pointers). */
mft_status mft_set_state(mft_ctx* ctx, const double* const* u, int nvars, double t);
mft_status mft_get_state(mft_ctx* ctx, double* const* u, int nvars, double* t);

/* Enables the HistoryCallback (src/callbacks_step/history.jl:43-152) with the given
 * reconstruction order; it runs after every accepted step. */
mft_status mft_history_init(mft_ctx* ctx, int approx_order);

/* Advances nsteps SSP-RK3 (Shu-Osher, FSAL) steps of size dt on the device state,
 * each step captured as one CUDA graph when use_graph != 0. */
mft_status mft_ssprk33(mft_ctx* ctx, double dt, int nsteps, int use_graph);

/* One step from host memory: uploads u, advances nsteps, downloads u (in place). */
mft_status mft_ssprk33_host(mft_ctx* ctx, double* const* u, int nvars, double* t, double dt,
                            int nsteps);

/* Sets the fields of the residual-viscosity cache that the HistoryCallback
 * maintains: approx_du (host StructArray-style, may be NULL to keep it) and
 * success_iter (SourceResidualViscosityTominec cache, hyperviscosity.jl:202-244;
 * written by modify_cache!, history.jl:91-103). */
mft_status mft_set_rv_state(mft_ctx* ctx, const double* const* approx_du, int nvars,
                            int success_iter);

/* Viscosity of the last RV/upwind source evaluation (host, n values). */
mft_status mft_get_viscosity(mft_ctx* ctx, double* eps);

/* ---------------------------------------------------------------- checkpoint / resume
 * The time-integration state of a context as one byte image, so that a run can stop and
 * resume bit for bit: t, the device state u_n, the pending first SSP-RK3 stage (first
 * same as last), the step-time origin, and the HistoryCallback's ring (times, states,
 * approx_du, success_iter).  The reference writes solution files only
 * (src/callbacks_step/save_solution_vtk.jl:158-194) and has no restart; this has no
 * counterpart there.  The operators, BCs, sources, options and limiter are not in the
 * image: the resuming context is set up as the saving one was (a pending stage from
 * another precision or gather arithmetic is dropped and recomputed).  The image starts
 * with the 8 bytes "MFTCKPT\0", is in host byte order and ends with an FNV-1a 64-bit hash
 * of the bytes before it; mft_checkpoint_load returns MFT_ERR_ARG for a truncated,
 * corrupted or foreign image, or one of another problem size, and changes nothing then. */
mft_status mft_checkpoint_size(mft_ctx* ctx, size_t* bytes);
mft_status mft_checkpoint_save(mft_ctx* ctx, void* buf, size_t bytes);
mft_status mft_checkpoint_load(mft_ctx* ctx, const void* buf, size_t bytes);

/* ---------------------------------------------------------------- positivity limiter
 * PositivityPreservingLimiterZhangShu(; thresholds, variables)
 * (src/callbacks_stage/positivity_zhang_shu.jl:22-66 with the point-cloud kernel
 * limiter_zhang_shu!, positivity_zhang_shu_point2d.jl:22-82), used as the stage limiter
 * of SSP-RK3: after every stage of mft_ssprk33 / mft_ssprk33_host, one pass per
 * variable in the given order.  2D Euler only.  A node's stencil is its operator row;
 * the stencil mean divides by that node's stencil size (the reference divides by the
 * global neighbour count, the same number for its uniform stencils). */
enum { MFT_LIM_DENSITY = 0, MFT_LIM_PRESSURE = 1 };

/* nvar (<= 4) variables with their thresholds; nvar = 0 turns the limiter off. */
mft_status mft_set_limiter(mft_ctx* ctx, int nvar, const int* variables,
                           const double* thresholds);

/* One application of the configured limiter to host StructArray-style arrays u (nvars
 * pointers of length n), in place: Trixi.limiter_zhang_shu!(u, thresholds, variables,
 * ...) (positivity_zhang_shu.jl:44-66). */
mft_status mft_limit(mft_ctx* ctx, double* const* u, int nvars);

/* ---------------------------------------------------------------- adjoint
 * Reverse-mode derivatives of rhs! and of the SSP-RK3 trajectory.  No function of
 * the reference corresponds: MeshfreeTrixi.jl differentiates rhs! only through
 * ForwardDiff.jl duals; these entry points are what a ChainRulesCore rrule for
 * rhs! and for solve() would call.  Covered: 2D Euler and linear advection, the
 * strong BCs (Dirichlet, slip wall, do-nothing), the hyperviscosity sources, the
 * residual-viscosity and upwind-viscosity sources (differentiated with their selections
 * -- min(eps_rv, eps_uw), the maximum over variables, the row of ode_maximum, |.| --
 * frozen as the forward evaluation takes them: the derivative away from ties; approx_du
 * and success_iter are inputs, as mft_set_rv_state leaves them), FP64.  A viscosity
 * source after a hyperviscosity source, or in an ensemble, gives MFT_ERR_UNSUPPORTED.
 * The recorded trajectory does not run the HistoryCallback: its residual viscosity uses
 * the approx_du and success_iter in place when recording starts. */

/* out = (d rhs!(u, t) / du)^T lam with host StructArray-style arrays (nvars pointers
 * of length n).  u is not mutated. */
mft_status mft_rhs_adjoint(mft_ctx* ctx, double* const* out, const double* const* lam,
                           const double* const* u, int nvars, double t);

/* Same on caller-owned device memory: out, lam, u are nvars x n (SoA) FP64. */
mft_status mft_rhs_adjoint_device(mft_ctx* ctx, double* out, const double* lam, const double* u,
                                  double t);

/* Advances the device state nsteps SSP-RK3 steps of size dt (the same arithmetic as
 * mft_ssprk33) and records the trajectory for mft_ssprk33_adjoint: the state every
 * `every` steps (the stage states are recomputed from these checkpoints during the
 * reverse sweep), or every stage state of every step when every == 0.  every == -1 picks:
 * every stage state when they take at most half of the free device memory (the sweep then
 * recomputes nothing), else checkpoints every ceil(sqrt(nsteps / 3)) steps; the choice is
 * read back through MFT_OPT_ADJ_EVERY. */
mft_status mft_ssprk33_record(mft_ctx* ctx, double dt, int nsteps, int every);

/* Reverse sweep over the recorded trajectory.  On entry lam (host StructArray-style)
 * holds dJ/du at the final state; on return it holds dJ/du at the initial state. */
mft_status mft_ssprk33_adjoint(mft_ctx* ctx, double* const* lam, int nvars);

/* Same on caller-owned device memory (nvars x n SoA FP64), in place. */
mft_status mft_ssprk33_adjoint_device(mft_ctx* ctx, double* lam);

/* ---------------------------------------------------------------- timing
 * Device timing with CUDA events on the context stream (the reference wraps the
 * same phases in @trixi_timeit timers, rbfsolver.jl:400-425). */

/* Kernel kinds reported by mft_profile_get. */
enum {
  MFT_K_BC = 0, MFT_K_FLUX, MFT_K_FWD, MFT_K_MEAN, MFT_K_LEXMAX, MFT_K_EPS, MFT_K_REV,
  MFT_K_REV_LAP, MFT_K_HISTORY, MFT_K_LAYOUT, MFT_K_ADJ, MFT_K_LIMITER, MFT_K_IGR,
  MFT_K_COUNT
};

/* enable != 0 starts recording an event pair around every kernel launch (and clears
 * the accumulated totals); 0 stops recording. */
mft_status mft_profile(mft_ctx* ctx, int enable);
/* Totals since mft_profile(ctx, 1) for one kernel kind: summed device milliseconds,
 * launch count and a static name. */
mft_status mft_profile_get(mft_ctx* ctx, int kind, double* total_ms, int64_t* launches,
                           const char** name);
/* begin != 0: records the start event of a timed region on the context stream;
 * begin == 0: records the stop event, waits for it and returns the region's device
 * time in *ms. */
mft_status mft_region(mft_ctx* ctx, int begin, double* ms);

#ifdef __cplusplus
}
#endif
#endif
