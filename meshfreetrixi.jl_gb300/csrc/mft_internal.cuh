// Internal declarations shared by the translation units of libmeshfree_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "meshfree_gb300.h"

namespace mft {

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define MFT_CUDA(call)                                                                      \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      throw ::mft::Error(MFT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define MFT_REQUIRE(cond, code, msg)                \
  do {                                              \
    if (!(cond)) throw ::mft::Error((code), (msg)); \
  } while (0)

#define MFT_LAUNCH_CHECK() MFT_CUDA(cudaGetLastError())

// Programmatic dependent launch.  A grid launched with launch_k(..., pdl = true) may start
// while the previous kernel in its stream still runs, once every block of that kernel has
// executed pdl_trigger() (or exited); before reading anything that kernel writes it must
// execute pdl_wait(), which returns when that kernel has completed and its writes are
// visible (at once for a grid launched without the attribute).  Everything earlier in the
// stream has completed before the previous kernel started, as with plain launches.
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline void launch_k(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                     bool pdl, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  MFT_CUDA(cudaLaunchKernelEx(&cfg, k, args...));
}

// Owning device buffer (cudaMalloc / cudaFree).
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void alloc(size_t count) {
    if (p && count == n) return;
    release();
    if (count) {
      cudaError_t e = cudaMalloc(&p, count * sizeof(T));
      if (e != cudaSuccess) {
        p = nullptr;
        throw Error(MFT_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
      }
      n = count;
    }
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    alloc(count);
    if (count) MFT_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void upload(const std::vector<T>& h, cudaStream_t s) { upload(h.data(), h.size(), s); }
  void zero(cudaStream_t s) {
    if (n) MFT_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
};

// Sliced ELL of a square sparse operator pattern: rows grouped in slices of 32
// (one warp), each slice padded to its longest row, slot-major inside a slice so
// that lane r of a warp reads element slice_off + slot*32 + r (coalesced).
constexpr int kSlice = 32;

// Row r of the layout holds node perm[r]'s row (perm null: node r).  slice_off and
// row_len are indexed by layout row; everything per node by perm[r].
// Neighbour halos of row groups: for each group of halo_rows consecutive layout rows (256,
// or 128 when 256-row groups would leave SMs idle), the
// distinct nodes its rows gather (ascending), at most kHaloMax of them, and per ELL
// element the element's position in its group's list.  A gather kernel stages a group's
// neighbour records into shared memory once with coalesced copies and reads them from
// there, instead of one scattered global load per element.  Groups with more distinct
// neighbours have an empty list and gather directly.  The rows of the groups with a list
// may take their entries in a bank-spreading order (build_ell, spread).
constexpr int kHaloRows = 256;  // largest group (and block) size
constexpr int kHaloMax = 640;

struct EllView {
  int64_t n;
  const int64_t* slice_off;
  const int32_t* row_len;
  const int32_t* col;
  const int32_t* perm;
  const int32_t* halo_off;   // groups + 1 offsets into halo_col (null: no halos built)
  const int32_t* halo_col;   // the groups' neighbour lists
  const uint16_t* lcol;      // per ELL element: position in its group's list
  int halo_stride;           // longest list (shared-memory stride of a staged chunk)
  int halo_rows;             // rows per group (= threads per block of a staged launch)
};

struct EllBuf {
  int64_t n = 0, n_elems = 0;
  int max_len = 0;
  int window = 0;  // rows sorted by length inside windows of this many rows (0: none)
  bool ordered = false;  // rows start from a spatial (Morton) order of the nodes
  DBuf<int64_t> slice_off;
  DBuf<int32_t> row_len;
  DBuf<int32_t> col;
  DBuf<int32_t> perm;
  DBuf<int32_t> halo_off, halo_col;
  DBuf<uint16_t> lcol;
  int64_t halo_groups = 0, halo_staged = 0;  // groups, and groups with a list
  int halo_stride = 0;
  int halo_rows = 0;
  bool spread = false;  // staged rows in the bank-spreading entry order
  int bank_milli = 0;   // staged loads: serialised accesses per quarter-warp load x 1000
  EllView view() const {
    return EllView{n,         slice_off.p, row_len.p,
                   col.p,     (window > 0 || ordered) ? perm.p : nullptr,
                   halo_off.p, halo_col.p, lcol.p,    halo_stride, halo_rows};
  }
};

__host__ __device__ __forceinline__ int64_t ell_node(const EllView& e, int64_t r) {
  return e.perm ? (int64_t)e.perm[r] : r;
}

// Host description of the boundary conditions, flattened per node for kernels.
struct BcDev {
  const int8_t* tag;      // n: 0 none, 1 Dirichlet, 2 slip wall
  const int32_t* slot;    // n: index into the per-boundary-node tables
  const double* normal;   // n_bnodes x 2 (raw outward normal, normalised in-kernel)
  const double* dvalues;  // n_bnodes x nvars (Dirichlet values of the current stage)
};

// Stage epilogue of the fused kernels (SSP-RK3 in Shu-Osher form, FSAL).
enum StageKind : int {
  kOutDu = 0,   // write du (rhs! output)
  kStage1 = 1,  // u_out = u_s + dt*du
  kStage2 = 2,  // u_out = ((3*u_n + u_s) + dt*du) / 4
  kStage3 = 3   // u_out = ((u_n + 2*u_s) + (2*dt)*du) / 3
};

struct Epilogue {
  int kind;
  double dt;
  const double* u_n;  // n x V (AoS) step-start state (stages 2, 3)
  double* u_s;        // n x V (AoS) stage state, mutated at slip nodes by BC pass 2
  double* out;        // n x V (AoS): du (kOutDu) or next stage state
  float* out32;       // optional FP32 shadow of the next stage state
  BcDev bc;
  int has_bc;
  const double* xadd; // n x 2 additions to the momentum rows (IGR source) or null
  // FP32-apply form: the stage combination as fused multiply-adds (within an ulp of the
  // FP64 form's separately rounded formulas, half the FP64 operations); cdt is dt / 4
  // (stage 2) or 2 dt / 3 (stage 3)
  int fused;
  double cdt;
  // device error word: MFT_ERR_NONFINITE is raised into it (atomic max, so a timeout
  // code stays) when a written du or stage value is NaN or infinite; null: no check
  int* err;
};

// ------------------------------------------------------------------ launchers
// (implemented in mft_apply.cu; all enqueue on `s` and return after launch)

void launch_aos_from_soa(const double* soa, double* aos, int64_t n, int V, cudaStream_t s);
void launch_soa_from_aos(const double* aos, double* soa, int64_t n, int V, cudaStream_t s);
void launch_aos_to_f32(const double* aos, float* a32, int64_t count, cudaStream_t s);
// out[pos[e]] = v[e] (and out32[pos[e]] = (float) v[e] when out32 is not null, and
// outdw[pos[e]] = the double-word pair of v[e] when outdw is not null): the operator
// values of structure entry e placed at their sliced-ELL element.
void launch_scatter_values(int64_t nnz, const int64_t* pos, const double* v, double* out,
                           float* out32, float2* outdw, cudaStream_t s);

// One pointer per variable (pinned host memory mapped for the device, or device memory).
struct VarPtrs {
  double* p[8];
};
void launch_aos_from_vars(const VarPtrs& src, double* aos, int64_t n, int V, cudaStream_t s);
void launch_vars_from_aos(const double* aos, const VarPtrs& dst, int64_t n, int V,
                          cudaStream_t s);

// BC pass 1 over the boundary-node list: Dirichlet u = g, slip wall u = slip(u).
void launch_bc_pass1(int64_t nb, const int32_t* bnode, int V, int eq, BcDev bc, double* u,
                     float* u32, cudaStream_t s);

// Flux precompute F(u) (Euler: n x 8) and optional block partial sums of u.
void launch_flux_f64(int64_t n, int eq, int V, double gamma, const double* u, double* F,
                     cudaStream_t s);

struct EpsArgs {
  int64_t n;
  int eq, V, kind;  // kind: MFT_SRC_RV or MFT_SRC_UPWIND
  double gamma, ax, ay, c_rv, c_uw, h;
  int success_iter;
  const struct StepParams* tab;  // graph mode: success_iter = tab[*ctr].si_eps
  const int* ctr;
  const int* seg_id;       // ensembles: segment of each node (null: one problem)
  const double* seg_h;     // ensembles: dx_avg per segment; norms hold 2V per segment
  // Node-independent factors, formed by launch_eps in the kernel's operation order
  // (one problem only; with seg_h the kernel forms them per node):
  double uw_coef;          // (c_uw * 0.5) * h
  double uw_adv;           // advection: uw_coef * sqrt(ax^2 + ay^2)
  double rv_coef;          // (0.5 * c_rv) * (h * h)
  double uw_bound;         // uw_coef^2 (1 - 1e-12) / (1 + 1e-12): the eps_uw bound's factor
  double gg1;              // gamma (gamma - 1): the sound speed's part of that bound
  // FP32 form: the FP32 shadow of u and the FP32 factors, formed by launch_eps in the
  // FP32 kernel's operation order
  const float* u32;
  float gamma32, gm1_32;   // (float) gamma, (float)(gamma - 1)
  float uw_coef32;         // ((float) c_uw * 0.5f) * (float) h
  float rv_coef32;         // ((0.5f * (float) c_rv) * (float) h) * (float) h
  const double* u;
  const double* du_p;
  const float* du_p32;     // FP32 apply: partial du in FP32 (du_p is then null)
  const double* hvf;       // added to du_p when the Flyer term precedes RV (else null)
  const double* approx_du; // n x V
  const double* norms;     // V
  double* t;               // n x 2V, scaled in place to eps*t
  double* eps;             // n (diagnostic copy)
  float* t32;              // FP32 path: scaled in place
  float2* tdw;             // double-word FP64 form: n x 2V pairs, scaled in place
};
// Node-independent factors of EpsArgs (uw_coef, uw_adv, rv_coef, uw_bound and the FP32
// ones), formed on the host in the kernels' operation order.
void prepare_eps(EpsArgs& a);

struct FwdArgs {
  int64_t n;
  EllView ell;
  const double* w[3];   // grad components (x, y, z)
  const double* wl;     // lap (Tominec) or H (Flyer) weights, or null
  const float* w32[3];
  const float* wl32;
  const double* F;      // n x 2V fluxes (Euler FP64; n x 3V on 3D clouds)
  const double* u;      // n x V state (FP64)
  const float* u32;     // n x V state (FP32 path)
  int eq, V;
  double gamma, ax, ay, az;
  double hv_gamma;      // Flyer: du += -gamma * H u
  float gm1_32, hg32;   // (float)(gamma - 1), (float) hv_gamma (FP32 kernels; set by the launchers)
  int want_t;           // write t = D u (n x 2V)
  int want_q;           // write q = lap u (n x V) (Tominec)
  int flyer;            // Flyer H in wl: 0 none, 1 add into du_p, 2 write hvf separately
  double* du_p;         // n x V partial du (flux [+ Flyer])
  double* t;            // n x 2V
  double* q;            // n x V
  double* hvf;          // n x V
  float* t32;
  float* q32;
  float* du_p32;
  int final_epilogue;   // 1: du is final here, apply BC2 + epilogue instead of writing du_p
  Epilogue ep;
  // FP64 form in double-word arithmetic (Euler): weights, fluxes and states as (h, l)
  // float pairs; t and q are written as pairs, du_p / hvf in FP64
  const float2* wdw[3];
  const float2* wldw;
  const float2* Fdw;    // n x 2V pairs
  const float2* udw;    // n x V pairs
  float2* tdw;          // n x 2V pairs
  float2* qdw;          // n x V pairs
  // double-word form with a viscosity source: the viscosity is formed in the epilogue
  // (ea, whose norms must be ready at launch) and t is written as s = eps * t
  int fuse_eps;
  EpsArgs ea;
  // double-word staged gathers: with fuse_flux the groups' state and flux pairs are formed
  // while staging, from ustate (the FP64 state after BC pass 1) and gm1dw (gamma - 1 as a
  // pair), instead of read from Fdw / udw (which the flux kernel then need not write).
  // Only when every row group is staged; a block of a group without a list sets *err.
  int fuse_flux;
  const double* ustate;
  float2 gm1dw;
  int* err;
  // launched as a programmatic dependent of the norm reductions just before it (the
  // viscosity epilogue waits for them; the staging and the sums do not)
  int pdl;
};
void launch_fwd_f64(const FwdArgs& a, cudaStream_t s);
// 3D clouds (mft_apply3d.cu): per-node Euler fluxes F = (F_x, F_y, F_z) (n x 15), and the
// plain flux divergence -sum_d D_d F_d with the stage epilogue (V = 5, Euler; V = 1,
// advection with the flux a_d u formed at the neighbour).
void launch_flux_euler3d(int64_t n, double gamma, const double* u, double* F, cudaStream_t s);
void launch_fwd3(const FwdArgs& a, cudaStream_t s);
// The same for 3D Euler in double-word arithmetic: flux pairs (n x 16 float2, the 15 of
// F_x, F_y, F_z and one pad) and the gather over the weight pairs a.wdw[0..2].
void launch_prep_euler3d_dw(int64_t n, double gamma, const double* u, float2* F,
                            cudaStream_t s);
void launch_fwd3_dw(const FwdArgs& a, cudaStream_t s);
// Double-word forms (mft_apply_dw.cu): per-node flux and state pairs, forward gather,
// transpose gather.
void launch_prep_euler_dw(int64_t n, double gamma, const double* u, float2* F, float2* U,
                          cudaStream_t s);
// variant: 0..12, the kernel variants the autotuner chooses among (same sums, same order)
constexpr int kDwVariants = 13;
void launch_fwd_dw(const FwdArgs& a, int variant, cudaStream_t s);
// Whether forward variant `variant` forms the flux pairs while staging when a.fuse_flux
// is set (the staged variants 7, 11 and 12).
bool dw_fwd_fuses(int variant);
// The pairs of gamma - 1 (h = RN32(gamma - 1), l = RN32 of the remainder).
float2 gm1_pair(double gamma);
void launch_fwd_f32(const FwdArgs& a, cudaStream_t s);

// Reductions for the residual viscosity normalisation (last-block-done pattern).
void launch_mean(int64_t n, int V, const double* u, double denom, double* partial,
                 unsigned* counter, double* mean, int nblocks, cudaStream_t s);
// pdl: launched as a programmatic dependent of the k_mean launch just before it
void launch_lexmax(int64_t n, int V, const double* u, const double* mean, int max_mode,
                   double* partial, unsigned* counter, double* norms, int nblocks,
                   cudaStream_t s, bool pdl = false);

void launch_eps(const EpsArgs& a, cudaStream_t s);
void launch_mean_seg(int nseg, const int64_t* off, int per, int V, const double* u, int mode,
                     double* partial, unsigned* counter, double* mean, cudaStream_t s);
void launch_lexmax_seg(int nseg, const int64_t* off, int per, int V, const double* u,
                       const double* mean, int max_mode, double* partial, unsigned* counter,
                       double* norms, cudaStream_t s, bool pdl = false);
void launch_eps_f32(const EpsArgs& a, cudaStream_t s);

struct RevArgs {
  int64_t n;
  EllView ell;
  const double* w[3];
  const double* wl;
  const float* w32[3];
  const float* wl32;
  int V;
  int rv;             // gather s = eps*D u over the reverse adjacency
  int lap;            // gather q = lap u over the reverse adjacency (Tominec)
  double hv_gamma;
  float hg32;           // (float) hv_gamma (FP32 kernels; set by the launchers)
  const double* s;    // n x 2V
  const double* q;    // n x V
  const float* s32;
  const float* q32;
  const double* du_p; // n x V
  const float* du_p32;
  const double* hvf;  // n x V Flyer term added after RV (or null)
  int final_epilogue; // 0: write du_p_out (intermediate), 1: BC2 + epilogue
  double* du_p_out;
  float* du_p_out32;
  Epilogue ep;
  const float2* wdw[3];  // double-word FP64 form: weights on the reverse layout
  const float2* wldw;
  const float2* sdw;     // n x 2V pairs (eps * t)
  const float2* qdw;     // n x V pairs
};
void launch_rev_f64(const RevArgs& a, cudaStream_t s);
void launch_rev_dw(const RevArgs& a, int variant, cudaStream_t s);
void launch_rev_f32(const RevArgs& a, cudaStream_t s);
// Bulk-copy-staged FP32 gathers (Euler); return false when the case is not covered.
// chunk: slots staged per bulk copy (4 or 8).
// The staged (halo) FP32 gathers: false when the layout has no halos or V != 4.
bool launch_fwd_f32_halo(const FwdArgs& a, cudaStream_t s);
bool launch_rev_f32_halo(const RevArgs& a, cudaStream_t s);
bool launch_fwd_f32_tma(const FwdArgs& a, int chunk, int* err, cudaStream_t s);
bool launch_rev_f32_tma(const RevArgs& a, int chunk, int* err, cudaStream_t s);
// One warp's bounded wait on an mbarrier that nothing completes (error-path self-test).
void launch_wait_selftest(int* err, unsigned polls, cudaStream_t s);

// Adjoint of rhs! (reverse mode) and the SSP-RK3 adjoint stage combinations.
// With r = (d rhs!/du)^T lam at state u and Pi the strong-BC projection:
//   kAdjPlain:  out = r
//   kAdjStage3: out = Pi(2/3 lam) + 2dt/3 r,  acc = lam / 3
//   kAdjStage2: out = Pi(lam / 4) + dt/4 r,   acc += 3/4 lam
//   kAdjStage1: out = Pi(acc + lam) + dt r
enum AdjKind : int { kAdjPlain = 0, kAdjStage1 = 1, kAdjStage2 = 2, kAdjStage3 = 3 };
struct AdjArgs {
  int64_t n;
  EllView ell;         // reverse adjacency (column j of D as row j)
  const double* w[2];  // D_x, D_y on the reverse layout
  const double* wh;    // lap (Tominec) or H (Flyer) on the reverse layout, or null
  int hv;              // 0 none, 1 Tominec (gathers q = lap M2 lam), 2 Flyer (gathers M2 lam)
  double hv_gamma;
  const double* lam;   // n x V cotangent
  const double* q;     // n x V lap M2 lam (Tominec)
  const double* u;     // n x V state the product linearises about
  int eq, V;
  double gamma, ax, ay;
  BcDev bc;
  int has_bc;
  int kind;
  double dt;
  double* acc;         // n x V stage accumulator (stage kinds)
  double* out;         // n x V
  const double* xadd;  // n x V added to the transpose product before the stage
                       // combination (the viscosity source's part), or null
  // double-word gathers (2D Euler, FP64 form): weights on the reverse layout as pairs
  const float2* wdw[2];
  const float2* whdw;
  const float2* lamdw;  // M2 lam as pairs (set by launch_adj_dw)
};
void launch_adj_f64(const AdjArgs& a, cudaStream_t s);
// The same product with the sums in double-word arithmetic; lam_pairs: n x 4 pair scratch;
// staged: each row group's neighbour pairs staged in shared memory (when halos exist).
void launch_adj_dw(const AdjArgs& a, float2* lam_pairs, bool staged, cudaStream_t s);
// q_i = sum_j lap[i,j] (M2 lam)_j over the forward layout (Tominec adjoint).
void launch_lap_masked(int64_t n, EllView fwd, const double* wl, const double* lam, int V,
                       BcDev bc, int has_bc, double* q, cudaStream_t s);
// lam = Pi lam at the listed boundary nodes (Dirichlet zero, slip-wall projection).
void launch_bc_project(int64_t nb, const int32_t* bnode, int V, BcDev bc, double* lam,
                       cudaStream_t s);

// One Zhang-Shu positivity-limiter pass (variable 0 density, 1 pressure) on the Euler
// state u (n x 4 AoS, FP32 shadow u32 optional) over the stencils of the forward layout;
// loc is n x 4 scratch.
void launch_zs_limiter(int64_t n, EllView ell, int variable, double threshold, double gamma,
                       double* u, float* u32, double* loc, cudaStream_t s);

// IGR source (mft_igr.cu): conjugate-gradient scalars kept in device memory.
struct IgrScalars {
  double res, prev, tol, alpha_cg, beta;
  int iter, done;
};
struct IgrArgs {
  int64_t n;
  EllView ell;          // forward layout
  const double* wx;     // D_x, D_y on the forward layout
  const double* wy;
  double alpha;
  int maxiter;
  double* prim;         // n x 3 (rho, v1, v2)
  double* rinv;         // n
  double* x;            // n: sigma
  double* r;            // n
  double* u0;           // n: CG directions, alternating
  double* u1;
  double* c;            // n
  double* t;            // n x 2
  double* add;          // n x 2 output: -(Dx sigma), -(Dy sigma)
  double* partial;      // one double per block
  unsigned* counter;
  IgrScalars* sc;
};
// Full IGR pipeline on the Euler state u (n x 4 AoS): prim, right-hand side, CG, flux.
void launch_igr(const IgrArgs& a, const double* u, cudaStream_t s);

// Sets *flag to 1 when a and b differ in any of `count` doubles (bitwise).
void launch_differs(const double* a, const double* b, int64_t count, int* flag, cudaStream_t s);

// approx_du = sum_i w_i * hist_i (history ring, FP64) and push of the newest state.
struct HistW {
  double w[8];
};
// approx_du = sum_k w_k hist[k]; hist[0] (the new state) is also copied to ring_dst.
// fused: multiply-adds (FP32-apply form) instead of separately rounded products and sums.
void launch_history(int64_t count, int m, const HistW& w, const double* const* hist,
                    double* ring_dst, double* approx_du, bool fused, cudaStream_t s);

// Per-step parameters of a captured SSP-RK3 step, read on the device through a step
// counter so that one graph serves every step of a batch.
struct StepParams {
  double w[8];       // time-derivative weights of the history push after the step
  int m;             // number of history points used (0: approx_du = 0)
  int si_eps;        // success_iter seen by the viscosity kernels during the step
  int head;          // ring slot that receives the new state
  int pad;
};
// Graph-mode history push: ring[tab.head] = u_new; approx_du = sum_k w_k ring_k.
void launch_history_dev(int64_t count, const double* u_new, const double* const* ring,
                        int slots, const StepParams* tab, const int* ctr, double* approx_du,
                        bool fused, cudaStream_t s);
void launch_step_advance(int* ctr, cudaStream_t s);

}  // namespace mft
