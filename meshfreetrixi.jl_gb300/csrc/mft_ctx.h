// Context object behind the opaque mft_ctx handle.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <string>
#include <vector>

#include "mft_internal.cuh"

// Operator value slots: 0..2 gradient components, 3 lap (sum of pure 2nd
// derivatives), 4 ready hyperviscosity operator.
constexpr int kSlotLap = 3;
constexpr int kSlotHv = 4;
constexpr int kSlots = 5;
// Threads per block of the node-parallel kernels (sizes the per-block reduction partials).
constexpr int kBlockHost = 128;
// Blocks per ensemble member in the segmented reductions.
constexpr int kSegBlocks = 8;

struct mft_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;

  // geometry
  int dim = 0;
  int64_t n = 0;
  std::vector<double> xyz;
  bool periodic = false;
  double period[3] = {0, 0, 0};
  mft::DBuf<double> d_xyz;

  // stencils in caller order (centre first)
  std::vector<int64_t> st_rp;
  std::vector<int32_t> st_ci;
  bool have_stencils = false;

  // operator pattern: CSR rows with ascending columns, its CSC view, and maps
  bool have_pattern = false;
  std::vector<int64_t> rp;
  std::vector<int32_t> ci;
  std::vector<int64_t> cp;
  std::vector<int32_t> ri;
  std::vector<int64_t> csc2csr;  // CSC entry -> CSR entry
  std::vector<int64_t> st2csr;   // stencil entry -> CSR entry (when built from stencils)
  std::vector<double> val[kSlots];
  bool have_val[kSlots] = {false, false, false, false, false};
  bool dev_dirty = true;
  mft::EllBuf fwd, rev;
  mft::DBuf<int64_t> fwd_pos, rev_pos;  // CSR entry -> ELL element
  mft::DBuf<double> fw[kSlots], rw[kSlots];
  mft::DBuf<float> fw32[kSlots], rw32[kSlots];
  mft::DBuf<float2> fwdw[kSlots], rwdw[kSlots];  // double-word pairs (FP64 form, Euler)

  // physics
  int eq = -1;
  int nvars = 0;
  double gamma = 1.4;
  double adv[3] = {0, 0, 0};

  // boundary conditions
  int n_bc = 0;
  std::vector<int> bc_kind;
  std::vector<int64_t> bc_ptr;
  std::vector<int32_t> bc_idx;
  std::vector<double> bc_normal;
  std::vector<double> dir_values;
  int64_t nb = 0;  // boundary nodes with an active BC
  mft::DBuf<int8_t> d_tag;
  mft::DBuf<int32_t> d_slot;
  mft::DBuf<double> d_normal;
  mft::DBuf<double> d_dvals;
  mft::DBuf<int32_t> d_bnode;
  bool bc_dirty = true;
  mft_dirichlet_fn dir_fn = nullptr;
  void* dir_user = nullptr;
  std::vector<double> dir_scratch;

  // sources
  std::vector<int> src_kind;
  std::vector<double> src_par;
  int precision = MFT_PREC_FP64;
  int gather_mode = MFT_GATHER_AUTO;
  int fp64_arith = MFT_ARITH_AUTO;
  int layout_order = 1;  // 1: operator layout rows in Morton order of the nodes
  int halo_rows_opt = 0;  // rows per staged group: 0 automatic, else 128 or 256
  int entry_order = 1;    // staged rows: 1 bank-spreading entry order, 0 structure order
  int fuse_flux = 1;      // staged double-word forward gathers may form the flux records
  int last_flux_fused = 0;  // the last evaluation did (and skipped the flux kernel)
  int tuned_fwd[16] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};
  int tuned_rev[4] = {-1, -1, -1, -1};
  int last_fwd_choice = -1, last_rev_choice = -1;
  int tuned_fwd_dw[16] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};
  int tuned_rev_dw[4] = {-1, -1, -1, -1};
  int dw_variant = -1;   // double-word gather variant: -1 autotuned, else forced

  // work buffers (AoS n x V unless noted)
  mft::DBuf<double> U[4];  // u_n, stage 1, stage 2, stage 3
  mft::DBuf<float> U32[4];
  mft::DBuf<double> F, du_p, du_p2, t, q, hvf, eps, approx_du, soa, soa2, work_u, work_du;
  mft::DBuf<float> du_p32, du_p2_32, t32, q32, work_u32, work_du32;
  mft::DBuf<float2> Fdw, udw, tdw, qdw;  // double-word FP64 form: per-node pairs
  mft::DBuf<double> red_partial, mean, norms;
  mft::DBuf<unsigned> red_counter;
  mft::DBuf<int> flag;
  mft::DBuf<int> kerr;  // device error word of kernels with bounded waits
  int red_blocks = 0;

  // time integration state
  double t_state = 0.0;
  bool state_valid = false;
  bool fsal_valid = false;
  double fsal_dt = 0.0;
  // step times are t_origin + k dt, k counted from the origin while dt stays the same
  bool origin_valid = false;
  double t_origin = 0.0, origin_dt = 0.0;
  int64_t origin_steps = 0;

  // history ring (HistoryCallback)
  int hist_order = -1;
  std::vector<double> hist_t;
  mft::DBuf<double> hist[8];
  int hist_head = 0;
  int success_iter = 0;
  mft::DBuf<double> hist_w;

  // ensemble members (segments)
  int nseg = 0;
  std::vector<int64_t> seg_off;
  mft::DBuf<int64_t> d_seg_off;
  mft::DBuf<int> d_seg_id;
  mft::DBuf<double> d_seg_h, seg_partial, seg_mean, seg_norms;
  mft::DBuf<unsigned> seg_counter;

  // IGR source work buffers and CG scalars
  mft::DBuf<double> igr_prim, igr_rinv, igr_x, igr_r, igr_u0, igr_u1, igr_c, igr_t, igr_add,
      igr_partial;
  mft::DBuf<unsigned> igr_counter;
  mft::DBuf<mft::IgrScalars> igr_sc;

  // Zhang-Shu positivity limiter after every SSP-RK3 stage (variables in order)
  int lim_n = 0;
  int lim_var[4] = {0, 0, 0, 0};
  double lim_thr[4] = {0, 0, 0, 0};
  mft::DBuf<double> lim_buf;

  // adjoint: recorded trajectory (checkpoints, or every stage state) and cotangents
  mft::DBuf<double> adj_lam[3], adj_acc, adj_q, adj_store, adj_ckpt;
  mft::DBuf<float2> adj_lamdw;  // M2 lam as double-word pairs (double-word adjoint gather)
  // viscosity-source adjoint: forward state and du, the added transpose product, the
  // norm cotangents and the ode_maximum rows
  mft::DBuf<double> adj_ubc, adj_du, adj_xadd, adj_nbar;
  mft::DBuf<int> adj_jstar;
  bool adj_valid = false;
  double adj_t0 = 0.0, adj_dt = 0.0;
  int adj_nsteps = 0, adj_every = 0;

  // one SSP-RK3 step as a CUDA graph (u_n in U0 / in U3) and its step table
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  const double* graph_un[2] = {nullptr, nullptr};
  double graph_dt = 0.0;
  bool graph_valid = false;
  bool capturing = false;
  mft::DBuf<mft::StepParams> d_tab;
  mft::StepParams* h_tab = nullptr;  // pinned staging of the step table
  size_t h_tab_n = 0;
  cudaEvent_t ev_tab = nullptr;      // the last table copy
  int* h_kerr = nullptr;             // pinned copy of the device error word
  mft::DBuf<int> d_ctr;

  // side stream for the residual-viscosity reductions (overlap with the gathers)
  cudaStream_t stream2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;

  // timing
  bool prof_on = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_pending;
  double prof_ms[MFT_K_COUNT] = {};
  int64_t prof_n[MFT_K_COUNT] = {};
  cudaEvent_t region_ev[2] = {nullptr, nullptr};
};

namespace mft {
// NVTX range on the host thread, named after the reference's timer keys ("rhs!",
// "boundary flux", "calc fluxes", "source terms": src/solvers/pointcloudsolver/
// rbfsolver.jl:397-428), so that a profiler shows the same breakdown.  NVTX is
// header-only; without a profiler attached a range costs a few nanoseconds.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Event pair around one kernel launch when profiling is on.
struct ProfScope {
  mft_ctx* c;
  int kind;
  cudaEvent_t e1 = nullptr;
  ProfScope(mft_ctx* ctx, int k);
  ~ProfScope();
};
}  // namespace mft

namespace mft {
// The FP64 form's gathers run in double-word FP32 arithmetic (2D Euler; the
// MFT_OPT_FP64_ARITH option); otherwise in FP64 fused multiply-adds.
inline bool use_dw(const mft_ctx* c) {
  return c->precision == MFT_PREC_FP64 && c->fp64_arith != MFT_ARITH_DFMA &&
         c->eq == MFT_EQ_EULER2D && c->nvars == 4;
}
// The 3D Euler gather in double-word arithmetic (FP64 form, MFT_OPT_FP64_ARITH not DFMA).
inline bool use_dw3(const mft_ctx* c) {
  return c->precision == MFT_PREC_FP64 && c->fp64_arith != MFT_ARITH_DFMA &&
         c->eq == MFT_EQ_EULER3D && c->nvars == 5;
}
// Builds (if needed) the device ELL layouts and operator values.
void ensure_device_ops(mft_ctx* c);
// One rhs! evaluation on the AoS state `us` (device), with the given epilogue.
void eval_rhs(mft_ctx* c, double* us, float* us32, double t, const Epilogue& ep_in);
// Work-buffer sizing for the current problem.
void ensure_work(mft_ctx* c);
// Pattern from stencils (caller order, centre first).
void pattern_from_stencils(mft_ctx* c);
// Reverse CSC view + ELL/maps rebuild flags after the CSR pattern is set.
void finish_pattern(mft_ctx* c);
// KNN and weights (mft_knn.cu, mft_weights.cu)
void knn_device(mft_ctx* c, int k, std::vector<int32_t>& idx, std::vector<double>* dist,
                double* dx_min, double* dx_avg);
void weights_device(mft_ctx* c, int rbf_pow, int polydeg, int deriv_order,
                    std::vector<double>& w_out, double* max_resid);
void weights_batch(mft_ctx* c, int ngroups, const mft_weight_group* groups, double* max_resid);
// The viscosity source's part of the adjoint of rhs! (mft_adjoint_visc.cu).
void visc_adjoint_terms(mft_ctx* c, const double* u_bc, const double* lam, double* out);
}  // namespace mft
