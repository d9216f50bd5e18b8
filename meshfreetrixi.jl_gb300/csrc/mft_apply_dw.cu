// FP64 form of the 2D Euler rhs! gathers in double-word FP32 arithmetic (mft_dw.cuh).
//
// Same passes, layouts and epilogues as the FP64 kernels (mft_apply.cu); what changes is
// how the sums over a stencil are formed.  Operator weights, the per-node fluxes and the
// neighbour states are read as double-word pairs (h, l) -- 8 bytes per value, the
// footprint of an FP64 value -- and the products and sums run on the FP32 pipe with
// error-free transformations; per-node values (the stage epilogue, the viscosity) stay
// in FP64.  Accumulation order per row is the layout's entry order (ascending columns, or
// in the rows of staged groups the bank-spreading order of build_ell), shared by every
// variant.
#include <cuda_runtime.h>
#include <math.h>

#include <mutex>
#include <set>
#include <utility>

#include "mft_device.cuh"
#include "mft_dw.cuh"
#include "mft_eps.cuh"
#include "mft_halo.cuh"
#include "mft_internal.cuh"
#include "mft_tma.cuh"

namespace mft {

namespace {

using namespace dev;

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

static __device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }

// The streamed arrays of a warp's slice (column indices and up to three weight arrays,
// read once per launch) requested into L2 a chunk of kPfSlots slots at a time by one
// lane, ahead of the slots the warp gathers (the weights otherwise arrive from DRAM on
// each slot's critical path).  The range stays inside the slice.
constexpr int kPfSlots = 8;
struct SliceArrays {
  const void* arr[4];
  int esize[4];
  int narr;
};
static __device__ __forceinline__ void prefetch_chunk(const SliceArrays& sa, int64_t s_lo,
                                                      int64_t s_hi, int chunk) {
  const int64_t e0 = s_lo + (int64_t)chunk * kPfSlots * 32;
  if (e0 >= s_hi) return;
  const int64_t ne = min((int64_t)kPfSlots * 32, s_hi - e0);
#pragma unroll
  for (int k = 0; k < 4; ++k)
    if (k < sa.narr)
      tma::bulk_prefetch_l2(static_cast<const char*>(sa.arr[k]) + e0 * sa.esize[k],
                            (uint32_t)(ne * sa.esize[k]));
}
static __device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }


// Per node: the state as double-word pairs and the Euler flux pair evaluated from them in
// double-word arithmetic (the textbook flux, one reciprocal for both velocities; each
// operation is accurate to about 2 u^2 of its operands, u = 2^-24), as the records the
// forward gather reads: F = (Fx_0..3, Fy_0..3) in four float4 (Fx_0 = m1, Fy_0 = m2),
// U = (u_0..3) in two, 8 floats per 4 values.  gm1 = gamma - 1 as a pair.  The only FP64
// operations are the four splits of the state.  Shared by the flux kernel and the staged
// gathers that form the records while staging, so both give the same bits.
static __device__ __forceinline__ void euler_records(double2 a, double2 b, float2 gm1,
                                                     float4* F, float4* U) {
  const float2 rho = dw::split(a.x), m1 = dw::split(a.y), m2 = dw::split(b.x);
  const float2 en = dw::split(b.y);
  const float2 r = dw::recip(rho);
  const float2 v1 = dw::mul(m1, r), v2 = dw::mul(m2, r);
  const float2 a1 = dw::mul(m1, v1), a2 = dw::mul(m2, v2);
  const float2 p = dw::mul(gm1, dw::add(en, dw::neg(dw::scale2(dw::add(a1, a2), 0.5f))));
  const float2 ep = dw::add(en, p);
  const float2 fx1 = dw::add(a1, p), fx2 = dw::mul(m1, v2), fx3 = dw::mul(ep, v1);
  const float2 fy1 = dw::mul(m2, v1), fy2 = dw::add(a2, p), fy3 = dw::mul(ep, v2);
  F[0] = make_float4(m1.x, m1.y, fx1.x, fx1.y);
  F[1] = make_float4(fx2.x, fx2.y, fx3.x, fx3.y);
  F[2] = make_float4(m2.x, m2.y, fy1.x, fy1.y);
  F[3] = make_float4(fy2.x, fy2.y, fy3.x, fy3.y);
  U[0] = make_float4(rho.x, rho.y, m1.x, m1.y);
  U[1] = make_float4(m2.x, m2.y, en.x, en.y);
}

__global__ void k_prep_euler_dw(int64_t n, float2 gm1, const double* __restrict__ u,
                                float4* __restrict__ F, float4* __restrict__ U) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2* ui = reinterpret_cast<const double2*>(u) + i * 2;
  float4 f[4], uu[2];
  euler_records(ui[0], ui[1], gm1, f, uu);
  float4* Fi = F + i * 4;
#pragma unroll
  for (int k = 0; k < 4; ++k) Fi[k] = f[k];
  U[i * 2] = uu[0];
  U[i * 2 + 1] = uu[1];
}

// Staging with the records formed on the fly: each thread reads the FP64 states of list
// entries q and q + blockDim.x (both loads in flight together), forms their records
// (euler_records) and writes the NCH chunks of each into shared memory at k * stride + q,
// the layout stage_halo's copies give.  Returns false for a group without a list.
template <int NCH>
static __device__ __forceinline__ bool stage_halo_records(const EllView& ell, float4* sm,
                                                          const double* __restrict__ u,
                                                          float2 gm1) {
  const int h0 = __ldg(ell.halo_off + blockIdx.x);
  const int nh = __ldg(ell.halo_off + blockIdx.x + 1) - h0;
  if (nh <= 0) return false;  // block-uniform
  const int hs = ell.halo_stride;
  const double2* __restrict__ u2 = reinterpret_cast<const double2*>(u);
  for (int q0 = threadIdx.x; q0 < nh; q0 += 2 * blockDim.x) {
    const int q1 = q0 + blockDim.x;
    const int64_t c0 = __ldg(ell.halo_col + h0 + q0);
    const int64_t c1 = q1 < nh ? (int64_t)__ldg(ell.halo_col + h0 + q1) : c0;
    const double2 a0 = __ldg(u2 + c0 * 2), b0 = __ldg(u2 + c0 * 2 + 1);
    const double2 a1 = __ldg(u2 + c1 * 2), b1 = __ldg(u2 + c1 * 2 + 1);
    float4 rec[6];
    euler_records(a0, b0, gm1, rec, rec + 4);
#pragma unroll
    for (int k = 0; k < NCH; ++k) sm[k * hs + q0] = rec[k];
    if (q1 < nh) {
      euler_records(a1, b1, gm1, rec, rec + 4);
#pragma unroll
      for (int k = 0; k < NCH; ++k) sm[k * hs + q1] = rec[k];
    }
  }
  __syncthreads();
  return true;
}

// One stencil entry of the forward gather: weights and the neighbour's flux and state
// records, requested together.
struct FwdEntry {
  float2 wx, wy, wl;
  F8 fa, fb, uu;
};

template <bool WT, bool WQ, int FLY>
static __device__ __forceinline__ FwdEntry fwd_load(const FwdArgs& a, const float* F,
                                                    const float* U, int64_t p, int64_t c) {
  FwdEntry e;
  e.wx = __ldg(a.wdw[0] + p);
  e.wy = __ldg(a.wdw[1] + p);
  e.fa = ldg_f8(F + c * 16);
  e.fb = ldg_f8(F + c * 16 + 8);
  if (WT || WQ || FLY) e.uu = ldg_f8(U + c * 8);
  if (WQ || FLY) e.wl = __ldg(a.wldw + p);
  return e;
}

// The same entry with the neighbour's records read from the staged halo (lc: position
// of the neighbour in the group's list).
template <bool WT, bool WQ, int FLY, bool HINT = false>
static __device__ __forceinline__ FwdEntry fwd_load_halo(const FwdArgs& a, const float4* sm,
                                                         int hs, int64_t p, int lc,
                                                         uint64_t pol = 0) {
  FwdEntry e;
  e.wx = HINT ? ldg_hint(a.wdw[0] + p, pol) : __ldg(a.wdw[0] + p);
  e.wy = HINT ? ldg_hint(a.wdw[1] + p, pol) : __ldg(a.wdw[1] + p);
  e.fa.lo = sm[lc];
  e.fa.hi = sm[hs + lc];
  e.fb.lo = sm[2 * hs + lc];
  e.fb.hi = sm[3 * hs + lc];
  if (WT || WQ || FLY) {
    e.uu.lo = sm[4 * hs + lc];
    e.uu.hi = sm[5 * hs + lc];
  }
  if (WQ || FLY) e.wl = HINT ? ldg_hint(a.wldw + p, pol) : __ldg(a.wldw + p);
  return e;
}

template <bool WT, bool WQ, int FLY>
static __device__ __forceinline__ void fwd_accum(const FwdEntry& e, dw::Acc* f, dw::Acc* tx,
                                                 dw::Acc* ty, dw::Acc* q) {
  const float2 Fx[4] = {lo2(e.fa.lo), hi2(e.fa.lo), lo2(e.fa.hi), hi2(e.fa.hi)};
  const float2 Fy[4] = {lo2(e.fb.lo), hi2(e.fb.lo), lo2(e.fb.hi), hi2(e.fb.hi)};
#pragma unroll
  for (int v = WT ? 1 : 0; v < 4; ++v) {
    // Fx[0] = m1, Fy[0] = m2: with t formed, the rho row is tx1 + ty2
    dw::fma_acc(f[v], e.wx, Fx[v]);
    dw::fma_acc(f[v], e.wy, Fy[v]);
  }
  if (WT || WQ || FLY) {
    const float2 uc[4] = {lo2(e.uu.lo), hi2(e.uu.lo), lo2(e.uu.hi), hi2(e.uu.hi)};
    if (WT) {
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        dw::fma_acc(tx[v], e.wx, uc[v]);
        dw::fma_acc(ty[v], e.wy, uc[v]);
      }
    }
    if (WQ || FLY) {
#pragma unroll
      for (int v = 0; v < 4; ++v) dw::fma_acc(q[v], e.wl, uc[v]);
    }
  }
}

// Forward gather (Euler), one node per thread over the sliced ELL: the flux divergence
// -sum_j (Dx F_x + Dy F_y), t = (Dx u, Dy u) (WT), q = lap u (WQ) or the Flyer term
// H u (FLY), as in k_fwd_euler_f64.  Per stencil entry: a 64-byte flux record and a
// 32-byte state record (both one or two 256-bit loads), 8-byte weights.
// PIPE = 0: one entry per loop iteration; PIPE = 2: two (the compiler overlaps their
// loads); PIPE = 1: software pipeline -- the column index is loaded two entries ahead and
// the weights and records one entry ahead, so that the gathers of entry j + 1 are in flight while entry j is
// accumulated (the gathers are latency-bound: most samples stall on their results).
// MINB: minimum resident blocks per SM requested from the compiler (register cap).
// The variants form the same sums in the same order; the autotuner picks one.
// HALO: blocks of one row group (ell.halo_rows rows) first stage the group's neighbour
// records in shared memory and read them from there (groups without a list gather
// directly); PIPE 0 or 2 then sets the loop's unrolling.  HINT: the staged loop reads the
// streamed positions and weights with an L2 evict-first policy and the epilogue writes t,
// q and the partial du with evict-last, which the transpose gather reads next.  FUSE: the
// staged records are formed from the FP64 state while staging (stage_halo_records), so
// the flux kernel's pairs are not read; launched only when every group is staged (a group
// without a list sets MFT_ERR_STATE in *a.err and its rows are not written).
template <bool WT, bool WQ, int FLY, int PIPE, int MINB, bool PREF, bool HALO, bool HINT = false,
          bool FUSE = false>
__global__ void __launch_bounds__(HALO ? kHaloRows : kBlock, MINB) k_fwd_euler_dw(FwdArgs a) {
  const int64_t r = blockIdx.x * (int64_t)(HALO ? (int)blockDim.x : kBlock) + threadIdx.x;
  const float* __restrict__ F = reinterpret_cast<const float*>(a.Fdw);
  const float* __restrict__ U = reinterpret_cast<const float*>(a.udw);
  extern __shared__ float4 hsm[];
  bool staged = false;
  constexpr int kNch = (WT || WQ || FLY) ? 6 : 4;
  if (HALO && FUSE) {
    staged = stage_halo_records<kNch>(a.ell, hsm, a.ustate, a.gm1dw);
    if (!staged) {
      if (threadIdx.x == 0) atomicExch(a.err, MFT_ERR_STATE);
      return;
    }
  } else if (HALO) {
    const float4* F4 = reinterpret_cast<const float4*>(a.Fdw);
    const float4* U4 = reinterpret_cast<const float4*>(a.udw);
    staged = stage_halo<kNch>(
        a.ell, hsm, [&](int k, int64_t c) { return k < 4 ? F4 + c * 4 + k : U4 + c * 2 + (k - 4); });
  }
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  const int32_t* __restrict__ col = a.ell.col;
  dw::Acc f[4], tx[4], ty[4], q[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    f[v] = dw::zero(); tx[v] = dw::zero(); ty[v] = dw::zero(); q[v] = dw::zero();
  }
  const uint16_t* __restrict__ lcol = a.ell.lcol;
  const int hs = a.ell.halo_stride;
  if (HALO && staged) {
    SliceArrays sa{};
    int64_t s_lo = 0, s_hi = 0;
    const bool pf_lane = PREF && (threadIdx.x & 31) == 0;
    if (pf_lane) {
      sa.arr[0] = lcol; sa.esize[0] = 2;
      sa.arr[1] = a.wdw[0]; sa.esize[1] = 8;
      sa.arr[2] = a.wdw[1]; sa.esize[2] = 8;
      sa.arr[3] = a.wldw; sa.esize[3] = 8;
      sa.narr = (WQ || FLY) ? 4 : 3;
      s_lo = a.ell.slice_off[r >> 5];
      s_hi = a.ell.slice_off[(r >> 5) + 1];
      prefetch_chunk(sa, s_lo, s_hi, 0);
      prefetch_chunk(sa, s_lo, s_hi, 1);
    }
    constexpr int UNR = PIPE < 1 ? 1 : PIPE;
    const uint64_t pol = HINT ? l2_evict_first() : 0;
#pragma unroll UNR
    for (int j = 0; j < len; ++j) {
      if (pf_lane && (j % kPfSlots) == 0) prefetch_chunk(sa, s_lo, s_hi, j / kPfSlots + 2);
      const int64_t p = base + ((int64_t)j << 5);
      const int lc = HINT ? ldg_hint(lcol + p, pol) : __ldg(lcol + p);
      fwd_accum<WT, WQ, FLY>(fwd_load_halo<WT, WQ, FLY, HINT>(a, hsm, hs, p, lc, pol), f, tx, ty, q);
    }
  } else if (PIPE == 0) {
#pragma unroll 1
    for (int j = 0; j < len; ++j) {
      const int64_t p = base + ((int64_t)j << 5);
      const int64_t c = __ldg(col + p);
      fwd_accum<WT, WQ, FLY>(fwd_load<WT, WQ, FLY>(a, F, U, p, c), f, tx, ty, q);
    }
  } else if (PIPE == 2 || (HALO && PIPE > 2)) {
    SliceArrays sa{};
    int64_t s_lo = 0, s_hi = 0;
    const bool pf_lane = PREF && (threadIdx.x & 31) == 0;
    if (pf_lane) {
      sa.arr[0] = col; sa.esize[0] = 4;
      sa.arr[1] = a.wdw[0]; sa.esize[1] = 8;
      sa.arr[2] = a.wdw[1]; sa.esize[2] = 8;
      sa.arr[3] = a.wldw; sa.esize[3] = 8;
      sa.narr = (WQ || FLY) ? 4 : 3;
      s_lo = a.ell.slice_off[r >> 5];
      s_hi = a.ell.slice_off[(r >> 5) + 1];
      prefetch_chunk(sa, s_lo, s_hi, 0);
      prefetch_chunk(sa, s_lo, s_hi, 1);
    }
#pragma unroll 2
    for (int j = 0; j < len; ++j) {
      if (pf_lane && (j % kPfSlots) == 0) prefetch_chunk(sa, s_lo, s_hi, j / kPfSlots + 2);
      const int64_t p = base + ((int64_t)j << 5);
      const int64_t c = __ldg(col + p);
      fwd_accum<WT, WQ, FLY>(fwd_load<WT, WQ, FLY>(a, F, U, p, c), f, tx, ty, q);
    }
  } else if (len > 0) {
    int64_t c_next = len > 1 ? (int64_t)__ldg(col + base + 32) : 0;
    FwdEntry cur = fwd_load<WT, WQ, FLY>(a, F, U, base, __ldg(col + base));
    for (int j = 0; j < len; ++j) {
      const int64_t p1 = base + ((int64_t)(j + 1) << 5);
      const int64_t c2 = j + 2 < len ? (int64_t)__ldg(col + p1 + 32) : 0;
      FwdEntry nxt;
      if (j + 1 < len) nxt = fwd_load<WT, WQ, FLY>(a, F, U, p1, c_next);
      fwd_accum<WT, WQ, FLY>(cur, f, tx, ty, q);
      cur = nxt;
      c_next = c2;
    }
  }
  double du[4];
  if (WT) du[0] = -dadd(dw::to_double(tx[1]), dw::to_double(ty[2]));
  else du[0] = -dw::to_double(f[0]);
#pragma unroll
  for (int v = 1; v < 4; ++v) du[v] = -dw::to_double(f[v]);
  double qv[4] = {0, 0, 0, 0};
  if (FLY) {
#pragma unroll
    for (int v = 0; v < 4; ++v) qv[v] = dw::to_double(q[v]);
  }
  if (FLY == 1) {
#pragma unroll
    for (int v = 0; v < 4; ++v) du[v] = fma(-a.hv_gamma, qv[v], du[v]);
  }
  if (WT) {
    float4* t4 = reinterpret_cast<float4*>(a.tdw) + i * 4;
    float2 x[4], y[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) { x[v] = dw::to_pair(tx[v]); y[v] = dw::to_pair(ty[v]); }
    if (a.fuse_eps) {
      // the viscosity of this node (FP64, as k_eps forms it from the partial du held
      // here) and s = eps * t written in place of t; this FP64 work overlaps the FP32
      // gathers of other warps.  The norms come from the reductions this grid may have
      // been launched beside (launch_k with a.pdl): wait for them here, not earlier.
      pdl_wait();
      const double eps = visc::eps_value<4>(a.ea, i, du);
      if (a.ea.eps) a.ea.eps[i] = eps;
      const float2 e2 = dw::split(eps);
#pragma unroll
      for (int v = 0; v < 4; ++v) { x[v] = dw::mul(e2, x[v]); y[v] = dw::mul(e2, y[v]); }
    }
    const float4 o[4] = {make_float4(x[0].x, x[0].y, x[1].x, x[1].y),
                         make_float4(x[2].x, x[2].y, x[3].x, x[3].y),
                         make_float4(y[0].x, y[0].y, y[1].x, y[1].y),
                         make_float4(y[2].x, y[2].y, y[3].x, y[3].y)};
    if (HINT) {
      const uint64_t keep = l2_evict_last();
#pragma unroll
      for (int k = 0; k < 4; ++k) st_hint(t4 + k, o[k], keep);
    } else {
#pragma unroll
      for (int k = 0; k < 4; ++k) t4[k] = o[k];
    }
  }
  if (WQ) {
    float4* q4 = reinterpret_cast<float4*>(a.qdw) + i * 2;
    float2 x[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) x[v] = dw::to_pair(q[v]);
    const float4 o0 = make_float4(x[0].x, x[0].y, x[1].x, x[1].y);
    const float4 o1 = make_float4(x[2].x, x[2].y, x[3].x, x[3].y);
    if (HINT) {
      const uint64_t keep = l2_evict_last();
      st_hint(q4, o0, keep);
      st_hint(q4 + 1, o1, keep);
    } else {
      q4[0] = o0;
      q4[1] = o1;
    }
  }
  if (FLY == 2) {
    double2* h2 = reinterpret_cast<double2*>(a.hvf) + i * 2;
    h2[0] = make_double2(-a.hv_gamma * qv[0], -a.hv_gamma * qv[1]);
    h2[1] = make_double2(-a.hv_gamma * qv[2], -a.hv_gamma * qv[3]);
  }
  if (a.final_epilogue) {
    finish_node<4>(a.ep, i, du);
  } else {
    double2* d2 = reinterpret_cast<double2*>(a.du_p) + i * 2;
    if (HINT) {
      const uint64_t keep = l2_evict_last();
      st_hint(d2, make_double2(du[0], du[1]), keep);
      st_hint(d2 + 1, make_double2(du[2], du[3]), keep);
    } else {
      d2[0] = make_double2(du[0], du[1]);
      d2[1] = make_double2(du[2], du[3]);
    }
  }
}

// One entry of the transpose gather: weights and the neighbour's s = eps t and q records.
struct RevEntry {
  float2 wx, wy, wl;
  F8 xa, ya, qq;
};

template <bool RV, bool LAP>
static __device__ __forceinline__ RevEntry rev_load(const RevArgs& a, const float* S,
                                                    const float* Q, int64_t p, int64_t c) {
  RevEntry e;
  if (RV) {
    e.wx = __ldg(a.wdw[0] + p);
    e.wy = __ldg(a.wdw[1] + p);
    e.xa = ldg_f8(S + c * 16);
    e.ya = ldg_f8(S + c * 16 + 8);
  }
  if (LAP) {
    e.wl = __ldg(a.wldw + p);
    e.qq = ldg_f8(Q + c * 8);
  }
  return e;
}

template <bool RV, bool LAP, bool HINT = false>
static __device__ __forceinline__ RevEntry rev_load_halo(const RevArgs& a, const float4* sm,
                                                         int hs, int64_t p, int lc,
                                                         uint64_t pol = 0) {
  RevEntry e;
  constexpr int kq = RV ? 4 : 0;  // first chunk of the q record
  if (RV) {
    e.wx = HINT ? ldg_hint(a.wdw[0] + p, pol) : __ldg(a.wdw[0] + p);
    e.wy = HINT ? ldg_hint(a.wdw[1] + p, pol) : __ldg(a.wdw[1] + p);
    e.xa.lo = sm[lc];
    e.xa.hi = sm[hs + lc];
    e.ya.lo = sm[2 * hs + lc];
    e.ya.hi = sm[3 * hs + lc];
  }
  if (LAP) {
    e.wl = HINT ? ldg_hint(a.wldw + p, pol) : __ldg(a.wldw + p);
    e.qq.lo = sm[kq * hs + lc];
    e.qq.hi = sm[(kq + 1) * hs + lc];
  }
  return e;
}

template <bool RV, bool LAP>
static __device__ __forceinline__ void rev_accum(const RevEntry& e, dw::Acc* sx, dw::Acc* sy,
                                                 dw::Acc* sl) {
  if (RV) {
    const float2 X[4] = {lo2(e.xa.lo), hi2(e.xa.lo), lo2(e.xa.hi), hi2(e.xa.hi)};
    const float2 Y[4] = {lo2(e.ya.lo), hi2(e.ya.lo), lo2(e.ya.hi), hi2(e.ya.hi)};
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      dw::fma_acc(sx[v], e.wx, X[v]);
      dw::fma_acc(sy[v], e.wy, Y[v]);
    }
  }
  if (LAP) {
    const float2 Z[4] = {lo2(e.qq.lo), hi2(e.qq.lo), lo2(e.qq.hi), hi2(e.qq.hi)};
#pragma unroll
    for (int v = 0; v < 4; ++v) dw::fma_acc(sl[v], e.wl, Z[v]);
  }
}

// Transpose gather (Euler) over the reverse adjacency, as k_rev_f64:
// du_i = du_p_i - sum_j (Dx[j,i] s_x[j] + Dy[j,i] s_y[j]) - gamma sum_j lap[j,i] q[j],
// with s = eps * t and q as double-word pairs.  PIPE and MINB as for k_fwd_euler_dw.
template <bool RV, bool LAP, int PIPE, int MINB, bool PREF, bool HALO, bool HINT = false>
__global__ void __launch_bounds__(HALO ? kHaloRows : kBlock, MINB) k_rev_euler_dw(RevArgs a) {
  constexpr int NCH = (RV ? 4 : 0) + (LAP ? 2 : 0);
  const int64_t r = blockIdx.x * (int64_t)(HALO ? (int)blockDim.x : kBlock) + threadIdx.x;
  const float* __restrict__ S = reinterpret_cast<const float*>(a.sdw);
  const float* __restrict__ Q = reinterpret_cast<const float*>(a.qdw);
  extern __shared__ float4 hsm[];
  bool staged = false;
  if (HALO && NCH > 0) {
    const float4* S4 = reinterpret_cast<const float4*>(a.sdw);
    const float4* Q4 = reinterpret_cast<const float4*>(a.qdw);
    staged = stage_halo<NCH>(a.ell, hsm, [&](int k, int64_t c) {
      return (RV && k < 4) ? S4 + c * 4 + k : Q4 + c * 2 + (k - (RV ? 4 : 0));
    });
  }
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  const int32_t* __restrict__ col = a.ell.col;
  dw::Acc sx[4], sy[4], sl[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) { sx[v] = dw::zero(); sy[v] = dw::zero(); sl[v] = dw::zero(); }
  const uint16_t* __restrict__ lcol = a.ell.lcol;
  const int hs = a.ell.halo_stride;
  if (HALO && staged) {
    SliceArrays sa{};
    int64_t s_lo = 0, s_hi = 0;
    const bool pf_lane = PREF && (threadIdx.x & 31) == 0;
    if (pf_lane) {
      int k = 0;
      sa.arr[k] = lcol; sa.esize[k++] = 2;
      if (RV) { sa.arr[k] = a.wdw[0]; sa.esize[k++] = 8; sa.arr[k] = a.wdw[1]; sa.esize[k++] = 8; }
      if (LAP) { sa.arr[k] = a.wldw; sa.esize[k++] = 8; }
      sa.narr = k;
      s_lo = a.ell.slice_off[r >> 5];
      s_hi = a.ell.slice_off[(r >> 5) + 1];
      prefetch_chunk(sa, s_lo, s_hi, 0);
      prefetch_chunk(sa, s_lo, s_hi, 1);
    }
    constexpr int UNR = PIPE < 1 ? 1 : PIPE;
    const uint64_t pol = HINT ? l2_evict_first() : 0;
#pragma unroll UNR
    for (int j = 0; j < len; ++j) {
      if (pf_lane && (j % kPfSlots) == 0) prefetch_chunk(sa, s_lo, s_hi, j / kPfSlots + 2);
      const int64_t p = base + ((int64_t)j << 5);
      const int lc = HINT ? ldg_hint(lcol + p, pol) : __ldg(lcol + p);
      rev_accum<RV, LAP>(rev_load_halo<RV, LAP, HINT>(a, hsm, hs, p, lc, pol), sx, sy, sl);
    }
  } else if (PIPE == 0) {
#pragma unroll 1
    for (int j = 0; j < len; ++j) {
      const int64_t p = base + ((int64_t)j << 5);
      const int64_t c = __ldg(col + p);
      rev_accum<RV, LAP>(rev_load<RV, LAP>(a, S, Q, p, c), sx, sy, sl);
    }
  } else if (PIPE == 2 || (HALO && PIPE > 2)) {
    SliceArrays sa{};
    int64_t s_lo = 0, s_hi = 0;
    const bool pf_lane = PREF && (threadIdx.x & 31) == 0;
    if (pf_lane) {
      int k = 0;
      sa.arr[k] = col; sa.esize[k++] = 4;
      if (RV) { sa.arr[k] = a.wdw[0]; sa.esize[k++] = 8; sa.arr[k] = a.wdw[1]; sa.esize[k++] = 8; }
      if (LAP) { sa.arr[k] = a.wldw; sa.esize[k++] = 8; }
      sa.narr = k;
      s_lo = a.ell.slice_off[r >> 5];
      s_hi = a.ell.slice_off[(r >> 5) + 1];
      prefetch_chunk(sa, s_lo, s_hi, 0);
      prefetch_chunk(sa, s_lo, s_hi, 1);
    }
#pragma unroll 2
    for (int j = 0; j < len; ++j) {
      if (pf_lane && (j % kPfSlots) == 0) prefetch_chunk(sa, s_lo, s_hi, j / kPfSlots + 2);
      const int64_t p = base + ((int64_t)j << 5);
      const int64_t c = __ldg(col + p);
      rev_accum<RV, LAP>(rev_load<RV, LAP>(a, S, Q, p, c), sx, sy, sl);
    }
  } else if (len > 0) {
    int64_t c_next = len > 1 ? (int64_t)__ldg(col + base + 32) : 0;
    RevEntry cur = rev_load<RV, LAP>(a, S, Q, base, __ldg(col + base));
    for (int j = 0; j < len; ++j) {
      const int64_t p1 = base + ((int64_t)(j + 1) << 5);
      const int64_t c2 = j + 2 < len ? (int64_t)__ldg(col + p1 + 32) : 0;
      RevEntry nxt;
      if (j + 1 < len) nxt = rev_load<RV, LAP>(a, S, Q, p1, c_next);
      rev_accum<RV, LAP>(cur, sx, sy, sl);
      cur = nxt;
      c_next = c2;
    }
  }
  double du[4];
  const double2* dp2 = reinterpret_cast<const double2*>(a.du_p) + i * 2;
  const double2 d0 = dp2[0], d1 = dp2[1];
  const double dp[4] = {d0.x, d0.y, d1.x, d1.y};
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    double d = dp[v];
    if (RV) d = dsub(dsub(d, dw::to_double(sx[v])), dw::to_double(sy[v]));
    if (LAP) d = fma(-a.hv_gamma, dw::to_double(sl[v]), d);
    if (a.hvf) d = dadd(d, a.hvf[i * 4 + v]);
    du[v] = d;
  }
  if (a.final_epilogue) {
    finish_node<4>(a.ep, i, du);
  } else {
    double2* o2 = reinterpret_cast<double2*>(a.du_p_out) + i * 2;
    o2[0] = make_double2(du[0], du[1]);
    o2[1] = make_double2(du[2], du[3]);
  }
}

}  // namespace

float2 gm1_pair(double gamma) {
  const double gm1 = gamma - 1.0;
  const float h = (float)gm1;
  return make_float2(h, (float)(gm1 - (double)h));
}

bool dw_fwd_fuses(int variant) { return variant == 7 || variant == 11 || variant == 12; }

void launch_prep_euler_dw(int64_t n, double gamma, const double* u, float2* F, float2* U,
                          cudaStream_t s) {
  if (n <= 0) return;
  k_prep_euler_dw<<<grid_for(n, 256), 256, 0, s>>>(n, gm1_pair(gamma), u,
                                                   reinterpret_cast<float4*>(F),
                                                   reinterpret_cast<float4*>(U));
  MFT_LAUNCH_CHECK();
}

namespace {

// Kernel variants: 0 = one entry per loop iteration (fewest registers, most resident
// warps), 1 = two entries per iteration with the register count capped at six blocks per
// SM, 2 = two entries per iteration uncapped, 3 = software pipeline, 4 = variant 1 with
// the slice's streamed arrays prefetched into L2 ahead of use, 5 = variant 2 with it,
// 6 / 7 = neighbour records staged per row group in shared memory (one / two entries per
// iteration, registers capped at three blocks of kHaloRows per SM), 8 = variant 7 capped
// at four blocks, 9 / 11 = staged with four / three entries per iteration, 10 = variant 7
// with the streamed position and weight arrays prefetched into L2 (as variant 4), 12 =
// variant 7 with L2 eviction-priority hints (streamed arrays evict-first; the forward
// gather's t, q and partial du evict-last for the transpose gather).  Without halos
// (not built) the staged variants run as variant 2.
// A staged launch: one block per row group, NCH chunks of the layout's longest list
// in dynamic shared memory (above 48 KB that needs a per-kernel opt-in, made once per
// kernel and device).
template <typename Args>
void launch_staged(void (*k)(Args), const Args& a, int nch, int64_t n, cudaStream_t s,
                   bool pdl = false) {
  const size_t smem = (size_t)nch * a.ell.halo_stride * sizeof(float4);
  if (smem > 48 * 1024) {
    static std::mutex mu;
    static std::set<std::pair<const void*, int>> done;
    int dev = 0;
    MFT_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (done.insert({reinterpret_cast<const void*>(k), dev}).second)
      MFT_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(6 * kHaloMax * sizeof(float4))));
  }
  const int rows = a.ell.halo_rows;
  launch_k(k, grid_for(n, rows), rows, smem, s, pdl, a);
}

template <bool WT, bool WQ, int FLY>
void fwd_variant(const FwdArgs& a, int variant, int64_t n, cudaStream_t s) {
  const unsigned g = grid_for(n, kBlock);
  constexpr int nch = (WT || WQ || FLY) ? 6 : 4;
  const bool pdl = a.pdl != 0;
  if (variant >= 6 && !a.ell.halo_off) variant = 2;
  if (a.fuse_flux && a.ell.halo_off && dw_fwd_fuses(variant)) {
    MFT_REQUIRE(a.ustate && a.err, MFT_ERR_STATE, "fused staging needs the state and error word");
    switch (variant) {
      case 7: launch_staged(k_fwd_euler_dw<WT, WQ, FLY, 2, 3, false, true, false, true>, a, nch, n, s, pdl); break;
      case 11: launch_staged(k_fwd_euler_dw<WT, WQ, FLY, 3, 3, false, true, false, true>, a, nch, n, s, pdl); break;
      default: launch_staged(k_fwd_euler_dw<WT, WQ, FLY, 2, 3, false, true, true, true>, a, nch, n, s, pdl); break;
    }
    return;
  }
  switch (variant) {
    case 1: launch_k(k_fwd_euler_dw<WT, WQ, FLY, 2, 6, false, false>, g, kBlock, 0, s, pdl, a); break;
    case 2: launch_k(k_fwd_euler_dw<WT, WQ, FLY, 2, 1, false, false>, g, kBlock, 0, s, pdl, a); break;
    case 3: launch_k(k_fwd_euler_dw<WT, WQ, FLY, 1, 1, false, false>, g, kBlock, 0, s, pdl, a); break;
    case 4: launch_k(k_fwd_euler_dw<WT, WQ, FLY, 2, 6, true, false>, g, kBlock, 0, s, pdl, a); break;
    case 5: launch_k(k_fwd_euler_dw<WT, WQ, FLY, 2, 1, true, false>, g, kBlock, 0, s, pdl, a); break;
    case 6: launch_staged(k_fwd_euler_dw<WT, WQ, FLY, 0, 3, false, true>, a, nch, n, s, pdl); break;
    case 7: launch_staged(k_fwd_euler_dw<WT, WQ, FLY, 2, 3, false, true>, a, nch, n, s, pdl); break;
    case 8: launch_staged(k_fwd_euler_dw<WT, WQ, FLY, 2, 4, false, true>, a, nch, n, s, pdl); break;
    case 9: launch_staged(k_fwd_euler_dw<WT, WQ, FLY, 4, 3, false, true>, a, nch, n, s, pdl); break;
    case 10: launch_staged(k_fwd_euler_dw<WT, WQ, FLY, 2, 3, true, true>, a, nch, n, s, pdl); break;
    case 11: launch_staged(k_fwd_euler_dw<WT, WQ, FLY, 3, 3, false, true>, a, nch, n, s, pdl); break;
    case 12: launch_staged(k_fwd_euler_dw<WT, WQ, FLY, 2, 3, false, true, true>, a, nch, n, s, pdl); break;
    default: launch_k(k_fwd_euler_dw<WT, WQ, FLY, 0, 1, false, false>, g, kBlock, 0, s, pdl, a); break;
  }
}

template <bool RV, bool LAP>
void rev_variant(const RevArgs& a, int variant, int64_t n, cudaStream_t s) {
  const unsigned g = grid_for(n, kBlock);
  constexpr int nch = (RV ? 4 : 0) + (LAP ? 2 : 0);
  if (variant >= 6 && !a.ell.halo_off) variant = 2;
  switch (variant) {
    case 1: k_rev_euler_dw<RV, LAP, 2, 6, false, false><<<g, kBlock, 0, s>>>(a); break;
    case 2: k_rev_euler_dw<RV, LAP, 2, 1, false, false><<<g, kBlock, 0, s>>>(a); break;
    case 3: k_rev_euler_dw<RV, LAP, 1, 1, false, false><<<g, kBlock, 0, s>>>(a); break;
    case 4: k_rev_euler_dw<RV, LAP, 2, 6, true, false><<<g, kBlock, 0, s>>>(a); break;
    case 5: k_rev_euler_dw<RV, LAP, 2, 1, true, false><<<g, kBlock, 0, s>>>(a); break;
    case 6: launch_staged(k_rev_euler_dw<RV, LAP, 0, 3, false, true>, a, nch, n, s); break;
    case 7: launch_staged(k_rev_euler_dw<RV, LAP, 2, 3, false, true>, a, nch, n, s); break;
    case 8: launch_staged(k_rev_euler_dw<RV, LAP, 2, 4, false, true>, a, nch, n, s); break;
    case 9: launch_staged(k_rev_euler_dw<RV, LAP, 4, 3, false, true>, a, nch, n, s); break;
    case 10: launch_staged(k_rev_euler_dw<RV, LAP, 2, 3, true, true>, a, nch, n, s); break;
    case 11: launch_staged(k_rev_euler_dw<RV, LAP, 3, 3, false, true>, a, nch, n, s); break;
    case 12: launch_staged(k_rev_euler_dw<RV, LAP, 2, 3, false, true, true>, a, nch, n, s); break;
    default: k_rev_euler_dw<RV, LAP, 0, 1, false, false><<<g, kBlock, 0, s>>>(a); break;
  }
}

}  // namespace

void launch_fwd_dw(const FwdArgs& a, int variant, cudaStream_t s) {
  if (a.n <= 0) return;
  MFT_REQUIRE(a.V == 4, MFT_ERR_UNSUPPORTED, "double-word gathers: 2D Euler only");
  MFT_REQUIRE(!(a.flyer && a.want_q), MFT_ERR_UNSUPPORTED,
              "Flyer and Tominec hyperviscosity together are not supported");
  const int64_t n = a.n;
  const bool wt = a.want_t != 0, wq = a.want_q != 0;
  if (a.flyer == 0) {
    if (wt && wq) fwd_variant<true, true, 0>(a, variant, n, s);
    else if (wt) fwd_variant<true, false, 0>(a, variant, n, s);
    else if (wq) fwd_variant<false, true, 0>(a, variant, n, s);
    else fwd_variant<false, false, 0>(a, variant, n, s);
  } else if (a.flyer == 1) {
    if (wt) fwd_variant<true, false, 1>(a, variant, n, s);
    else fwd_variant<false, false, 1>(a, variant, n, s);
  } else {
    if (wt) fwd_variant<true, false, 2>(a, variant, n, s);
    else fwd_variant<false, false, 2>(a, variant, n, s);
  }
  MFT_LAUNCH_CHECK();
}

void launch_rev_dw(const RevArgs& a, int variant, cudaStream_t s) {
  if (a.n <= 0) return;
  MFT_REQUIRE(a.V == 4, MFT_ERR_UNSUPPORTED, "double-word gathers: 2D Euler only");
  const int64_t n = a.n;
  if (a.rv && a.lap) rev_variant<true, true>(a, variant, n, s);
  else if (a.rv) rev_variant<true, false>(a, variant, n, s);
  else if (a.lap) rev_variant<false, true>(a, variant, n, s);
  else rev_variant<false, false>(a, variant, n, s);
  MFT_LAUNCH_CHECK();
}

}  // namespace mft
