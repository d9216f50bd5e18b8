// Operator-apply kernels of the RBF-FD rhs! (FP64 form) for sm_103a.
//
// Pass structure of one rhs! evaluation (reference: Trixi.rhs!,
// src/solvers/pointcloudsolver/rbfsolver.jl:397-428):
//   bc_pass1   strong BCs on the boundary-node list (rbfsolver.jl:288-318)
//   flux       F(u) per node (Euler flux in FP64 is issue-bound on this part,
//              so it is evaluated once per node, not once per stencil entry)
//   fwd        one sliced-ELL gather over the stencil: -sum_d D_d F_d, and, for the
//              viscosity sources, t = D_d u and q = lap u (calc_fluxes!, :247-265)
//   mean/lexmax  ode_mean / ode_maximum (src/auxiliary/mpi.jl:40-81)
//   eps        update_upwind_visc! / update_residual_visc! / update_visc!
//              (src/sources/hyperviscosity.jl:246-349), s = eps * t
//   rev        transpose gather -sum_d D_d' s_d (and lap' q) over the reverse
//              adjacency (hyperviscosity.jl:401-407, :121-134), BC pass 2 and the
//              SSP-RK stage combination as epilogue.
#include <cuda_runtime.h>
#include <math.h>

#include <cmath>

#include "mft_device.cuh"
#include "mft_dw.cuh"
#include "mft_eps.cuh"
#include "mft_internal.cuh"

namespace mft {

namespace {

using namespace dev;

// ------------------------------------------------------------------ layout

__global__ void k_aos_from_soa(const double* __restrict__ soa, double* __restrict__ aos,
                               int64_t n, int V) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int v = 0; v < V; ++v) aos[i * V + v] = soa[(int64_t)v * n + i];
}
__global__ void k_soa_from_aos(const double* __restrict__ aos, double* __restrict__ soa,
                               int64_t n, int V) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int v = 0; v < V; ++v) soa[(int64_t)v * n + i] = aos[i * V + v];
}
// SoA <-> AoS between the engine state and caller arrays addressed one pointer per
// variable (pinned, device-mapped host memory or device memory).
template <int V>
__global__ void k_aos_from_vars(VarPtrs src, double* __restrict__ aos, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int v = 0; v < V; ++v) aos[i * V + v] = src.p[v][i];
}
template <int V>
__global__ void k_vars_from_aos(const double* __restrict__ aos, VarPtrs dst, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int v = 0; v < V; ++v) dst.p[v][i] = aos[i * V + v];
}
// The same for V = 4 with two nodes per thread and 16-byte accesses to the caller's
// arrays (host memory read or written over the host link: fewer, wider requests).  The
// caller checks that every array is 16-byte aligned; an odd last node is taken singly.
__global__ void k_aos_from_vars4x2(VarPtrs src, double* __restrict__ aos, int64_t n) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = 2 * j;
  if (i >= n) return;
  if (i + 1 < n) {
    double2 v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = reinterpret_cast<const double2*>(src.p[k])[j];
    double2* o = reinterpret_cast<double2*>(aos) + i * 2;
    o[0] = make_double2(v[0].x, v[1].x);
    o[1] = make_double2(v[2].x, v[3].x);
    o[2] = make_double2(v[0].y, v[1].y);
    o[3] = make_double2(v[2].y, v[3].y);
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) aos[i * 4 + k] = src.p[k][i];
  }
}
__global__ void k_vars_from_aos4x2(const double* __restrict__ aos, VarPtrs dst, int64_t n) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = 2 * j;
  if (i >= n) return;
  if (i + 1 < n) {
    const double2* a = reinterpret_cast<const double2*>(aos) + i * 2;
    const double2 a0 = a[0], a1 = a[1], a2 = a[2], a3 = a[3];
    reinterpret_cast<double2*>(dst.p[0])[j] = make_double2(a0.x, a2.x);
    reinterpret_cast<double2*>(dst.p[1])[j] = make_double2(a0.y, a2.y);
    reinterpret_cast<double2*>(dst.p[2])[j] = make_double2(a1.x, a3.x);
    reinterpret_cast<double2*>(dst.p[3])[j] = make_double2(a1.y, a3.y);
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) dst.p[k][i] = aos[i * 4 + k];
  }
}
__global__ void k_to_f32(const double* __restrict__ a, float* __restrict__ b, int64_t count) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < count) b[i] = fpconv::d2f(a[i]);
}

// ------------------------------------------------------------------ BC pass 1

__global__ void k_bc_pass1(int64_t nb, const int32_t* __restrict__ bnode, int V, int eq, BcDev bc,
                           double* __restrict__ u, float* __restrict__ u32) {
  int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b >= nb) return;
  const int64_t i = bnode[b];
  const int tag = bc.tag[i];
  const int64_t slot = bc.slot[i];
  if (tag == 1) {
    for (int v = 0; v < V; ++v) u[i * V + v] = bc.dvalues[slot * V + v];
  } else if (tag == 2 && eq == MFT_EQ_EULER2D) {
    double uu[4] = {u[i * 4 + 0], u[i * 4 + 1], u[i * 4 + 2], u[i * 4 + 3]};
    slip(bc.normal + 2 * slot, uu);
    u[i * 4 + 1] = uu[1];
    u[i * 4 + 2] = uu[2];
  } else {
    return;
  }
  if (u32)
    for (int v = 0; v < V; ++v) u32[i * V + v] = fpconv::d2f(u[i * V + v]);
}

// ------------------------------------------------------------------ flux

__global__ void k_flux_euler(int64_t n, double g, const double* __restrict__ u,
                             double* __restrict__ F) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2* ui = reinterpret_cast<const double2*>(u) + i * 2;
  const double2 a = ui[0], b = ui[1];
  // The textbook flux with one reciprocal for both velocities (an FP64 division is a
  // long sequence on this part): v = m * (1 / rho) is within an ulp of m / rho.
  const double rho = a.x, m1 = a.y, m2 = b.x, en = b.y;
  const double rinv = ddiv(1.0, rho);
  const double v1 = dmul(m1, rinv), v2 = dmul(m2, rinv);
  const double p = dmul(dsub(g, 1.0), dsub(en, dmul(0.5, dadd(dmul(m1, v1), dmul(m2, v2)))));
  const double ep = dadd(en, p);
  const double fx[4] = {m1, dadd(dmul(m1, v1), p), dmul(m1, v2), dmul(ep, v1)};
  const double fy[4] = {m2, dmul(m2, v1), dadd(dmul(m2, v2), p), dmul(ep, v2)};
  double2* Fi = reinterpret_cast<double2*>(F) + i * 4;
  Fi[0] = make_double2(fx[0], fx[1]);
  Fi[1] = make_double2(fx[2], fx[3]);
  Fi[2] = make_double2(fy[0], fy[1]);
  Fi[3] = make_double2(fy[2], fy[3]);
}

// ------------------------------------------------------------------ forward gather

// Euler (V = 4), FP64.  One node per thread; lane r of a warp owns row 32*s + r of
// slice s and reads slot j at slice_off[s] + 32*j + r (coalesced weights/indices).
// Per stencil entry: 64 B flux gather (+32 B state gather for t/q), 8 FP64 FMAs for
// the flux divergence (6 when t is formed: d rho/dt reuses t).
template <bool WT, bool WQ, int FLY>
__global__ void __launch_bounds__(kBlock) k_fwd_euler_f64(FwdArgs a) {
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  const int32_t* __restrict__ col = a.ell.col;
  const double* __restrict__ wxp = a.w[0];
  const double* __restrict__ wyp = a.w[1];
  const double* __restrict__ wlp = a.wl;
  const double2* __restrict__ F2 = reinterpret_cast<const double2*>(a.F);
  const double2* __restrict__ U2 = reinterpret_cast<const double2*>(a.u);
  double f0 = 0, f1 = 0, f2 = 0, f3 = 0;                 // sum wx Fx + wy Fy
  double tx0 = 0, tx1 = 0, tx2 = 0, tx3 = 0, ty0 = 0, ty1 = 0, ty2 = 0, ty3 = 0;
  double q0 = 0, q1 = 0, q2 = 0, q3 = 0;
#pragma unroll 2
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int64_t c = __ldg(col + p);
    const double wx = __ldg(wxp + p), wy = __ldg(wyp + p);
    const double2 fa = __ldg(F2 + c * 4 + 0), fb = __ldg(F2 + c * 4 + 1);
    const double2 fc = __ldg(F2 + c * 4 + 2), fd = __ldg(F2 + c * 4 + 3);
    if (WT) {
      // Fx[0] = rho v1 = u[1], Fy[0] = rho v2 = u[2]: the rho row of the flux
      // divergence is tx1 + ty2, so it needs no FMAs of its own.
      f1 = fma(wx, fa.y, f1); f1 = fma(wy, fc.y, f1);
      f2 = fma(wx, fb.x, f2); f2 = fma(wy, fd.x, f2);
      f3 = fma(wx, fb.y, f3); f3 = fma(wy, fd.y, f3);
    } else {
      f0 = fma(wx, fa.x, f0); f0 = fma(wy, fc.x, f0);
      f1 = fma(wx, fa.y, f1); f1 = fma(wy, fc.y, f1);
      f2 = fma(wx, fb.x, f2); f2 = fma(wy, fd.x, f2);
      f3 = fma(wx, fb.y, f3); f3 = fma(wy, fd.y, f3);
    }
    if (WT || WQ || FLY) {
      const double2 ua = __ldg(U2 + c * 2), ub = __ldg(U2 + c * 2 + 1);
      if (WT) {
        tx0 = fma(wx, ua.x, tx0); tx1 = fma(wx, ua.y, tx1); tx2 = fma(wx, ub.x, tx2); tx3 = fma(wx, ub.y, tx3);
        ty0 = fma(wy, ua.x, ty0); ty1 = fma(wy, ua.y, ty1); ty2 = fma(wy, ub.x, ty2); ty3 = fma(wy, ub.y, ty3);
      }
      if (WQ || FLY) {
        const double wl = __ldg(wlp + p);
        q0 = fma(wl, ua.x, q0); q1 = fma(wl, ua.y, q1); q2 = fma(wl, ub.x, q2); q3 = fma(wl, ub.y, q3);
      }
    }
  }
  if (WT) f0 = tx1 + ty2;
  double du[4] = {-f0, -f1, -f2, -f3};
  if (FLY == 1) {
    du[0] = fma(-a.hv_gamma, q0, du[0]); du[1] = fma(-a.hv_gamma, q1, du[1]);
    du[2] = fma(-a.hv_gamma, q2, du[2]); du[3] = fma(-a.hv_gamma, q3, du[3]);
  }
  if (WT) {
    double2* t2 = reinterpret_cast<double2*>(a.t) + i * 4;
    t2[0] = make_double2(tx0, tx1); t2[1] = make_double2(tx2, tx3);
    t2[2] = make_double2(ty0, ty1); t2[3] = make_double2(ty2, ty3);
  }
  if (WQ) {
    double2* q2p = reinterpret_cast<double2*>(a.q) + i * 2;
    q2p[0] = make_double2(q0, q1); q2p[1] = make_double2(q2, q3);
  }
  if (FLY == 2) {
    double2* h2 = reinterpret_cast<double2*>(a.hvf) + i * 2;
    h2[0] = make_double2(-a.hv_gamma * q0, -a.hv_gamma * q1);
    h2[1] = make_double2(-a.hv_gamma * q2, -a.hv_gamma * q3);
  }
  if (a.final_epilogue) {
    finish_node<4>(a.ep, i, du);
  } else {
    double2* d2 = reinterpret_cast<double2*>(a.du_p) + i * 2;
    d2[0] = make_double2(du[0], du[1]);
    d2[1] = make_double2(du[2], du[3]);
  }
}

// Scalar advection (V = 1), FP64: flux a_d * u evaluated at the neighbour.
template <bool WT, bool WQ, int FLY>
__global__ void __launch_bounds__(kBlock) k_fwd_adv_f64(FwdArgs a) {
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  double f = 0, tx = 0, ty = 0, q = 0;
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int64_t c = __ldg(a.ell.col + p);
    const double wx = __ldg(a.w[0] + p), wy = __ldg(a.w[1] + p);
    const double uc = __ldg(a.u + c);
    f = fma(wx, a.ax * uc, f);
    f = fma(wy, a.ay * uc, f);
    if (WT) { tx = fma(wx, uc, tx); ty = fma(wy, uc, ty); }
    if (WQ || FLY) q = fma(__ldg(a.wl + p), uc, q);
  }
  double du[1] = {-f};
  if (FLY == 1) du[0] = fma(-a.hv_gamma, q, du[0]);
  if (WT) { a.t[i * 2] = tx; a.t[i * 2 + 1] = ty; }
  if (WQ) a.q[i] = q;
  if (FLY == 2) a.hvf[i] = -a.hv_gamma * q;
  if (a.final_epilogue) finish_node<1>(a.ep, i, du);
  else a.du_p[i] = du[0];
}

// ------------------------------------------------------------------ reductions

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarps = kBlock / 32;

// The warp's totals of V FP64 partial sums per lane.  For V = 4 the lanes first
// reduce-scatter (lanes 16 apart exchange half of their sums, then lanes 8 apart half of
// the rest), so that each FP64 addition of those steps serves two or four sums; then each
// group of 8 lanes finishes its sum with a shuffle tree.  Afterwards lane l holds the
// total of sum l >> 3 (V = 4) or of the only sum (V = 1).  Six full-warp additions for
// four sums instead of twenty; a fixed order, so the result is deterministic.
template <int V>
__device__ __forceinline__ double warp_sum_scatter(const double* v, int lane) {
  static_assert(V == 1 || V == 4, "one or four sums");
  double k;
  if (V == 4) {
    const bool hi16 = (lane & 16) != 0;
    double a0 = hi16 ? v[2 % V] : v[0], a1 = hi16 ? v[3 % V] : v[1 % V];
    const double s0 = hi16 ? v[0] : v[2 % V], s1 = hi16 ? v[1 % V] : v[3 % V];
    a0 = dadd(a0, __shfl_xor_sync(kFull, s0, 16));
    a1 = dadd(a1, __shfl_xor_sync(kFull, s1, 16));
    const bool hi8 = (lane & 8) != 0;
    k = hi8 ? a1 : a0;
    k = dadd(k, __shfl_xor_sync(kFull, hi8 ? a0 : a1, 8));
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) k = dadd(k, __shfl_xor_sync(kFull, k, o));
  } else {
    k = v[0];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) k = dadd(k, __shfl_xor_sync(kFull, k, o));
  }
  return k;
}

// Block totals of V partial sums per thread: lane k < V of warp 0 returns total k (other
// threads return 0).  The warps' totals are combined by warp 0 with a shuffle tree.
template <int V>
__device__ double block_sum_lanes(const double* v) {
  static_assert(kWarps * V <= 32, "one warp combines the warps' totals");
  __shared__ double sh[V * kWarps];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const double k = warp_sum_scatter<V>(v, lane);
  if ((lane & (V == 4 ? 7 : 31)) == 0) sh[(V == 4 ? lane >> 3 : 0) * kWarps + wid] = k;
  __syncthreads();
  double r = 0.0;
  if (wid == 0) {
    double x = lane < V * kWarps ? sh[lane] : 0.0;  // lane = sum * kWarps + warp
#pragma unroll
    for (int o = kWarps / 2; o > 0; o >>= 1) x = dadd(x, __shfl_xor_sync(kFull, x, o));
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const double t = __shfl_sync(kFull, x, q * kWarps);
      if (lane == q) r = t;
    }
  }
  __syncthreads();
  return r;
}

// Sum of u per variable; the last block to finish reduces the block partials in a fixed
// order (deterministic) and writes mean = sum / denom.  A grid launched after this one
// with launch_k(pdl) may start at once (it waits for the means with pdl_wait).
template <int V, bool VEC>
__global__ void __launch_bounds__(kBlock) k_mean(int64_t n, const double* __restrict__ u,
                                                 double denom, double* partial,
                                                 unsigned* counter, double* mean) {
  pdl_trigger();
  double acc[V];
#pragma unroll
  for (int k = 0; k < V; ++k) acc[k] = 0.0;
  // unrolled so that four nodes' loads are in flight together; the additions keep the
  // node order of the plain grid-stride loop
#pragma unroll 4
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kBlock) {
    if (VEC && V == 4) {
      const double2* u2 = reinterpret_cast<const double2*>(u) + i * 2;
      const double2 a = __ldg(u2), b = __ldg(u2 + 1);
      acc[0] = dadd(acc[0], a.x); acc[1 % V] = dadd(acc[1 % V], a.y);
      acc[2 % V] = dadd(acc[2 % V], b.x); acc[3 % V] = dadd(acc[3 % V], b.y);
    } else {
#pragma unroll
      for (int k = 0; k < V; ++k) acc[k] = dadd(acc[k], u[i * V + k]);
    }
  }
  const double tot = block_sum_lanes<V>(acc);
  __shared__ int last;
  if (threadIdx.x < 32) {
    double t[V];
#pragma unroll
    for (int k = 0; k < V; ++k) t[k] = __shfl_sync(kFull, tot, k);
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < V; ++k) partial[blockIdx.x * V + k] = t[k];
      __threadfence();
      last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
#pragma unroll
  for (int k = 0; k < V; ++k) acc[k] = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += kBlock)
#pragma unroll
    for (int k = 0; k < V; ++k) acc[k] = dadd(acc[k], __ldcg(partial + b * V + k));
  const double all = block_sum_lanes<V>(acc);
  if (threadIdx.x < V) mean[threadIdx.x] = all / denom;
  if (threadIdx.x == 0) *counter = 0u;
}

// ode_maximum(|u - mean|) (mpi.jl:61-81): lexicographic Base.isless order on vectors
// (max_mode 0) or per component (1); zero entries become eps() (update_residual_visc!,
// hyperviscosity.jl:310-311).  |u - mean| >= 0, so the IEEE bit pattern of every
// component orders like its value (NaN above +Inf, as Base.isless does): the maximum
// is taken on 64-bit integer keys.
typedef unsigned long long u64;
// |x| as a bit pattern: the sign bit cleared (fabs, without an FP64 instruction)
constexpr u64 kAbsMask = 0x7FFFFFFFFFFFFFFFull;

template <int V>
__device__ __forceinline__ bool key_less(const u64* a, const u64* b) {
#pragma unroll
  for (int k = 0; k < V; ++k)
    if (a[k] != b[k]) return a[k] < b[k];
  return false;
}

// max(a, b) = isless(b, a) ? a : b, written into a.
template <int V>
__device__ __forceinline__ void key_max_into(u64* a, const u64* b, int max_mode) {
  if (max_mode == 0) {
    if (!key_less<V>(b, a)) {
#pragma unroll
      for (int k = 0; k < V; ++k) a[k] = b[k];
    }
  } else {
#pragma unroll
    for (int k = 0; k < V; ++k) a[k] = a[k] < b[k] ? b[k] : a[k];
  }
}

// The block's maximum key (integer shuffles and one exchange through shared memory);
// valid in lane 0 of warp 0.  The maximum is a value, not a position: any order gives it.
template <int V>
__device__ void block_keymax(u64* best, int max_mode) {
  __shared__ u64 sh[kWarps][V];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    u64 c[V];
#pragma unroll
    for (int k = 0; k < V; ++k) c[k] = __shfl_xor_sync(kFull, best[k], o);
    key_max_into<V>(best, c, max_mode);
  }
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < V; ++k) sh[wid][k] = best[k];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < V; ++k) best[k] = lane < kWarps ? sh[lane][k] : 0ull;
#pragma unroll
    for (int o = kWarps / 2; o > 0; o >>= 1) {
      u64 c[V];
#pragma unroll
      for (int k = 0; k < V; ++k) c[k] = __shfl_xor_sync(kFull, best[k], o);
      key_max_into<V>(best, c, max_mode);
    }
  }
  __syncthreads();
}

// The norms from the maximum key (warp 0; lane k < V writes component k).
template <int V>
__device__ __forceinline__ void write_norms(const u64* best, double* norms) {
  const int lane = threadIdx.x & 31;
  double v = 0.0;
#pragma unroll
  for (int k = 0; k < V; ++k) {
    const double t = __longlong_as_double((long long)__shfl_sync(kFull, best[k], 0));
    if (lane == k) v = t;
  }
  if (lane < V) {
    const double nv = v == 0.0 ? 2.220446049250313e-16 : v;
    norms[lane] = nv;
    norms[V + lane] = 1.0 / nv;
  }
}

template <int V, bool VEC>
__global__ void __launch_bounds__(kBlock) k_lexmax(int64_t n, const double* __restrict__ u,
                                                   const double* __restrict__ mean, int max_mode,
                                                   double* partial, unsigned* counter,
                                                   double* norms) {
  pdl_trigger();
  pdl_wait();  // the means (k_mean, which this grid may overlap)
  double m[V];
  u64 best[V];
#pragma unroll
  for (int k = 0; k < V; ++k) { m[k] = __ldcg(mean + k); best[k] = 0ull; }
  // Threads without nodes keep the all-zero key, the smallest possible: it can only
  // tie with a real all-zero vector, which has the same value.
#pragma unroll 4
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kBlock) {
    double uv[V];
    if (VEC && V == 4) {
      const double2* u2 = reinterpret_cast<const double2*>(u) + i * 2;
      const double2 a = __ldg(u2), b = __ldg(u2 + 1);
      uv[0] = a.x; uv[1 % V] = a.y; uv[2 % V] = b.x; uv[3 % V] = b.y;
    } else {
#pragma unroll
      for (int k = 0; k < V; ++k) uv[k] = u[i * V + k];
    }
    u64 x[V];
#pragma unroll
    for (int k = 0; k < V; ++k) x[k] = (u64)__double_as_longlong(dsub(uv[k], m[k])) & kAbsMask;
    key_max_into<V>(best, x, max_mode);
  }
  block_keymax<V>(best, max_mode);
  __shared__ int last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < V; ++k) partial[blockIdx.x * V + k] = __longlong_as_double((long long)best[k]);
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
#pragma unroll
  for (int k = 0; k < V; ++k) best[k] = 0ull;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += kBlock) {
    u64 c[V];
#pragma unroll
    for (int k = 0; k < V; ++k) c[k] = (u64)__double_as_longlong(__ldcg(partial + b * V + k));
    key_max_into<V>(best, c, max_mode);
  }
  block_keymax<V>(best, max_mode);
  if (threadIdx.x < 32) write_norms<V>(best, norms);
  if (threadIdx.x == 0) *counter = 0u;
}

// Segmented versions for ensembles: segment s owns nodes [off[s], off[s+1]) and is
// reduced by `per` blocks (blockIdx.x = s * per + part); the last block of a segment
// finishes it in the same fixed order as above.
template <int V>
__global__ void __launch_bounds__(kBlock) k_mean_seg(const int64_t* __restrict__ off, int per,
                                                     const double* __restrict__ u, int mode,
                                                     double* partial, unsigned* counter,
                                                     double* mean) {
  pdl_trigger();
  const int sg = blockIdx.x / per, part = blockIdx.x % per;
  const int64_t lo = off[sg], hi = off[sg + 1];
  double acc[V];
#pragma unroll
  for (int k = 0; k < V; ++k) acc[k] = 0.0;
  for (int64_t i = lo + (int64_t)part * kBlock + threadIdx.x; i < hi; i += (int64_t)per * kBlock) {
#pragma unroll
    for (int k = 0; k < V; ++k) acc[k] = dadd(acc[k], u[i * V + k]);
  }
  const double tot = block_sum_lanes<V>(acc);
  __shared__ int last;
  if (threadIdx.x < 32) {
    double t[V];
#pragma unroll
    for (int k = 0; k < V; ++k) t[k] = __shfl_sync(kFull, tot, k);
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < V; ++k) partial[blockIdx.x * V + k] = t[k];
      __threadfence();
      last = (atomicAdd(counter + sg, 1u) == (unsigned)per - 1);
    }
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
#pragma unroll
  for (int k = 0; k < V; ++k) acc[k] = 0.0;
  for (int b = threadIdx.x; b < per; b += kBlock)
#pragma unroll
    for (int k = 0; k < V; ++k) acc[k] = dadd(acc[k], __ldcg(partial + (sg * per + b) * V + k));
  const double all = block_sum_lanes<V>(acc);
  if (threadIdx.x < V) {
    const double denom = mode == 0 ? (double)(hi - lo) * V : (double)(hi - lo);
    mean[sg * V + threadIdx.x] = all / denom;
  }
  if (threadIdx.x == 0) counter[sg] = 0u;
}

template <int V>
__global__ void __launch_bounds__(kBlock) k_lexmax_seg(const int64_t* __restrict__ off, int per,
                                                       const double* __restrict__ u,
                                                       const double* __restrict__ mean,
                                                       int max_mode, double* partial,
                                                       unsigned* counter, double* norms) {
  pdl_trigger();
  pdl_wait();  // the means (k_mean_seg)
  const int sg = blockIdx.x / per, part = blockIdx.x % per;
  const int64_t lo = off[sg], hi = off[sg + 1];
  double m[V];
  u64 best[V];
#pragma unroll
  for (int k = 0; k < V; ++k) { m[k] = __ldcg(mean + sg * V + k); best[k] = 0ull; }
  for (int64_t i = lo + (int64_t)part * kBlock + threadIdx.x; i < hi; i += (int64_t)per * kBlock) {
    u64 x[V];
#pragma unroll
    for (int k = 0; k < V; ++k) x[k] = (u64)__double_as_longlong(dsub(u[i * V + k], m[k])) & kAbsMask;
    key_max_into<V>(best, x, max_mode);
  }
  block_keymax<V>(best, max_mode);
  __shared__ int last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < V; ++k) partial[blockIdx.x * V + k] = __longlong_as_double((long long)best[k]);
    __threadfence();
    last = (atomicAdd(counter + sg, 1u) == (unsigned)per - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
#pragma unroll
  for (int k = 0; k < V; ++k) best[k] = 0ull;
  for (int b = threadIdx.x; b < per; b += kBlock) {
    u64 c[V];
#pragma unroll
    for (int k = 0; k < V; ++k)
      c[k] = (u64)__double_as_longlong(__ldcg(partial + (sg * per + b) * V + k));
    key_max_into<V>(best, c, max_mode);
  }
  block_keymax<V>(best, max_mode);
  if (threadIdx.x < 32) write_norms<V>(best, norms + sg * 2 * V);
  if (threadIdx.x == 0) counter[sg] = 0u;
}

// ------------------------------------------------------------------ viscosity

template <int V>
__global__ void __launch_bounds__(kBlock) k_eps(EpsArgs a) {
  const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  if (i >= a.n) return;
  const double eps = visc::eps_value<V>(a, i, nullptr);
  if (a.eps) a.eps[i] = eps;
  if (a.t) {
    if (V == 4) {
      double2* t2 = reinterpret_cast<double2*>(a.t) + i * 4;
      double2 x[4] = {t2[0], t2[1], t2[2], t2[3]};
#pragma unroll
      for (int q = 0; q < 4; ++q) t2[q] = make_double2(dmul(eps, x[q].x), dmul(eps, x[q].y));
    } else {
#pragma unroll
      for (int k = 0; k < 2 * V; ++k) a.t[i * 2 * V + k] = dmul(eps, a.t[i * 2 * V + k]);
    }
  }
  if (a.tdw) {
    // s = eps * t in double-word arithmetic (eps split once per node)
    const float2 e2 = dw::split(eps);
    float4* t4 = reinterpret_cast<float4*>(a.tdw) + i * V;
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const float4 x = t4[q];
      const float2 lo = dw::mul(e2, make_float2(x.x, x.y));
      const float2 hi = dw::mul(e2, make_float2(x.z, x.w));
      t4[q] = make_float4(lo.x, lo.y, hi.x, hi.y);
    }
  }
  if (a.t32) {
    const float e32 = __double2float_rn(eps);
#pragma unroll
    for (int k = 0; k < 2 * V; ++k) a.t32[i * 2 * V + k] = e32 * a.t32[i * 2 * V + k];
  }
}

// ------------------------------------------------------------------ transpose gather

// du_i = du_p_i - sum_{j: i in stencil(j)} (Dx[j,i] s_x[j] + Dy[j,i] s_y[j])
//               - gamma * sum_j lap[j,i] q[j]
// over the reverse adjacency (CSC column i), in the layout's entry order.
template <int V, bool RV, bool LAP>
__global__ void __launch_bounds__(kBlock) k_rev_f64(RevArgs a) {
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  double sx[V], sy[V], sl[V];
#pragma unroll
  for (int v = 0; v < V; ++v) { sx[v] = 0; sy[v] = 0; sl[v] = 0; }
#pragma unroll 2
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int64_t c = __ldg(a.ell.col + p);
    if (RV) {
      const double wx = __ldg(a.w[0] + p), wy = __ldg(a.w[1] + p);
      if (V == 4) {
        const double2* S2 = reinterpret_cast<const double2*>(a.s) + c * 4;
        const double2 xa = __ldg(S2), xb = __ldg(S2 + 1), ya = __ldg(S2 + 2), yb = __ldg(S2 + 3);
        sx[0] = fma(wx, xa.x, sx[0]); sx[1] = fma(wx, xa.y, sx[1]);
        sx[2] = fma(wx, xb.x, sx[2]); sx[3] = fma(wx, xb.y, sx[3]);
        sy[0] = fma(wy, ya.x, sy[0]); sy[1] = fma(wy, ya.y, sy[1]);
        sy[2] = fma(wy, yb.x, sy[2]); sy[3] = fma(wy, yb.y, sy[3]);
      } else {
        sx[0] = fma(wx, __ldg(a.s + c * 2), sx[0]);
        sy[0] = fma(wy, __ldg(a.s + c * 2 + 1), sy[0]);
      }
    }
    if (LAP) {
      const double wl = __ldg(a.wl + p);
#pragma unroll
      for (int v = 0; v < V; ++v) sl[v] = fma(wl, __ldg(a.q + c * V + v), sl[v]);
    }
  }
  double du[V];
#pragma unroll
  for (int v = 0; v < V; ++v) {
    double d = a.du_p[i * V + v];
    if (RV) d = (d - sx[v]) - sy[v];
    if (LAP) d = fma(-a.hv_gamma, sl[v], d);
    if (a.hvf) d = d + a.hvf[i * V + v];
    du[v] = d;
  }
  if (a.final_epilogue) {
    finish_node<V>(a.ep, i, du);
  } else {
#pragma unroll
    for (int v = 0; v < V; ++v) a.du_p_out[i * V + v] = du[v];
  }
}

// ------------------------------------------------------------------ history

// FUSED (FP32-apply form): fused multiply-adds, half the FP64 operations; the FP64 form
// keeps the separately rounded products and sums of the reference's broadcasts.
template <bool FUSED>
__device__ __forceinline__ double hist_acc(double acc, double w, double h) {
  return FUSED ? fma(w, h, acc) : dadd(acc, dmul(w, h));
}

// The first term: 0 + w h is w h itself (it can differ only in the sign of a zero, which
// |approx_du - du| in the viscosity does not see), so the addition is skipped.
__device__ __forceinline__ double hist_first(int m, double w, double h) {
  return m > 0 ? dmul(w, h) : 0.0;
}

// approx_du = sum_{k<M} w_k h_k for two values per thread, M known at compile time so
// that the M 16-byte loads of a thread are in flight together (h_0 is the new state).
template <bool FUSED, int M>
__device__ __forceinline__ double2 history_pair(const double2 (&h)[M > 0 ? M : 1],
                                                const double* w) {
  double ax = hist_first(M, w[0], h[0].x), ay = hist_first(M, w[0], h[0].y);
#pragma unroll
  for (int k = 1; k < M; ++k) {
    ax = hist_acc<FUSED>(ax, w[k], h[k].x);
    ay = hist_acc<FUSED>(ay, w[k], h[k].y);
  }
  return make_double2(ax, ay);
}

// approx_du .= 0; approx_du .+= w_k .* sol_k (history.jl:115-126) outside a captured
// step, two values per thread: h0 is the new state, also copied into its ring slot dst
// (never one of h1..h7).
template <bool FUSED, int M>
__device__ __forceinline__ void history_host_pair(int64_t j, const double* const (&hs)[8],
                                                  const HistW& w, double* dst, double* out) {
  double2 h[M > 0 ? M : 1];
#pragma unroll
  for (int k = 0; k < (M > 0 ? M : 1); ++k) h[k] = reinterpret_cast<const double2*>(hs[k])[j];
  reinterpret_cast<double2*>(dst)[j] = h[0];
  reinterpret_cast<double2*>(out)[j] = history_pair<FUSED, M>(h, w.w);
}

template <bool FUSED>
__global__ void k_history(int64_t count, int m, HistW w, const double* h0,
                          const double* h1, const double* h2, const double* h3,
                          const double* h4, const double* h5, const double* h6,
                          const double* h7, double* __restrict__ dst,
                          double* __restrict__ out) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = 2 * j;
  if (i >= count) return;
  const double* hs[8] = {h0, h1, h2, h3, h4, h5, h6, h7};
  if (i + 1 < count) {
    switch (m) {
#define MFT_HIST_CASE(M) \
  case M: history_host_pair<FUSED, M>(j, hs, w, dst, out); return;
      MFT_HIST_CASE(0) MFT_HIST_CASE(1) MFT_HIST_CASE(2) MFT_HIST_CASE(3)
      MFT_HIST_CASE(4) MFT_HIST_CASE(5) MFT_HIST_CASE(6) MFT_HIST_CASE(7)
      default: history_host_pair<FUSED, 8>(j, hs, w, dst, out); return;
#undef MFT_HIST_CASE
    }
  }
  const double un = h0[i];
  dst[i] = un;
  double acc = hist_first(m, w.w[0], un);
#pragma unroll
  for (int k = 1; k < 8; ++k)  // constant indices: hs and w stay in registers
    if (k < m) acc = hist_acc<FUSED>(acc, w.w[k], hs[k][i]);
  out[i] = acc;
}

__global__ void k_differs(const double* __restrict__ a, const double* __restrict__ b,
                          int64_t count, int* flag) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < count && __double_as_longlong(a[i]) != __double_as_longlong(b[i])) *flag = 1;
}

__global__ void k_scatter_values(int64_t nnz, const int64_t* __restrict__ pos,
                                 const double* __restrict__ v, double* __restrict__ out,
                                 float* __restrict__ out32, float2* __restrict__ outdw) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= nnz) return;
  const int64_t p = pos[e];
  out[p] = v[e];
  if (out32) out32[p] = fpconv::d2f(v[e]);
  if (outdw) outdw[p] = dw::split(v[e]);
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

// ====================================================================== launchers

void launch_scatter_values(int64_t nnz, const int64_t* pos, const double* v, double* out,
                           float* out32, float2* outdw, cudaStream_t s) {
  if (nnz <= 0) return;
  k_scatter_values<<<grid_for(nnz, 256), 256, 0, s>>>(nnz, pos, v, out, out32, outdw);
  MFT_LAUNCH_CHECK();
}

void launch_aos_from_soa(const double* soa, double* aos, int64_t n, int V, cudaStream_t s) {
  if (n <= 0) return;
  k_aos_from_soa<<<grid_for(n, 256), 256, 0, s>>>(soa, aos, n, V);
  MFT_LAUNCH_CHECK();
}
static bool aligned16(const VarPtrs& v, int nv) {
  for (int k = 0; k < nv; ++k)
    if (reinterpret_cast<uintptr_t>(v.p[k]) & 15) return false;
  return true;
}
void launch_aos_from_vars(const VarPtrs& src, double* aos, int64_t n, int V, cudaStream_t s) {
  if (n <= 0) return;
  MFT_REQUIRE(V == 1 || V == 4, MFT_ERR_UNSUPPORTED, "1 or 4 variables");
  if (V == 4 && aligned16(src, 4))
    k_aos_from_vars4x2<<<grid_for((n + 1) / 2, 256), 256, 0, s>>>(src, aos, n);
  else if (V == 4) k_aos_from_vars<4><<<grid_for(n, 256), 256, 0, s>>>(src, aos, n);
  else k_aos_from_vars<1><<<grid_for(n, 256), 256, 0, s>>>(src, aos, n);
  MFT_LAUNCH_CHECK();
}
void launch_vars_from_aos(const double* aos, const VarPtrs& dst, int64_t n, int V,
                          cudaStream_t s) {
  if (n <= 0) return;
  MFT_REQUIRE(V == 1 || V == 4, MFT_ERR_UNSUPPORTED, "1 or 4 variables");
  if (V == 4 && aligned16(dst, 4))
    k_vars_from_aos4x2<<<grid_for((n + 1) / 2, 256), 256, 0, s>>>(aos, dst, n);
  else if (V == 4) k_vars_from_aos<4><<<grid_for(n, 256), 256, 0, s>>>(aos, dst, n);
  else k_vars_from_aos<1><<<grid_for(n, 256), 256, 0, s>>>(aos, dst, n);
  MFT_LAUNCH_CHECK();
}
void launch_soa_from_aos(const double* aos, double* soa, int64_t n, int V, cudaStream_t s) {
  if (n <= 0) return;
  k_soa_from_aos<<<grid_for(n, 256), 256, 0, s>>>(aos, soa, n, V);
  MFT_LAUNCH_CHECK();
}
void launch_aos_to_f32(const double* aos, float* a32, int64_t count, cudaStream_t s) {
  if (count <= 0) return;
  k_to_f32<<<grid_for(count, 256), 256, 0, s>>>(aos, a32, count);
  MFT_LAUNCH_CHECK();
}

void launch_bc_pass1(int64_t nb, const int32_t* bnode, int V, int eq, BcDev bc, double* u,
                     float* u32, cudaStream_t s) {
  if (nb <= 0) return;
  k_bc_pass1<<<grid_for(nb, 128), 128, 0, s>>>(nb, bnode, V, eq, bc, u, u32);
  MFT_LAUNCH_CHECK();
}

void launch_flux_f64(int64_t n, int eq, int V, double gamma, const double* u, double* F,
                     cudaStream_t s) {
  if (eq != MFT_EQ_EULER2D || n <= 0) return;
  (void)V;
  k_flux_euler<<<grid_for(n, 256), 256, 0, s>>>(n, gamma, u, F);
  MFT_LAUNCH_CHECK();
}

template <int V>
static void fwd_dispatch(const FwdArgs& a, cudaStream_t s) {
  const unsigned g = grid_for(a.n, kBlock);
  const bool wt = a.want_t != 0, wq = a.want_q != 0;
#define MFT_FWD(WT, WQ, FLY)                                                       \
  do {                                                                             \
    if (V == 4) k_fwd_euler_f64<WT, WQ, FLY><<<g, kBlock, 0, s>>>(a);              \
    else k_fwd_adv_f64<WT, WQ, FLY><<<g, kBlock, 0, s>>>(a);                       \
  } while (0)
  if (a.flyer == 0) {
    if (wt && wq) MFT_FWD(true, true, 0);
    else if (wt) MFT_FWD(true, false, 0);
    else if (wq) MFT_FWD(false, true, 0);
    else MFT_FWD(false, false, 0);
  } else if (a.flyer == 1) {
    if (wt) MFT_FWD(true, false, 1);
    else MFT_FWD(false, false, 1);
  } else {
    if (wt) MFT_FWD(true, false, 2);
    else MFT_FWD(false, false, 2);
  }
#undef MFT_FWD
  MFT_LAUNCH_CHECK();
}

void launch_fwd_f64(const FwdArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  MFT_REQUIRE(!(a.flyer && a.want_q), MFT_ERR_UNSUPPORTED,
              "Flyer and Tominec hyperviscosity together are not supported");
  if (a.V == 4) fwd_dispatch<4>(a, s);
  else fwd_dispatch<1>(a, s);
}

void launch_mean(int64_t n, int V, const double* u, double denom, double* partial,
                 unsigned* counter, double* mean, int nblocks, cudaStream_t s) {
  const bool vec = (reinterpret_cast<uintptr_t>(u) & 15) == 0;
  if (V == 4 && vec) k_mean<4, true><<<nblocks, kBlock, 0, s>>>(n, u, denom, partial, counter, mean);
  else if (V == 4) k_mean<4, false><<<nblocks, kBlock, 0, s>>>(n, u, denom, partial, counter, mean);
  else k_mean<1, false><<<nblocks, kBlock, 0, s>>>(n, u, denom, partial, counter, mean);
  MFT_LAUNCH_CHECK();
}

void launch_lexmax(int64_t n, int V, const double* u, const double* mean, int max_mode,
                   double* partial, unsigned* counter, double* norms, int nblocks,
                   cudaStream_t s, bool pdl) {
  const bool vec = (reinterpret_cast<uintptr_t>(u) & 15) == 0;
  if (V == 4 && vec)
    launch_k(k_lexmax<4, true>, nblocks, kBlock, 0, s, pdl, n, u, mean, max_mode, partial,
             counter, norms);
  else if (V == 4)
    launch_k(k_lexmax<4, false>, nblocks, kBlock, 0, s, pdl, n, u, mean, max_mode, partial,
             counter, norms);
  else
    launch_k(k_lexmax<1, false>, nblocks, kBlock, 0, s, pdl, n, u, mean, max_mode, partial,
             counter, norms);
}

void launch_mean_seg(int nseg, const int64_t* off, int per, int V, const double* u, int mode,
                     double* partial, unsigned* counter, double* mean, cudaStream_t s) {
  if (nseg <= 0) return;
  if (V == 4) k_mean_seg<4><<<nseg * per, kBlock, 0, s>>>(off, per, u, mode, partial, counter, mean);
  else k_mean_seg<1><<<nseg * per, kBlock, 0, s>>>(off, per, u, mode, partial, counter, mean);
  MFT_LAUNCH_CHECK();
}

void launch_lexmax_seg(int nseg, const int64_t* off, int per, int V, const double* u,
                       const double* mean, int max_mode, double* partial, unsigned* counter,
                       double* norms, cudaStream_t s, bool pdl) {
  if (nseg <= 0) return;
  if (V == 4)
    launch_k(k_lexmax_seg<4>, nseg * per, kBlock, 0, s, pdl, off, per, u, mean, max_mode,
             partial, counter, norms);
  else
    launch_k(k_lexmax_seg<1>, nseg * per, kBlock, 0, s, pdl, off, per, u, mean, max_mode,
             partial, counter, norms);
}

void prepare_eps(EpsArgs& a) {
  // host IEEE double arithmetic without contraction: the same values the per-node
  // products give
  a.uw_coef = (a.c_uw * 0.5) * a.h;
  a.uw_adv = a.uw_coef * std::sqrt(a.ax * a.ax + a.ay * a.ay);
  a.rv_coef = (0.5 * a.c_rv) * (a.h * a.h);
  a.uw_bound = a.uw_coef * a.uw_coef * ((1.0 - 1e-12) / (1.0 + 1e-12));
  a.gg1 = a.gamma * (a.gamma - 1.0);
  const float h32 = (float)a.h;
  a.gamma32 = (float)a.gamma;
  a.gm1_32 = (float)(a.gamma - 1.0);
  a.uw_coef32 = ((float)a.c_uw * 0.5f) * h32;
  a.rv_coef32 = ((0.5f * (float)a.c_rv) * h32) * h32;
}

void launch_eps(const EpsArgs& args, cudaStream_t s) {
  if (args.n <= 0) return;
  EpsArgs a = args;
  prepare_eps(a);
  if (a.du_p32) {
    launch_eps_f32(a, s);
    return;
  }
  if (a.V == 4) k_eps<4><<<grid_for(a.n, kBlock), kBlock, 0, s>>>(a);
  else k_eps<1><<<grid_for(a.n, kBlock), kBlock, 0, s>>>(a);
  MFT_LAUNCH_CHECK();
}

void launch_rev_f64(const RevArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  const unsigned g = grid_for(a.n, kBlock);
  if (a.V == 4) {
    if (a.rv && a.lap) k_rev_f64<4, true, true><<<g, kBlock, 0, s>>>(a);
    else if (a.rv) k_rev_f64<4, true, false><<<g, kBlock, 0, s>>>(a);
    else if (a.lap) k_rev_f64<4, false, true><<<g, kBlock, 0, s>>>(a);
    else k_rev_f64<4, false, false><<<g, kBlock, 0, s>>>(a);
  } else {
    if (a.rv && a.lap) k_rev_f64<1, true, true><<<g, kBlock, 0, s>>>(a);
    else if (a.rv) k_rev_f64<1, true, false><<<g, kBlock, 0, s>>>(a);
    else if (a.lap) k_rev_f64<1, false, true><<<g, kBlock, 0, s>>>(a);
    else k_rev_f64<1, false, false><<<g, kBlock, 0, s>>>(a);
  }
  MFT_LAUNCH_CHECK();
}

namespace {

struct RingPtrs {
  double* p[8];
};

// Ring slot k of the history (constant-offset parameter loads, no local copy).
__device__ __forceinline__ double* ring_slot(const RingPtrs& r, int k) {
  switch (k) {
    case 0: return r.p[0];
    case 1: return r.p[1];
    case 2: return r.p[2];
    case 3: return r.p[3];
    case 4: return r.p[4];
    case 5: return r.p[5];
    case 6: return r.p[6];
    default: return r.p[7];
  }
}

template <bool FUSED, int M>
__device__ __forceinline__ void history_dev_pair(int64_t j, const double* u_new,
                                                 const RingPtrs& ring, int slots, int head,
                                                 const double* w, double* out) {
  double2 h[M > 0 ? M : 1];
  h[0] = reinterpret_cast<const double2*>(u_new)[j];
#pragma unroll
  for (int k = 1; k < M; ++k) {
    int q = head + k;
    if (q >= slots) q -= slots;
    h[k] = reinterpret_cast<const double2*>(ring_slot(ring, q))[j];
  }
  reinterpret_cast<double2*>(ring_slot(ring, head))[j] = h[0];
  reinterpret_cast<double2*>(out)[j] = history_pair<FUSED, M>(h, w);
}

// HistoryCallback push inside a captured step: the step's parameters come from the
// step table at the device step counter.  ring[head] = u_new, then
// approx_du = sum_{k<m} w_k ring[(head + k) % slots] (k = 0 is u_new itself).
// Two values per thread (16-byte loads and stores); count is even or the last thread
// takes the single remaining value.  The ring slots read are never ring[head], the one
// written.
template <bool FUSED>
__global__ void k_history_dev(int64_t count, const double* __restrict__ u_new, RingPtrs ring,
                              int slots, const StepParams* __restrict__ tab,
                              const int* __restrict__ ctr, double* __restrict__ out) {
  const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t i = 2 * j;
  if (i >= count) return;
  const StepParams* sp = tab + *ctr;
  const int m = sp->m, head = sp->head;
  if (i + 1 < count) {
    switch (m) {
#define MFT_HIST_CASE(M) \
  case M: history_dev_pair<FUSED, M>(j, u_new, ring, slots, head, sp->w, out); return;
      MFT_HIST_CASE(0) MFT_HIST_CASE(1) MFT_HIST_CASE(2) MFT_HIST_CASE(3)
      MFT_HIST_CASE(4) MFT_HIST_CASE(5) MFT_HIST_CASE(6) MFT_HIST_CASE(7)
      default: history_dev_pair<FUSED, 8>(j, u_new, ring, slots, head, sp->w, out); return;
#undef MFT_HIST_CASE
    }
  }
  double* dst = ring_slot(ring, head);
  const double un = u_new[i];
  dst[i] = un;
  double acc = hist_first(m, sp->w[0], un);
  for (int k = 1; k < m; ++k) {
    int q = head + k;
    if (q >= slots) q -= slots;
    acc = hist_acc<FUSED>(acc, sp->w[k], ring_slot(ring, q)[i]);
  }
  out[i] = acc;
}

__global__ void k_step_advance(int* ctr) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *ctr += 1;
}

}  // namespace

void launch_history_dev(int64_t count, const double* u_new, const double* const* ring,
                        int slots, const StepParams* tab, const int* ctr, double* approx_du,
                        bool fused, cudaStream_t s) {
  if (count <= 0) return;
  RingPtrs rp{};
  for (int k = 0; k < slots && k < 8; ++k) rp.p[k] = const_cast<double*>(ring[k]);
  const unsigned g = grid_for((count + 1) / 2, 256);
  if (fused) k_history_dev<true><<<g, 256, 0, s>>>(count, u_new, rp, slots, tab, ctr, approx_du);
  else k_history_dev<false><<<g, 256, 0, s>>>(count, u_new, rp, slots, tab, ctr, approx_du);
  MFT_LAUNCH_CHECK();
}

void launch_step_advance(int* ctr, cudaStream_t s) {
  k_step_advance<<<1, 32, 0, s>>>(ctr);
  MFT_LAUNCH_CHECK();
}

void launch_differs(const double* a, const double* b, int64_t count, int* flag, cudaStream_t s) {
  if (count <= 0) return;
  k_differs<<<grid_for(count, 256), 256, 0, s>>>(a, b, count, flag);
  MFT_LAUNCH_CHECK();
}

void launch_history(int64_t count, int m, const HistW& w, const double* const* hist,
                    double* ring_dst, double* approx_du, bool fused, cudaStream_t s) {
  if (count <= 0) return;
  const double* h[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  for (int k = 0; k < m && k < 8; ++k) h[k] = hist[k];
  const unsigned g = grid_for((count + 1) / 2, 256);
  if (fused)
    k_history<true><<<g, 256, 0, s>>>(count, m, w, h[0], h[1], h[2], h[3], h[4], h[5], h[6],
                                      h[7], ring_dst, approx_du);
  else
    k_history<false><<<g, 256, 0, s>>>(count, m, w, h[0], h[1], h[2], h[3], h[4], h[5], h[6],
                                       h[7], ring_dst, approx_du);
  MFT_LAUNCH_CHECK();
}

}  // namespace mft
