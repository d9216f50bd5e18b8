// FP64 form of the 2D Euler rhs! gathers in double-word FP32 arithmetic (mft_dw.cuh).
//
// Same passes, layouts and epilogues as the FP64 kernels (mft_apply.cu); what changes is
// how the sums over a stencil are formed.  Operator weights, the per-node fluxes and the
// neighbour states are read as double-word pairs (h, l) -- 8 bytes per value, the
// footprint of an FP64 value -- and the products and sums run on the FP32 pipe with
// error-free transformations; per-node values (the stage epilogue, the viscosity) stay
// in FP64.  Accumulation order per row is the layout's ascending-column order, as in the
// FP64 kernels.
#include <cuda_runtime.h>
#include <math.h>

#include "mft_device.cuh"
#include "mft_dw.cuh"
#include "mft_eps.cuh"
#include "mft_internal.cuh"

namespace mft {

namespace {

using namespace dev;

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

static __device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
static __device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }

// Per node: the state as double-word pairs and the Euler flux pair evaluated from them in
// double-word arithmetic (the textbook flux, one reciprocal for both velocities; each
// operation is accurate to about 2 u^2 of its operands, u = 2^-24), stored as pairs:
// F[i] = (Fx_0..3, Fy_0..3), U[i] = (u_0..3), 8 floats per 4 values.  gm1 = gamma - 1 as
// a pair.  The only FP64 operations are the four splits of the state.
__global__ void k_prep_euler_dw(int64_t n, float2 gm1, const double* __restrict__ u,
                                float4* __restrict__ F, float4* __restrict__ U) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2* ui = reinterpret_cast<const double2*>(u) + i * 2;
  const double2 a = ui[0], b = ui[1];
  const float2 rho = dw::split(a.x), m1 = dw::split(a.y), m2 = dw::split(b.x);
  const float2 en = dw::split(b.y);
  const float2 r = dw::recip(rho);
  const float2 v1 = dw::mul(m1, r), v2 = dw::mul(m2, r);
  const float2 a1 = dw::mul(m1, v1), a2 = dw::mul(m2, v2);
  const float2 p = dw::mul(gm1, dw::add(en, dw::neg(dw::scale2(dw::add(a1, a2), 0.5f))));
  const float2 ep = dw::add(en, p);
  const float2 fx1 = dw::add(a1, p), fx2 = dw::mul(m1, v2), fx3 = dw::mul(ep, v1);
  const float2 fy1 = dw::mul(m2, v1), fy2 = dw::add(a2, p), fy3 = dw::mul(ep, v2);
  float4* Fi = F + i * 4;
  Fi[0] = make_float4(m1.x, m1.y, fx1.x, fx1.y);
  Fi[1] = make_float4(fx2.x, fx2.y, fx3.x, fx3.y);
  Fi[2] = make_float4(m2.x, m2.y, fy1.x, fy1.y);
  Fi[3] = make_float4(fy2.x, fy2.y, fy3.x, fy3.y);
  U[i * 2] = make_float4(rho.x, rho.y, m1.x, m1.y);
  U[i * 2 + 1] = make_float4(m2.x, m2.y, en.x, en.y);
}

// Forward gather (Euler), one node per thread over the sliced ELL: the flux divergence
// -sum_j (Dx F_x + Dy F_y), t = (Dx u, Dy u) (WT), q = lap u (WQ) or the Flyer term
// H u (FLY), as in k_fwd_euler_f64.  Per stencil entry: a 64-byte flux record and a
// 32-byte state record (both one or two 256-bit loads), 8-byte weights.
template <bool WT, bool WQ, int FLY>
__global__ void __launch_bounds__(kBlock) k_fwd_euler_dw(FwdArgs a) {
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  const int32_t* __restrict__ col = a.ell.col;
  const float2* __restrict__ wxp = a.wdw[0];
  const float2* __restrict__ wyp = a.wdw[1];
  const float2* __restrict__ wlp = a.wldw;
  const float* __restrict__ F = reinterpret_cast<const float*>(a.Fdw);
  const float* __restrict__ U = reinterpret_cast<const float*>(a.udw);
  dw::Acc f[4], tx[4], ty[4], q[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    f[v] = dw::zero(); tx[v] = dw::zero(); ty[v] = dw::zero(); q[v] = dw::zero();
  }
#pragma unroll 2
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int64_t c = __ldg(col + p);
    const float2 wx = __ldg(wxp + p), wy = __ldg(wyp + p);
    const F8 fa = ldg_f8(F + c * 16), fb = ldg_f8(F + c * 16 + 8);
    const float2 Fx[4] = {lo2(fa.lo), hi2(fa.lo), lo2(fa.hi), hi2(fa.hi)};
    const float2 Fy[4] = {lo2(fb.lo), hi2(fb.lo), lo2(fb.hi), hi2(fb.hi)};
#pragma unroll
    for (int v = WT ? 1 : 0; v < 4; ++v) {
      // Fx[0] = m1, Fy[0] = m2: with t formed, the rho row is tx1 + ty2
      dw::fma_acc(f[v], wx, Fx[v]);
      dw::fma_acc(f[v], wy, Fy[v]);
    }
    if (WT || WQ || FLY) {
      const F8 uu = ldg_f8(U + c * 8);
      const float2 uc[4] = {lo2(uu.lo), hi2(uu.lo), lo2(uu.hi), hi2(uu.hi)};
      if (WT) {
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          dw::fma_acc(tx[v], wx, uc[v]);
          dw::fma_acc(ty[v], wy, uc[v]);
        }
      }
      if (WQ || FLY) {
        const float2 wl = __ldg(wlp + p);
#pragma unroll
        for (int v = 0; v < 4; ++v) dw::fma_acc(q[v], wl, uc[v]);
      }
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
      // gathers of other warps
      const double eps = visc::eps_value<4>(a.ea, i, du);
      if (a.ea.eps) a.ea.eps[i] = eps;
      const float2 e2 = dw::split(eps);
#pragma unroll
      for (int v = 0; v < 4; ++v) { x[v] = dw::mul(e2, x[v]); y[v] = dw::mul(e2, y[v]); }
    }
    t4[0] = make_float4(x[0].x, x[0].y, x[1].x, x[1].y);
    t4[1] = make_float4(x[2].x, x[2].y, x[3].x, x[3].y);
    t4[2] = make_float4(y[0].x, y[0].y, y[1].x, y[1].y);
    t4[3] = make_float4(y[2].x, y[2].y, y[3].x, y[3].y);
  }
  if (WQ) {
    float4* q4 = reinterpret_cast<float4*>(a.qdw) + i * 2;
    float2 x[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) x[v] = dw::to_pair(q[v]);
    q4[0] = make_float4(x[0].x, x[0].y, x[1].x, x[1].y);
    q4[1] = make_float4(x[2].x, x[2].y, x[3].x, x[3].y);
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
    d2[0] = make_double2(du[0], du[1]);
    d2[1] = make_double2(du[2], du[3]);
  }
}

// Transpose gather (Euler) over the reverse adjacency, as k_rev_f64:
// du_i = du_p_i - sum_j (Dx[j,i] s_x[j] + Dy[j,i] s_y[j]) - gamma sum_j lap[j,i] q[j],
// with s = eps * t and q as double-word pairs.
template <bool RV, bool LAP>
__global__ void __launch_bounds__(kBlock) k_rev_euler_dw(RevArgs a) {
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  const float* __restrict__ S = reinterpret_cast<const float*>(a.sdw);
  const float* __restrict__ Q = reinterpret_cast<const float*>(a.qdw);
  dw::Acc sx[4], sy[4], sl[4];
#pragma unroll
  for (int v = 0; v < 4; ++v) { sx[v] = dw::zero(); sy[v] = dw::zero(); sl[v] = dw::zero(); }
#pragma unroll 2
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int64_t c = __ldg(a.ell.col + p);
    if (RV) {
      const float2 wx = __ldg(a.wdw[0] + p), wy = __ldg(a.wdw[1] + p);
      const F8 xa = ldg_f8(S + c * 16), ya = ldg_f8(S + c * 16 + 8);
      const float2 X[4] = {lo2(xa.lo), hi2(xa.lo), lo2(xa.hi), hi2(xa.hi)};
      const float2 Y[4] = {lo2(ya.lo), hi2(ya.lo), lo2(ya.hi), hi2(ya.hi)};
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        dw::fma_acc(sx[v], wx, X[v]);
        dw::fma_acc(sy[v], wy, Y[v]);
      }
    }
    if (LAP) {
      const float2 wl = __ldg(a.wldw + p);
      const F8 qq = ldg_f8(Q + c * 8);
      const float2 Z[4] = {lo2(qq.lo), hi2(qq.lo), lo2(qq.hi), hi2(qq.hi)};
#pragma unroll
      for (int v = 0; v < 4; ++v) dw::fma_acc(sl[v], wl, Z[v]);
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

void launch_prep_euler_dw(int64_t n, double gamma, const double* u, float2* F, float2* U,
                          cudaStream_t s) {
  if (n <= 0) return;
  const double gm1 = gamma - 1.0;
  const float h = (float)gm1;
  const float2 gm1dw = make_float2(h, (float)(gm1 - (double)h));
  k_prep_euler_dw<<<grid_for(n, 256), 256, 0, s>>>(n, gm1dw, u, reinterpret_cast<float4*>(F),
                                                   reinterpret_cast<float4*>(U));
  MFT_LAUNCH_CHECK();
}

void launch_fwd_dw(const FwdArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  MFT_REQUIRE(a.V == 4, MFT_ERR_UNSUPPORTED, "double-word gathers: 2D Euler only");
  MFT_REQUIRE(!(a.flyer && a.want_q), MFT_ERR_UNSUPPORTED,
              "Flyer and Tominec hyperviscosity together are not supported");
  const unsigned g = grid_for(a.n, kBlock);
  const bool wt = a.want_t != 0, wq = a.want_q != 0;
  if (a.flyer == 0) {
    if (wt && wq) k_fwd_euler_dw<true, true, 0><<<g, kBlock, 0, s>>>(a);
    else if (wt) k_fwd_euler_dw<true, false, 0><<<g, kBlock, 0, s>>>(a);
    else if (wq) k_fwd_euler_dw<false, true, 0><<<g, kBlock, 0, s>>>(a);
    else k_fwd_euler_dw<false, false, 0><<<g, kBlock, 0, s>>>(a);
  } else if (a.flyer == 1) {
    if (wt) k_fwd_euler_dw<true, false, 1><<<g, kBlock, 0, s>>>(a);
    else k_fwd_euler_dw<false, false, 1><<<g, kBlock, 0, s>>>(a);
  } else {
    if (wt) k_fwd_euler_dw<true, false, 2><<<g, kBlock, 0, s>>>(a);
    else k_fwd_euler_dw<false, false, 2><<<g, kBlock, 0, s>>>(a);
  }
  MFT_LAUNCH_CHECK();
}

void launch_rev_dw(const RevArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  MFT_REQUIRE(a.V == 4, MFT_ERR_UNSUPPORTED, "double-word gathers: 2D Euler only");
  const unsigned g = grid_for(a.n, kBlock);
  if (a.rv && a.lap) k_rev_euler_dw<true, true><<<g, kBlock, 0, s>>>(a);
  else if (a.rv) k_rev_euler_dw<true, false><<<g, kBlock, 0, s>>>(a);
  else if (a.lap) k_rev_euler_dw<false, true><<<g, kBlock, 0, s>>>(a);
  else k_rev_euler_dw<false, false><<<g, kBlock, 0, s>>>(a);
  MFT_LAUNCH_CHECK();
}

}  // namespace mft
