// FP32-apply form of the rhs! gathers: FP32 weights (generated in FP64), FP32
// states and FP32 accumulation in the operator apply; the SSP-RK stage combination
// (finish_node) stays in FP64.  The Euler flux is cheap in FP32, so it is evaluated
// at every stencil neighbour from the 16-byte FP32 state instead of being stored.
#include <cuda_runtime.h>
#include <math.h>

#include "mft_device.cuh"
#include "mft_halo.cuh"
#include "mft_internal.cuh"

namespace mft {

namespace {

using namespace dev;

// HALO: one block per row group (ell.halo_rows rows) first stages the group's neighbour
// states in shared memory (mft_halo.cuh) and reads them from there; groups without a list
// load them directly.  The sums are the same in the same order either way.
template <bool WT, bool WQ, int FLY, bool HALO = false>
__global__ void __launch_bounds__(HALO ? kHaloRows : kBlock) k_fwd_euler_f32(FwdArgs a) {
  const int64_t r = blockIdx.x * (int64_t)(HALO ? (int)blockDim.x : kBlock) + threadIdx.x;
  const float4* __restrict__ U4 = reinterpret_cast<const float4*>(a.u32);
  extern __shared__ float4 hsm[];
  bool staged = false;
  if (HALO) staged = stage_halo<1>(a.ell, hsm, [&](int, int64_t c) { return U4 + c; });
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  const int32_t* __restrict__ col = a.ell.col;
  const uint16_t* __restrict__ lcol = a.ell.lcol;
  const float* __restrict__ wxp = a.w32[0];
  const float* __restrict__ wyp = a.w32[1];
  const float* __restrict__ wlp = a.wl32;
  const float gm1 = a.gm1_32;
  float f[4] = {0, 0, 0, 0}, tx[4] = {0, 0, 0, 0}, ty[4] = {0, 0, 0, 0}, q[4] = {0, 0, 0, 0};
  auto entry = [&](int64_t p, const float4 uc) {
    const float wx = __ldg(wxp + p), wy = __ldg(wyp + p);
    euler_accum_f32<WT>(gm1, uc, wx, wy, f, tx, ty);
    if (WQ || FLY) {
      const float wl = __ldg(wlp + p);
      q[0] = fmaf(wl, uc.x, q[0]); q[1] = fmaf(wl, uc.y, q[1]);
      q[2] = fmaf(wl, uc.z, q[2]); q[3] = fmaf(wl, uc.w, q[3]);
    }
  };
  if (HALO && staged) {
#pragma unroll 4
    for (int j = 0; j < len; ++j) {
      const int64_t p = base + ((int64_t)j << 5);
      entry(p, hsm[__ldg(lcol + p)]);
    }
  } else {
#pragma unroll 4
    for (int j = 0; j < len; ++j) {
      const int64_t p = base + ((int64_t)j << 5);
      entry(p, __ldg(U4 + __ldg(col + p)));
    }
  }
  const float hg = a.hg32;
  if (WT) f[0] = tx[1] + ty[2];
  float du[4] = {-f[0], -f[1], -f[2], -f[3]};
  if (FLY == 1)
    for (int v = 0; v < 4; ++v) du[v] = fmaf(-hg, q[v], du[v]);
  if (WT) {
    float4* t4 = reinterpret_cast<float4*>(a.t32) + i * 2;
    t4[0] = make_float4(tx[0], tx[1], tx[2], tx[3]);
    t4[1] = make_float4(ty[0], ty[1], ty[2], ty[3]);
  }
  if (WQ) reinterpret_cast<float4*>(a.q32)[i] = make_float4(q[0], q[1], q[2], q[3]);
  if (FLY == 2)
    for (int v = 0; v < 4; ++v) a.hvf[i * 4 + v] = fpconv::f2d(-hg * q[v]);
  if (a.final_epilogue) {
    double d[4] = {fpconv::f2d(du[0]), fpconv::f2d(du[1]), fpconv::f2d(du[2]),
                   fpconv::f2d(du[3])};
    finish_node<4>(a.ep, i, d);
  } else {
    reinterpret_cast<float4*>(a.du_p32)[i] = make_float4(du[0], du[1], du[2], du[3]);
  }
}

template <bool WT, bool WQ, int FLY>
__global__ void __launch_bounds__(kBlock) k_fwd_adv_f32(FwdArgs a) {
  const int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;  // layout row
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  const float ax = (float)a.ax, ay = (float)a.ay;
  float f = 0, tx = 0, ty = 0, q = 0;
#pragma unroll 4
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int c = __ldg(a.ell.col + p);
    const float wx = __ldg(a.w32[0] + p), wy = __ldg(a.w32[1] + p);
    const float uc = __ldg(a.u32 + c);
    f = fmaf(wy, ay * uc, fmaf(wx, ax * uc, f));
    if (WT) { tx = fmaf(wx, uc, tx); ty = fmaf(wy, uc, ty); }
    if (WQ || FLY) q = fmaf(__ldg(a.wl32 + p), uc, q);
  }
  const float hg = a.hg32;
  float du = -f;
  if (FLY == 1) du = fmaf(-hg, q, du);
  if (WT) { a.t32[i * 2] = tx; a.t32[i * 2 + 1] = ty; }
  if (WQ) a.q32[i] = q;
  if (FLY == 2) a.hvf[i] = fpconv::f2d(-hg * q);
  if (a.final_epilogue) {
    double d[1] = {fpconv::f2d(du)};
    finish_node<1>(a.ep, i, d);
  } else {
    a.du_p32[i] = du;
  }
}

// update_upwind_visc! / update_residual_visc! / update_visc! in FP32
// (src/sources/hyperviscosity.jl:246-349); approx_du and the norms come from the
// FP64 history and reductions.
template <int V>
__global__ void __launch_bounds__(kBlock) k_eps_f32(EpsArgs a) {
  // FP64 -> FP32 conversions run on the FP64 pipe of this part: the state comes from its
  // FP32 shadow (the same rounded values), the node-independent factors from the launch
  // and, for one problem, the norms' reciprocals are converted once per block.
  // V = 4: the node's records (state, partial du, approx_du, t) are requested before the
  // block reads the norms and meets its barrier, so one memory latency covers them all.
  const int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  const bool valid = i < a.n;
  float4 q4 = {}, d4 = {}, tx4 = {}, ty4 = {};
  double2 a0 = {}, a1 = {};
  if (V == 4 && valid) {
    if (a.u32) q4 = reinterpret_cast<const float4*>(a.u32)[i];
    if (a.kind == MFT_SRC_RV) {
      d4 = reinterpret_cast<const float4*>(a.du_p32)[i];
      a0 = reinterpret_cast<const double2*>(a.approx_du)[i * 2];
      a1 = reinterpret_cast<const double2*>(a.approx_du)[i * 2 + 1];
    }
    const float4* t4 = reinterpret_cast<const float4*>(a.t32) + i * 2;
    tx4 = t4[0];
    ty4 = t4[1];
  }
  __shared__ float s_rnorm[V];
  if (!a.seg_id && threadIdx.x < V) s_rnorm[threadIdx.x] = (float)a.norms[V + threadIdx.x];
  __syncthreads();
  if (!valid) return;
  const int sg = a.seg_id ? a.seg_id[i] : 0;
  const float h = a.seg_h ? (float)a.seg_h[sg] : (float)a.h;
  float eps_uw;
  if (V == 4) {
    float rho, m1, m2, en;
    if (a.u32) {
      rho = q4.x; m1 = q4.y; m2 = q4.z; en = q4.w;
    } else {
      const double2 ua = reinterpret_cast<const double2*>(a.u)[i * 2];
      const double2 ub = reinterpret_cast<const double2*>(a.u)[i * 2 + 1];
      rho = (float)ua.x; m1 = (float)ua.y; m2 = (float)ub.x; en = (float)ub.y;
    }
    const float r = __frcp_rn(rho);
    const float v1 = m1 * r, v2 = m2 * r;
    const float p = a.gm1_32 * (en - 0.5f * (m1 * v1 + m2 * v2));
    const float speed = sqrtf(v1 * v1 + v2 * v2);
    const float c = (p < 0.0f || rho < 0.0f) ? 0.0f : sqrtf(a.gamma32 * p * r);
    const float uwc = a.seg_h ? (float)a.c_uw * 0.5f * h : a.uw_coef32;
    eps_uw = uwc * (speed + c);
  } else {
    eps_uw = (float)a.c_uw * 0.5f * h * (float)sqrt(a.ax * a.ax + a.ay * a.ay);
  }
  float eps;
  if (a.kind == MFT_SRC_RV) {
    // node records as 16-byte vectors (V = 4): du_p32 one float4, approx_du two double2
    float dpv[V], adv[V];
    if (V == 4) {
      dpv[0] = d4.x; dpv[1 % V] = d4.y; dpv[2 % V] = d4.z; dpv[3 % V] = d4.w;
      adv[0] = fpconv::d2f(a0.x); adv[1 % V] = fpconv::d2f(a0.y);
      adv[2 % V] = fpconv::d2f(a1.x); adv[3 % V] = fpconv::d2f(a1.y);
    } else {
      dpv[0] = a.du_p32[i];
      adv[0] = fpconv::d2f(a.approx_du[i]);
    }
    float mr = 0.0f;
#pragma unroll
    for (int v = 0; v < V; ++v) {
      float dp = dpv[v];
      if (a.hvf) dp += fpconv::d2f(a.hvf[i * V + v]);
      const float r = fabsf(adv[v] - dp);
      const float rn = a.seg_id ? (float)a.norms[sg * 2 * V + V + v] : s_rnorm[v];
      const float qv = r * rn;
      mr = v == 0 ? qv : fmaxf(mr, qv);
      if (isnan(qv)) mr = qv;
    }
    const float rvc = a.seg_h ? 0.5f * (float)a.c_rv * h * h : a.rv_coef32;
    const float eps_rv = rvc * mr;
    const int si = a.tab ? a.tab[*a.ctr].si_eps : a.success_iter;
    if (isnan(eps_rv) || isinf(eps_rv) || si == 0)
      eps = (isnan(eps_uw) || isinf(eps_uw)) ? 2.220446049250313e-16f : eps_uw;
    else
      eps = fminf(eps_rv, eps_uw);
  } else {
    eps = eps_uw;
  }
  if (a.eps) a.eps[i] = fpconv::f2d(eps);
  if (V == 4) {
    float4* t4 = reinterpret_cast<float4*>(a.t32) + i * 2;
    float4 x = tx4, y = ty4;
    x.x *= eps; x.y *= eps; x.z *= eps; x.w *= eps;
    y.x *= eps; y.y *= eps; y.z *= eps; y.w *= eps;
    t4[0] = x;
    t4[1] = y;
  } else {
#pragma unroll
    for (int k = 0; k < 2 * V; ++k) a.t32[i * 2 * V + k] *= eps;
  }
}

// HALO (V = 4 only): staged neighbour records as in k_fwd_euler_f32 -- s = eps t (two
// chunks) and q (one chunk).
template <int V, bool RV, bool LAP, bool HALO = false>
__global__ void __launch_bounds__(HALO ? kHaloRows : kBlock) k_rev_f32(RevArgs a) {
  static_assert(!HALO || V == 4, "staged transpose gather: 2D Euler");
  constexpr int NCH = (RV ? 2 : 0) + (LAP ? 1 : 0);
  const int64_t r = blockIdx.x * (int64_t)(HALO ? (int)blockDim.x : kBlock) + threadIdx.x;
  extern __shared__ float4 hsm[];
  bool staged = false;
  if (HALO && NCH > 0) {
    const float4* S4 = reinterpret_cast<const float4*>(a.s32);
    const float4* Q4 = reinterpret_cast<const float4*>(a.q32);
    staged = stage_halo<NCH>(a.ell, hsm, [&](int k, int64_t c) {
      return (RV && k < 2) ? S4 + c * 2 + k : Q4 + c;
    });
  }
  if (r >= a.n) return;
  const int64_t i = ell_node(a.ell, r);
  const int64_t base = a.ell.slice_off[r >> 5] + (r & 31);
  const int len = a.ell.row_len[r];
  const int hs = a.ell.halo_stride;
  float sx[V], sy[V], sl[V];
#pragma unroll
  for (int v = 0; v < V; ++v) { sx[v] = 0.f; sy[v] = 0.f; sl[v] = 0.f; }
#pragma unroll 4
  for (int j = 0; j < len; ++j) {
    const int64_t p = base + ((int64_t)j << 5);
    const int c = (HALO && staged) ? (int)__ldg(a.ell.lcol + p) : __ldg(a.ell.col + p);
    if (RV) {
      const float wx = __ldg(a.w32[0] + p), wy = __ldg(a.w32[1] + p);
      if (V == 4) {
        float4 xs, ys;
        if (HALO && staged) {
          xs = hsm[c];
          ys = hsm[hs + c];
        } else {
          const F8 st = ldg_f8(a.s32 + (int64_t)c * 8);
          xs = st.lo;
          ys = st.hi;
        }
        sx[0] = fmaf(wx, xs.x, sx[0]); sx[1] = fmaf(wx, xs.y, sx[1]);
        sx[2] = fmaf(wx, xs.z, sx[2]); sx[3] = fmaf(wx, xs.w, sx[3]);
        sy[0] = fmaf(wy, ys.x, sy[0]); sy[1] = fmaf(wy, ys.y, sy[1]);
        sy[2] = fmaf(wy, ys.z, sy[2]); sy[3] = fmaf(wy, ys.w, sy[3]);
      } else {
        const float2 s2 = __ldg(reinterpret_cast<const float2*>(a.s32) + c);
        sx[0] = fmaf(wx, s2.x, sx[0]);
        sy[0] = fmaf(wy, s2.y, sy[0]);
      }
    }
    if (LAP) {
      const float wl = __ldg(a.wl32 + p);
      if (V == 4) {
        const float4 qq = (HALO && staged)
                              ? hsm[(RV ? 2 : 0) * hs + c]
                              : __ldg(reinterpret_cast<const float4*>(a.q32) + c);
        sl[0] = fmaf(wl, qq.x, sl[0]); sl[1] = fmaf(wl, qq.y, sl[1]);
        sl[2] = fmaf(wl, qq.z, sl[2]); sl[3] = fmaf(wl, qq.w, sl[3]);
      } else {
        sl[0] = fmaf(wl, __ldg(a.q32 + c), sl[0]);
      }
    }
  }
  const float hg = a.hg32;
  float du[V];
  const float* dp32 = a.du_p32;
#pragma unroll
  for (int v = 0; v < V; ++v) {
    float d = dp32[i * V + v];
    if (RV) d = (d - sx[v]) - sy[v];
    if (LAP) d = fmaf(-hg, sl[v], d);
    if (a.hvf) d += fpconv::d2f(a.hvf[i * V + v]);
    du[v] = d;
  }
  if (a.final_epilogue) {
    double d[V];
#pragma unroll
    for (int v = 0; v < V; ++v) d[v] = fpconv::f2d(du[v]);
    finish_node<V>(a.ep, i, d);
  } else {
    float* out = a.du_p_out32;
#pragma unroll
    for (int v = 0; v < V; ++v) out[i * V + v] = du[v];
  }
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

void launch_fwd_f32(const FwdArgs& args, cudaStream_t s) {
  if (args.n <= 0) return;
  FwdArgs a = args;
  a.gm1_32 = (float)(a.gamma - 1.0);
  a.hg32 = (float)a.hv_gamma;
  MFT_REQUIRE(!(a.flyer && a.want_q), MFT_ERR_UNSUPPORTED,
              "Flyer and Tominec hyperviscosity together are not supported");
  const unsigned g = grid_for(a.n, kBlock);
  const bool wt = a.want_t != 0, wq = a.want_q != 0;
#define MFT_FWD32(WT, WQ, FLY)                                              \
  do {                                                                      \
    if (a.V == 4) k_fwd_euler_f32<WT, WQ, FLY><<<g, kBlock, 0, s>>>(a);     \
    else k_fwd_adv_f32<WT, WQ, FLY><<<g, kBlock, 0, s>>>(a);                \
  } while (0)
  if (a.flyer == 0) {
    if (wt && wq) MFT_FWD32(true, true, 0);
    else if (wt) MFT_FWD32(true, false, 0);
    else if (wq) MFT_FWD32(false, true, 0);
    else MFT_FWD32(false, false, 0);
  } else if (a.flyer == 1) {
    if (wt) MFT_FWD32(true, false, 1);
    else MFT_FWD32(false, false, 1);
  } else {
    if (wt) MFT_FWD32(true, false, 2);
    else MFT_FWD32(false, false, 2);
  }
#undef MFT_FWD32
  MFT_LAUNCH_CHECK();
}

bool launch_fwd_f32_halo(const FwdArgs& args, cudaStream_t s) {
  if (args.n <= 0) return true;
  if (args.V != 4 || !args.ell.halo_off) return false;
  FwdArgs a = args;
  a.gm1_32 = (float)(a.gamma - 1.0);
  a.hg32 = (float)a.hv_gamma;
  MFT_REQUIRE(!(a.flyer && a.want_q), MFT_ERR_UNSUPPORTED,
              "Flyer and Tominec hyperviscosity together are not supported");
  const int rows = a.ell.halo_rows;
  const unsigned g = grid_for(a.n, rows);
  const size_t smem = (size_t)a.ell.halo_stride * sizeof(float4);
  const bool wt = a.want_t != 0, wq = a.want_q != 0;
#define MFT_FWD32H(WT, WQ, FLY) k_fwd_euler_f32<WT, WQ, FLY, true><<<g, rows, smem, s>>>(a)
  if (a.flyer == 0) {
    if (wt && wq) MFT_FWD32H(true, true, 0);
    else if (wt) MFT_FWD32H(true, false, 0);
    else if (wq) MFT_FWD32H(false, true, 0);
    else MFT_FWD32H(false, false, 0);
  } else if (a.flyer == 1) {
    if (wt) MFT_FWD32H(true, false, 1);
    else MFT_FWD32H(false, false, 1);
  } else {
    if (wt) MFT_FWD32H(true, false, 2);
    else MFT_FWD32H(false, false, 2);
  }
#undef MFT_FWD32H
  MFT_LAUNCH_CHECK();
  return true;
}

void launch_eps_f32(const EpsArgs& a, cudaStream_t s) {
  if (a.n <= 0) return;
  if (a.V == 4) k_eps_f32<4><<<grid_for(a.n, kBlock), kBlock, 0, s>>>(a);
  else k_eps_f32<1><<<grid_for(a.n, kBlock), kBlock, 0, s>>>(a);
  MFT_LAUNCH_CHECK();
}

void launch_rev_f32(const RevArgs& args, cudaStream_t s) {
  if (args.n <= 0) return;
  RevArgs a = args;
  a.hg32 = (float)a.hv_gamma;
  const unsigned g = grid_for(a.n, kBlock);
  if (a.V == 4) {
    if (a.rv && a.lap) k_rev_f32<4, true, true><<<g, kBlock, 0, s>>>(a);
    else if (a.rv) k_rev_f32<4, true, false><<<g, kBlock, 0, s>>>(a);
    else if (a.lap) k_rev_f32<4, false, true><<<g, kBlock, 0, s>>>(a);
    else k_rev_f32<4, false, false><<<g, kBlock, 0, s>>>(a);
  } else {
    if (a.rv && a.lap) k_rev_f32<1, true, true><<<g, kBlock, 0, s>>>(a);
    else if (a.rv) k_rev_f32<1, true, false><<<g, kBlock, 0, s>>>(a);
    else if (a.lap) k_rev_f32<1, false, true><<<g, kBlock, 0, s>>>(a);
    else k_rev_f32<1, false, false><<<g, kBlock, 0, s>>>(a);
  }
  MFT_LAUNCH_CHECK();
}

bool launch_rev_f32_halo(const RevArgs& args, cudaStream_t s) {
  if (args.n <= 0) return true;
  if (args.V != 4 || !args.ell.halo_off) return false;
  RevArgs a = args;
  a.hg32 = (float)a.hv_gamma;
  const int rows = a.ell.halo_rows;
  const unsigned g = grid_for(a.n, rows);
  const size_t smem = (size_t)3 * a.ell.halo_stride * sizeof(float4);
  if (a.rv && a.lap) k_rev_f32<4, true, true, true><<<g, rows, smem, s>>>(a);
  else if (a.rv) k_rev_f32<4, true, false, true><<<g, rows, smem, s>>>(a);
  else if (a.lap) k_rev_f32<4, false, true, true><<<g, rows, smem, s>>>(a);
  else k_rev_f32<4, false, false, true><<<g, rows, smem, s>>>(a);
  MFT_LAUNCH_CHECK();
  return true;
}

}  // namespace mft
