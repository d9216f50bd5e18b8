// Device helpers shared by the FP64 and FP32 apply kernels.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "mft_fpbits.h"
#include "mft_internal.cuh"

namespace mft {
namespace dev {

constexpr int kBlock = 128;

static __device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
static __device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
static __device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
static __device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// One 32-byte read-only global load (the 256-bit vector load of sm_100 and later): both
// halves of a node's 8-float record in one request, so each cache line it touches is
// looked up once instead of once per 16-byte half.  p must be 32-byte aligned and the
// data must not change during the kernel.
struct F8 {
  float4 lo, hi;
};
static __device__ __forceinline__ F8 ldg_f8(const float* p) {
  F8 r;
  asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=f"(r.lo.x), "=f"(r.lo.y), "=f"(r.lo.z), "=f"(r.lo.w), "=f"(r.hi.x), "=f"(r.hi.y),
        "=f"(r.hi.z), "=f"(r.hi.w)
      : "l"(p));
  return r;
}

// Textbook Euler flux (Trixi's `flux(u, orientation, ::CompressibleEulerEquations2D)`),
// each operation rounded separately.
static __device__ __forceinline__ void euler_flux(double g, const double* uu, double* fx, double* fy) {
  const double rho = uu[0], m1 = uu[1], m2 = uu[2], en = uu[3];
  const double v1 = ddiv(m1, rho), v2 = ddiv(m2, rho);
  const double p = dmul(dsub(g, 1.0), dsub(en, dmul(0.5, dadd(dmul(m1, v1), dmul(m2, v2)))));
  fx[0] = m1;
  fx[1] = dadd(dmul(m1, v1), p);
  fx[2] = dmul(m1, v2);
  fx[3] = dmul(dadd(en, p), v1);
  fy[0] = m2;
  fy[1] = dmul(m2, v1);
  fy[2] = dadd(dmul(m2, v2), p);
  fy[3] = dmul(dadd(en, p), v2);
}

// Reverse-mode product of the Euler flux pair at state uu:
// ub = (dF/du)^T gx + (dG/du)^T gy for F = (m1, m1 v1 + p, m1 v2, (E + p) v1),
// G = (m2, m2 v1, m2 v2 + p, (E + p) v2), v = m / rho,
// p = (gamma - 1)(E - (m1 v1 + m2 v2) / 2).
static __device__ __forceinline__ void euler_flux_vjp(double g, const double* uu, const double* gx,
                                                      const double* gy, double* ub) {
  const double rho = uu[0], m1 = uu[1], m2 = uu[2], en = uu[3];
  const double ri = 1.0 / rho;
  const double v1 = m1 * ri, v2 = m2 * ri;
  const double gm1 = g - 1.0;
  const double p = gm1 * (en - 0.5 * (m1 * v1 + m2 * v2));
  const double ep = en + p;
  const double pb = gx[1] + gx[3] * v1 + gy[2] + gy[3] * v2;
  const double hp = 0.5 * gm1 * pb;
  const double v1b = gx[1] * m1 + gx[3] * ep + gy[1] * m2 - hp * m1;
  const double v2b = gx[2] * m1 + gy[2] * m2 + gy[3] * ep - hp * m2;
  ub[0] = -(v1b * v1 + v2b * v2) * ri;
  ub[1] = gx[0] + gx[1] * v1 + gx[2] * v2 - hp * v1 + v1b * ri;
  ub[2] = gy[0] + gy[1] * v1 + gy[2] * v2 - hp * v2 + v2b * ri;
  ub[3] = gx[3] * v1 + gy[3] * v2 + gm1 * pb;
}

// apply_slip_velocity (src/equations/PointCloudBCs.jl:15-21) with the normal
// normalised as boundary_condition_slip_wall does (:87-106).
static __device__ __forceinline__ void slip(const double* nrm, double* uu) {
  const double n1r = nrm[0], n2r = nrm[1];
  const double nn = sqrt(dadd(dmul(n1r, n1r), dmul(n2r, n2r)));
  const double n1 = ddiv(n1r, nn), n2 = ddiv(n2r, nn);
  const double vn = dadd(dmul(uu[1], n1), dmul(uu[2], n2));
  const double s1 = dsub(uu[1], dmul(vn, n1));
  const double s2 = dsub(uu[2], dmul(vn, n2));
  uu[1] = s1;
  uu[2] = s2;
}

// x / 3 correctly rounded without the division sequence: q = x * RN(1/3), the exact
// residual r = x - 3q by one fused multiply-add, then RN(q + r * RN(1/3)).  x / 3 is never
// a rounding midpoint (3 times a 54-bit odd significand needs more than 53 bits), and the
// corrected product equals IEEE x / 3.0 on 8e8 random doubles over the whole range.
static __device__ __forceinline__ double div3(double x) {
  const double c = 1.0 / 3.0;
  const double q = dmul(x, c);
  const double r = fma(-q, 3.0, x);
  return fma(r, c, q);
}

// BC pass 2 on du (and u at slip walls), then the stage epilogue.  Division by 4 is the
// exact product with 0.25; division by 3 is div3 (both equal IEEE division).
template <int V>
static __device__ __forceinline__ void finish_node(const Epilogue& ep, int64_t i, double* du) {
  if constexpr (V == 4) {
    if (ep.xadd) {
      du[1] = dadd(du[1], ep.xadd[i * 2]);
      du[2] = dadd(du[2], ep.xadd[i * 2 + 1]);
    }
  }
  double us[V];
#pragma unroll
  for (int v = 0; v < V; ++v) us[v] = ep.u_s[i * V + v];
  if (ep.has_bc) {
    const int tag = ep.bc.tag[i];
    if (tag == 1) {
#pragma unroll
      for (int v = 0; v < V; ++v) du[v] = 0.0;
    } else if (tag == 2 && V == 4) {
      du[1] = 0.0;
      du[2] = 0.0;
      slip(ep.bc.normal + 2 * (int64_t)ep.bc.slot[i], us);
      ep.u_s[i * V + 1] = us[1];
      ep.u_s[i * V + 2] = us[2];
    }
  }
  double o[V];
  if (ep.fused && ep.kind != kOutDu) {
    // FP32-apply form: u1 = us + dt du; u2 = (3 un + us)/4 + (dt/4) du;
    // u3 = un/3 + (2/3) us + (2dt/3) du as fused multiply-adds
#pragma unroll
    for (int v = 0; v < V; ++v) {
      if (ep.kind == kStage1) {
        o[v] = fma(ep.dt, du[v], us[v]);
      } else if (ep.kind == kStage2) {
        o[v] = fma(ep.cdt, du[v], fma(0.75, ep.u_n[i * V + v], 0.25 * us[v]));
      } else {
        o[v] = fma(ep.cdt, du[v], fma(2.0 / 3.0, us[v], ep.u_n[i * V + v] * (1.0 / 3.0)));
      }
    }
  } else switch (ep.kind) {
    case kOutDu:
#pragma unroll
      for (int v = 0; v < V; ++v) o[v] = du[v];
      break;
    case kStage1:
#pragma unroll
      for (int v = 0; v < V; ++v) o[v] = dadd(us[v], dmul(ep.dt, du[v]));
      break;
    case kStage2:
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const double un = ep.u_n[i * V + v];
        o[v] = dmul(dadd(dadd(dmul(3.0, un), us[v]), dmul(ep.dt, du[v])), 0.25);
      }
      break;
    default:
#pragma unroll
      for (int v = 0; v < V; ++v) {
        const double un = ep.u_n[i * V + v];
        o[v] = div3(dadd(dadd(un, dmul(2.0, us[v])), dmul(2.0 * ep.dt, du[v])));
      }
      break;
  }
  // non-finite outputs raise MFT_ERR_NONFINITE in the error word (the exponent field
  // of NaN and infinity is all ones; a rare atomic, no cost on the normal path)
  if (ep.err) {
    bool bad = false;
#pragma unroll
    for (int v = 0; v < V; ++v)
      bad |= ((__double_as_longlong(o[v]) >> 52) & 0x7FF) == 0x7FF;
    if (bad) atomicMax(ep.err, (int)MFT_ERR_NONFINITE);
  }
#pragma unroll
  for (int v = 0; v < V; ++v) ep.out[i * V + v] = o[v];
  if (ep.out32) {
#pragma unroll
    for (int v = 0; v < V; ++v) ep.out32[i * V + v] = fpconv::d2f(o[v]);
  }
}


// FP32 Euler flux divergence contribution of one neighbour state u with weights
// (wx, wy), in the form that needs no flux vector: with a = wx v1 + wy v2,
//   sum wx Fx + wy Fy = (rho a, m1 a + wx p, m2 a + wy p, (E + p) a).
// With WT the rho row is left to the caller (it equals tx[1] + ty[2]) and
// t = (wx u, wy u) is accumulated.  Shared by every FP32 gather variant so that they
// round identically.
template <bool WT>
static __device__ __forceinline__ void euler_accum_f32(float gm1, float4 u, float wx, float wy,
                                                       float* f, float* tx, float* ty) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(u.x));
  const float v1 = u.y * r, v2 = u.z * r;
  const float p = gm1 * fmaf(-0.5f, fmaf(u.z, v2, u.y * v1), u.w);
  const float a = fmaf(wx, v1, wy * v2);
  if (!WT) f[0] = fmaf(u.x, a, f[0]);
  f[1] = fmaf(u.y, a, fmaf(wx, p, f[1]));
  f[2] = fmaf(u.z, a, fmaf(wy, p, f[2]));
  f[3] = fmaf(u.w + p, a, f[3]);
  if (WT) {
    tx[0] = fmaf(wx, u.x, tx[0]); tx[1] = fmaf(wx, u.y, tx[1]);
    tx[2] = fmaf(wx, u.z, tx[2]); tx[3] = fmaf(wx, u.w, tx[3]);
    ty[0] = fmaf(wy, u.x, ty[0]); ty[1] = fmaf(wy, u.y, ty[1]);
    ty[2] = fmaf(wy, u.z, ty[2]); ty[3] = fmaf(wy, u.w, ty[3]);
  }
}

}  // namespace dev
}  // namespace mft
