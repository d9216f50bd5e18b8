// Viscosity of one node: update_upwind_visc!, update_residual_visc! and update_visc!
// (src/sources/hyperviscosity.jl:246-349).  Shared by the viscosity kernel (k_eps) and by
// the double-word forward gather, which forms it in its epilogue.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#include "mft_internal.cuh"

namespace mft {
namespace visc {

static __device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
static __device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
static __device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// Base.isless for Float64 (NaN above everything, -0.0 before +0.0)
static __device__ __forceinline__ int jl_isless(double a, double b) {
  if (isnan(a)) return 0;
  if (isnan(b)) return 1;
  if (a < b) return 1;
  if (a > b) return 0;
  return signbit(a) && !signbit(b);
}
static __device__ __forceinline__ double jl_min(double a, double b) {
  if (isnan(a) || isnan(b)) return a + b;
  return jl_isless(b, a) ? b : a;
}

// Julia's max for arguments that are +0 or larger, or NaN (NaN propagates as a + b):
// without NaN the larger value is the larger IEEE bit pattern, so no FP64 comparison
// is issued.
static __device__ __forceinline__ double jl_max_nonneg(double a, double b) {
  const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
  const long long inf = 0x7FF0000000000000LL;
  if ((ia & 0x7FFFFFFFFFFFFFFFLL) > inf || (ib & 0x7FFFFFFFFFFFFFFFLL) > inf) return a + b;
  return ib > ia ? b : a;
}

// isnan(x) || isinf(x) on the exponent bits
static __device__ __forceinline__ bool not_finite(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7FF) == 0x7FF;
}

// 1 / x within an ulp: an FP32 reciprocal estimate refined by two Newton steps
// y <- y + y (1 - x y) in FP64 fused multiply-adds (quadratic convergence from 2^-23:
// 2^-46, then below the final rounding).  Outside 1e-30 <= |x| <= 1e30 (the FP32 estimate
// could underflow or overflow) and for non-finite x it is the IEEE division.
static __device__ __forceinline__ double recip(double x) {
  const double ax = fabs(x);
  if (!(ax >= 1e-30 && ax <= 1e30)) return __ddiv_rn(1.0, x);
  float y0;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(__double2float_rn(x)));
  double y = (double)y0;
  y = fma(y, fma(-x, y, 1.0), y);
  y = fma(y, fma(-x, y, 1.0), y);
  return y;
}

// eps of node i.  dpv: the node's partial du (flux divergence [+ earlier sources]) when the
// caller has it in registers, or null to read it from a.du_p.
template <int V>
static __device__ __forceinline__ double eps_value(const EpsArgs& a, int64_t i,
                                                   const double* dpv_in) {
  const int sg = a.seg_id ? a.seg_id[i] : 0;
  const double h = a.seg_h ? a.seg_h[sg] : a.h;
  const double* __restrict__ norms = a.norms + (a.seg_id ? sg * 2 * V : 0);
  const int si = a.tab ? a.tab[*a.ctr].si_eps : a.success_iter;
  const bool rv = a.kind == MFT_SRC_RV && si != 0;
  double eps_rv = 0.0;
  bool rv_finite = false;
  if (rv) {
    // residual / norm with the norms' reciprocals (written by k_lexmax after the norms);
    // r >= 0 and the reciprocals are positive, so every qv is +0 or larger, or NaN
    double dpv[V], adv[V];
    if (V == 4) {
      const double2* ad2 = reinterpret_cast<const double2*>(a.approx_du) + i * 2;
      const double2 a0 = ad2[0], a1 = ad2[1];
      adv[0] = a0.x; adv[1 % V] = a0.y; adv[2 % V] = a1.x; adv[3 % V] = a1.y;
      if (dpv_in) {
#pragma unroll
        for (int v = 0; v < V; ++v) dpv[v] = dpv_in[v];
      } else {
        const double2* dp2 = reinterpret_cast<const double2*>(a.du_p) + i * 2;
        const double2 d0 = dp2[0], d1 = dp2[1];
        dpv[0] = d0.x; dpv[1 % V] = d0.y; dpv[2 % V] = d1.x; dpv[3 % V] = d1.y;
      }
    } else {
      dpv[0] = dpv_in ? dpv_in[0] : a.du_p[i];
      adv[0] = a.approx_du[i];
    }
    double mr = 0.0;
#pragma unroll
    for (int v = 0; v < V; ++v) {
      double dp = dpv[v];
      if (a.hvf) dp = dadd(dp, a.hvf[i * V + v]);
      const double r = fabs(dsub(adv[v], dp));
      const double qv = dmul(r, norms[V + v]);
      mr = v == 0 ? qv : jl_max_nonneg(mr, qv);
    }
    const double rvc = a.seg_h ? dmul(dmul(0.5, a.c_rv), dmul(h, h)) : a.rv_coef;
    eps_rv = dmul(rvc, mr);
    rv_finite = !not_finite(eps_rv);
  }
  double eps;
  double rho = 0.0, m1 = 0.0, m2 = 0.0, en = 0.0;
  if (V == 4) {
    const double2 ua = reinterpret_cast<const double2*>(a.u)[i * 2];
    const double2 ub = reinterpret_cast<const double2*>(a.u)[i * 2 + 1];
    rho = ua.x; m1 = ua.y; m2 = ub.x; en = ub.y;
  }
  const double uwc = a.seg_h ? dmul(dmul(a.c_uw, 0.5), h) : a.uw_coef;
  // Decided without forming eps_uw: speed + c >= sqrt(speed^2 + c^2), so in exact
  // arithmetic (rho eps_uw)^2 >= uwc^2 (|m|^2 + gamma p rho) with
  // p rho = (gamma - 1) (E rho - |m|^2 / 2).  The pressure term is counted only where
  // |m|^2 <= E rho: the difference then keeps at least half of E rho (a few ulps of
  // error), and p > 0, so the computed c is that of the formula; elsewhere the bound
  // uses the speed alone (c >= 0).  The computed eps_uw is within ~20 u of the exact one
  // (u = 2^-53), so (eps_rv rho)^2 < uwc^2 (1 - 1e-12) / (1 + 1e-12) w, evaluated in FP64
  // with a normal, finite right side, proves eps_rv < eps_uw and update_visc!'s min is
  // eps_rv.  This skips the reciprocal and the two square roots wherever the residual
  // viscosity is the smaller one (smooth flow, and still flow: with the sound speed in the
  // bound a node at rest qualifies too).  A NaN energy, or a density so small that
  // 1 / rho overflows (0 * inf in a velocity), would make eps_uw NaN: no shortcut then.
  // The final comparison is on bit patterns of values >= 0 (or NaN, which fails it).
  bool done = false;
  const double kb = a.seg_h ? dmul(dmul(uwc, uwc), (1.0 - 1e-12) / (1.0 + 1e-12)) : a.uw_bound;
  const long long bits_rho = __double_as_longlong(rho);
  const long long bits_en = __double_as_longlong(en) & 0x7FFFFFFFFFFFFFFFLL;
  if (V == 4 && rv_finite && bits_rho >= 0x01A56E1FC2F8F359LL /* 1e-300 */ &&
      __double_as_longlong(uwc) > 0 && bits_en <= 0x7FF0000000000000LL) {
    const double er = dmul(eps_rv, rho);
    const double lhs = dmul(er, er);
    const double mm = dadd(dmul(m1, m1), dmul(m2, m2));
    const double erho = dmul(en, rho);
    double w = mm;
    if (mm <= erho) w = dadd(mm, dmul(a.gg1, dsub(erho, dmul(0.5, mm))));
    const double rhs = dmul(kb, w);
    const long long bl = __double_as_longlong(lhs), br = __double_as_longlong(rhs);
    if (br >= 0x03B8F2B061AEA072LL /* 1e-290 */ && br <= 0x7FE0000000000000LL /* 2^1023 */ &&
        bl < br) {
      eps = eps_rv;
      done = true;
    }
  }
  if (!done) {
    double eps_uw;
    if (V == 4) {
      // one reciprocal instead of three divisions (FP64 division is a long sequence on
      // this part); results differ from the divisions by at most an ulp or two
      const double rinv = recip(rho);
      const double v1 = dmul(m1, rinv), v2 = dmul(m2, rinv);
      const double p =
          dmul(dsub(a.gamma, 1.0), dsub(en, dmul(0.5, dadd(dmul(m1, v1), dmul(m2, v2)))));
      const double speed = sqrt(dadd(dmul(v1, v1), dmul(v2, v2)));
      double c;
      if (p < 0.0 || rho < 0.0) c = 0.0;
      else c = sqrt(dmul(dmul(a.gamma, p), rinv));
      eps_uw = dmul(uwc, dadd(speed, c));
    } else if (a.seg_h) {
      const double an = sqrt(dadd(dmul(a.ax, a.ax), dmul(a.ay, a.ay)));
      eps_uw = dmul(uwc, an);
    } else {
      eps_uw = a.uw_adv;
    }
    if (rv) {
      if (!rv_finite) eps = not_finite(eps_uw) ? 2.220446049250313e-16 : eps_uw;
      else eps = jl_min(eps_rv, eps_uw);
    } else if (a.kind == MFT_SRC_RV) {
      // success_iter == 0: update_visc! takes eps_uw (or eps() when it is not finite)
      eps = not_finite(eps_uw) ? 2.220446049250313e-16 : eps_uw;
    } else {
      eps = eps_uw;
    }
  }
  return eps;
}

}  // namespace visc
}  // namespace mft
