// Double-word FP32 arithmetic ("double-float": a value is an unevaluated sum h + l of two
// floats with |l| <= ulp(h) / 2, 48 significand bits) for the FP64 form's gathers.
//
// On this part an FP64 fused multiply-add issues at 1/74 of the FP32 rate, and the FP64
// gathers are bound by it.  The sums of products those gathers form are evaluated here
// on the FP32 pipe with error-free transformations instead:
//   * the exact product of the high parts by an FMA:  p = RN(a_h b_h),
//     e = a_h b_h - p exactly = fma(a_h, b_h, -p)  (Dekker 1971, with an FMA);
//   * the cross terms a_h b_l + a_l b_h folded into e (a_l b_l < 2^-48 |ab| is dropped);
//   * the exact sum of the running high part and p by Knuth's TwoSum (branch-free),
//     whose rounding error joins e in a float carry.
// This is the compensated dot product "Dot2" of Ogita, Rump and Oishi (SIAM J. Sci.
// Comput. 26(6), 2005) on double-word inputs (Joldes, Muller and Popescu, ACM TOMS
// 44(2), 2017).  With u = 2^-24, a length-n sum of products carries the inputs' split
// error (< 3 u^2 sum |a_i b_i|) and the carry's own rounding, at most gamma_n^2
// sum |a_i b_i| with gamma_n = n u / (1 - n u) when every rounding error has the same
// sign and its largest size (n = 35: 4.4e-12 of the condition scale sum |a_i b_i|);
// errors of mixed sign give about sqrt(n) u^2 of it (~2e-14).  The result is rounded
// once to FP64.  Every operation is an explicitly rounded intrinsic, so no contraction
// or reassociation by the compiler can break the error-free steps.
#pragma once

#include <cuda_runtime.h>

#include "mft_fpbits.h"

namespace mft {
namespace dw {

using fpconv::d2f;
using fpconv::f2d;

// x -> (h, l): h = RN32(x), l = RN32(x - h) (x - h is exact in FP64).
static __device__ __forceinline__ float2 split(double x) {
  const float h = d2f(x);
  const float l = d2f(__dsub_rn(x, f2d(h)));
  return make_float2(h, l);
}

static __device__ __forceinline__ double value(float2 a) {
  return __dadd_rn(f2d(a.x), f2d(a.y));
}

// Running sum of products: s is the float running sum, c the float carry of every
// rounding error (products and sums).
struct Acc {
  float s, c;
};

static __device__ __forceinline__ Acc zero() { return Acc{0.f, 0.f}; }

// acc += a * b (a, b double-word)
static __device__ __forceinline__ void fma_acc(Acc& acc, float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  const float t = __fadd_rn(acc.s, p);
  const float bp = __fsub_rn(t, acc.s);
  const float err = __fadd_rn(__fsub_rn(acc.s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  acc.s = t;
  acc.c = __fadd_rn(acc.c, __fadd_rn(err, e));
}

// The accumulated value rounded once to FP64.
static __device__ __forceinline__ double to_double(const Acc& a) {
  return __dadd_rn(f2d(a.s), f2d(a.c));
}

// The accumulated value as a normalised double-word pair (TwoSum of s and c).
static __device__ __forceinline__ float2 to_pair(const Acc& a) {
  const float t = __fadd_rn(a.s, a.c);
  const float bp = __fsub_rn(t, a.s);
  const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bp)), __fsub_rn(a.c, bp));
  return make_float2(t, err);
}

// a * b for a double-word a and b, normalised (|e| <= ulp(p), so Fast2Sum is exact).
static __device__ __forceinline__ float2 mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  const float t = __fadd_rn(p, e);
  return make_float2(t, __fsub_rn(e, __fsub_rn(t, p)));
}

// a + b for double-word a and b: TwoSum of the high parts, the low parts added to its
// error, renormalised (absolute error about 2 u^2 (|a| + |b|)).
static __device__ __forceinline__ float2 add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bb = __fsub_rn(s, a.x);
  float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
  e = __fadd_rn(e, __fadd_rn(a.y, b.y));
  const float t = __fadd_rn(s, e);
  return make_float2(t, __fsub_rn(e, __fsub_rn(t, s)));
}

static __device__ __forceinline__ float2 neg(float2 a) { return make_float2(-a.x, -a.y); }

// a * 2^k for a power of two c = 2^k (exact)
static __device__ __forceinline__ float2 scale2(float2 a, float c) {
  return make_float2(__fmul_rn(a.x, c), __fmul_rn(a.y, c));
}

// 1 / a for a double-word a: the correctly rounded FP32 reciprocal y of a_h and one
// Newton step y + y (1 - a y) with 1 - a y formed exactly up to the low-order product
// (relative error about 2 u^2).
static __device__ __forceinline__ float2 recip(float2 a) {
  const float y = __frcp_rn(a.x);
  const float p = __fmul_rn(a.x, y);
  float ep = fmaf(a.x, y, -p);
  ep = fmaf(a.y, y, ep);
  const float d = __fsub_rn(__fsub_rn(1.0f, p), ep);
  const float c = __fmul_rn(y, d);
  const float t = __fadd_rn(y, c);
  return make_float2(t, __fsub_rn(c, __fsub_rn(t, y)));
}

// The Euler flux-Jacobian-transpose product ub = J_Fx(u)^T gx + J_Fy(u)^T gy (as
// euler_flux_vjp in FP64) in double-word arithmetic: u as pairs, gx / gy as pairs,
// gm1 = gamma - 1 as a pair; each operation is accurate to about 2 u^2 of its operands.
static __device__ __forceinline__ void euler_flux_vjp(float2 gm1, const float2* u,
                                                      const float2* gx, const float2* gy,
                                                      float2* ub) {
  const float2 rho = u[0], m1 = u[1], m2 = u[2], en = u[3];
  const float2 ri = recip(rho);
  const float2 v1 = mul(m1, ri), v2 = mul(m2, ri);
  const float2 p = mul(gm1, add(en, neg(scale2(add(mul(m1, v1), mul(m2, v2)), 0.5f))));
  const float2 ep = add(en, p);
  const float2 pb = add(add(gx[1], mul(gx[3], v1)), add(gy[2], mul(gy[3], v2)));
  const float2 hp = scale2(mul(gm1, pb), 0.5f);
  const float2 v1b = add(add(mul(gx[1], m1), mul(gx[3], ep)), add(mul(gy[1], m2), neg(mul(hp, m1))));
  const float2 v2b = add(add(mul(gx[2], m1), mul(gy[2], m2)), add(mul(gy[3], ep), neg(mul(hp, m2))));
  ub[0] = neg(mul(add(mul(v1b, v1), mul(v2b, v2)), ri));
  ub[1] = add(add(add(gx[0], mul(gx[1], v1)), add(mul(gx[2], v2), neg(mul(hp, v1)))), mul(v1b, ri));
  ub[2] = add(add(add(gy[0], mul(gy[1], v1)), add(mul(gy[2], v2), neg(mul(hp, v2)))), mul(v2b, ri));
  ub[3] = add(add(mul(gx[3], v1), mul(gy[3], v2)), mul(gm1, pb));
}

}  // namespace dw
}  // namespace mft
