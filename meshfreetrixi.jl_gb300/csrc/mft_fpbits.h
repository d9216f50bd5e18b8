// Exact float <-> double conversions on the integer pipe, for the double-word arithmetic.
//
// On this part the conversions between FP32 and FP64 run on the FP64 pipe, which issues at
// 1/74 of the FP32 rate.  Splitting an FP64 value into a double-word pair takes three of
// them and one subtraction; the staged forward gather that forms its neighbours' flux
// records splits four state values per record at the start of every block, where the
// block's FP64 work is not hidden behind other warps; the FP32-apply form converts its
// partial du to FP64 and every new state to its FP32 shadow in the stage epilogues.  Here
// the conversions are formed from the IEEE-754 bit fields with 32-bit integer operations
// (fpconv::f2d / d2f below, the same bits as the hardware conversions):
//   * float -> double is exact: the exponent is rebiased (127 -> 1023) and the 23-bit
//     significand moved to the top of the 52-bit one;
//   * double -> float rounds to nearest, ties to even: the 52-bit significand is cut to
//     23 bits, and one is added to the truncated bit pattern when the 29 dropped bits
//     exceed half an ulp, or equal it with the kept pattern odd; a carry out of the
//     significand moves into the exponent, and from the largest finite exponent into the
//     infinity pattern, which is the IEEE result in both cases.
// Each function handles the operands whose result is a normal number (and signed zeros)
// and returns false otherwise (subnormal results, infinities, NaN); the caller then uses
// the hardware conversion, so every input gets the IEEE result.  Plain C++ on 32-bit
// words: the same code compiles for the host, where a test checks it against the host's
// own conversions.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define MFT_FPBITS_FN __host__ __device__ __forceinline__
#else
#define MFT_FPBITS_FN static inline
#endif

namespace mft {
namespace fpbits {

// b: the bits of a float.  On success (*hi, *lo) are the high and low words of the
// double with the same value.
MFT_FPBITS_FN bool f2d_words(uint32_t b, uint32_t* hi, uint32_t* lo) {
  const uint32_t e = (b >> 23) & 0xFFu;
  if (e - 1u < 254u) {  // normal
    *hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b >> 3) & 0xFFFFFu);
    *lo = b << 29;
    return true;
  }
  if ((b << 1) == 0u) {  // +0 or -0
    *hi = b;
    *lo = 0u;
    return true;
  }
  return false;  // subnormal, infinity, NaN
}

// (hi, lo): the words of a double.  On success *out is the bits of the float nearest to
// it (ties to even).
MFT_FPBITS_FN bool d2f_bits(uint32_t hi, uint32_t lo, uint32_t* out) {
  const uint32_t e = (hi >> 20) & 0x7FFu;
  if (e - 897u < 254u) {  // the float exponent e - 896 is normal (1 .. 254)
    uint32_t r = ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
    const uint32_t rem = lo & 0x1FFFFFFFu;
    const uint32_t half = 0x10000000u;
    r += (rem > half || (rem == half && (r & 1u))) ? 1u : 0u;
    *out = r | (hi & 0x80000000u);
    return true;
  }
  if (((hi << 1) | lo) == 0u) {  // +0 or -0
    *out = hi;
    return true;
  }
  return false;  // below the normal floats, above them, infinity, NaN
}

}  // namespace fpbits

#if defined(__CUDACC__)
namespace fpconv {
// (double)f, exact, on the integer pipe where the result is normal or zero.
static __device__ __forceinline__ double f2d(float f) {
  uint32_t hi, lo;
  if (fpbits::f2d_words(__float_as_uint(f), &hi, &lo)) return __hiloint2double((int)hi, (int)lo);
  return (double)f;
}
// RN32(x), on the integer pipe where the result is a normal float or zero.
static __device__ __forceinline__ float d2f(double x) {
  uint32_t r;
  if (fpbits::d2f_bits((uint32_t)__double2hiint(x), (uint32_t)__double2loint(x), &r))
    return __uint_as_float(r);
  return __double2float_rn(x);
}
}  // namespace fpconv
#endif
}  // namespace mft

#undef MFT_FPBITS_FN
