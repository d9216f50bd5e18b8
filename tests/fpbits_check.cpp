// Host check of the integer float <-> double conversions (csrc/mft_fpbits.h) against the
// host's IEEE conversions: float -> double over every float bit pattern; double -> float
// over every double exponent and sign with random significands and the rounding edge cases
// (exact ties with the kept pattern odd and even, one below and above a tie, all ones).
// Where a function declines (returns false), its input must lie outside the range it
// handles (a float that is neither normal nor zero; a nonzero double whose exponent is
// outside the normal floats').  Prints one line per mismatch (at most 20) and
// "ok <counts>" when all agree; exit status 0 only then.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mft_fpbits.h"

using mft::fpbits::d2f_bits;
using mft::fpbits::f2d_words;

static uint64_t dbits(double x) { uint64_t b; memcpy(&b, &x, 8); return b; }
static uint32_t fbits(float x) { uint32_t b; memcpy(&b, &x, 4); return b; }
static double from_dbits(uint64_t b) { double x; memcpy(&x, &b, 8); return x; }
static float from_fbits(uint32_t b) { float x; memcpy(&x, &b, 4); return x; }

static uint64_t rng = 0x9E3779B97F4A7C15ull;
static uint64_t next() {  // xorshift64*
  rng ^= rng >> 12; rng ^= rng << 25; rng ^= rng >> 27;
  return rng * 2685821657736338717ull;
}

int main(int argc, char** argv) {
  const uint64_t stride = argc > 1 ? strtoull(argv[1], nullptr, 10) : 1;
  long bad = 0, f2d_done = 0, f2d_declined = 0, d2f_done = 0, d2f_declined = 0;
  // float -> double
  for (uint64_t k = 0; k < (1ull << 32); k += stride) {
    const uint32_t b = (uint32_t)k;
    uint32_t hi, lo;
    const float f = from_fbits(b);
    if (f2d_words(b, &hi, &lo)) {
      ++f2d_done;
      const uint64_t want = dbits((double)f);
      const uint64_t got = ((uint64_t)hi << 32) | lo;
      if (got != want && bad++ < 20)
        printf("f2d %08x: got %016llx want %016llx\n", b, (unsigned long long)got,
               (unsigned long long)want);
    } else {
      ++f2d_declined;
      if (isnormal(f) || f == 0.0f) {
        if (bad++ < 20) printf("f2d %08x declined a normal or zero float\n", b);
      }
    }
  }
  // double -> float
  const uint64_t half = 1ull << 28;
  const uint64_t tails[] = {0, 1, half - 1, half, half + 1, (1ull << 29) - 1};
  for (uint64_t e = 0; e < 2048; ++e) {
    for (uint64_t sgn = 0; sgn < 2; ++sgn) {
      for (int t = 0; t < 4000; ++t) {
        uint64_t m = next() & ((1ull << 52) - 1);
        if (t < 12) {  // the rounding edge cases, kept pattern even then odd
          m = (m & ~((1ull << 30) - 1)) | ((uint64_t)(t & 1) << 29) | tails[t >> 1];
        } else if (t < 14) {
          m = t == 12 ? 0 : (1ull << 52) - 1;
        }
        const uint64_t b = (sgn << 63) | (e << 52) | m;
        const double x = from_dbits(b);
        uint32_t got;
        if (d2f_bits((uint32_t)(b >> 32), (uint32_t)b, &got)) {
          ++d2f_done;
          const uint32_t want = fbits((float)x);
          if (got != want && bad++ < 20)
            printf("d2f %016llx: got %08x want %08x\n", (unsigned long long)b, got, want);
        } else {
          ++d2f_declined;
          const float want = (float)x;
          if ((isnormal(want) && e >= 897 && e <= 1150) || x == 0.0) {
            if (bad++ < 20)
              printf("d2f %016llx declined a normal-range or zero double\n",
                     (unsigned long long)b);
          }
        }
      }
    }
  }
  if (bad) {
    printf("%ld mismatches\n", bad);
    return 1;
  }
  printf("ok f2d %ld (declined %ld) d2f %ld (declined %ld)\n", f2d_done, f2d_declined,
         d2f_done, d2f_declined);
  return 0;
}
