// Recombination of exact integer-slice sums into one FP64 value, and the
// fixed-point conversions of the tensor-core DFT stages, with integer
// instructions only (GB300's FP64 pipe issues ~2 instructions per clock
// per SM, so one FP64 add per output of a tensor-core contraction or DFT
// stage costs as much as the rest of its epilogue).  Host and device: the
// CPU tests compile this header with g++ and check it bit for bit.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define FALCON_HD __host__ __device__ __forceinline__
#else
#define FALCON_HD inline
#endif

namespace falcon {

FALCON_HD int clz64(unsigned long long x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

FALCON_HD double double_of_bits(unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, sizeof d);
  return d;
#endif
}

// v 2^k for |v| < 2^53 built from its bits when the result is a normal
// number (exact), else from ldexp.
FALCON_HD double i64_scaled(long long v, int k) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = (unsigned long long)v & (1ull << 63);
  const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  const int lz = clz64(a);
  const long long ex = (long long)(63 - lz) + 1023 + k;
  if (ex < 1 || ex > 2046) return ldexp((double)v, k);
  const unsigned long long frac = ((a << lz) << 1) >> 12;
  return double_of_bits(sgn | ((unsigned long long)ex << 52) | frac);
}

// RN(H 2^(k + sh) + L 2^k) for |H|, |L| < 2^53 and 0 < sh < 40: the sum
// formed exactly as a 128-bit integer and rounded once to nearest even.
// With k >= -1022 and k + sh + 55 <= 1024 both terms and every nonzero sum
// are normal numbers, so this is bit for bit i64_scaled(H, k + sh) +
// i64_scaled(L, k) (two exact terms, one correctly rounded FP64 add); out
// of that range it returns exactly that two-term form.
FALCON_HD double combine_rn(long long H, long long L, int k, int sh) {
  if (k < -1022 || k + sh + 55 > 1024) return i64_scaled(H, k + sh) + i64_scaled(L, k);
  // S = H 2^sh + L in two's complement (hi:lo)
  const unsigned long long hl = (unsigned long long)H << sh;
  unsigned long long lo = hl + (unsigned long long)L;
  unsigned long long hi = (unsigned long long)(H >> (64 - sh)) + (L < 0 ? ~0ull : 0ull) + (lo < hl ? 1ull : 0ull);
  const bool neg = (long long)hi < 0;
  if (neg) {  // magnitude
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0ull ? 1ull : 0ull);
  }
  if (hi == 0ull && lo == 0ull) return 0.0;
  const int n = hi ? 128 - clz64(hi) : 64 - clz64(lo);  // bit length, <= 54 + sh < 94
  int e = n - 1 + k;                                     // exponent of the leading bit
  unsigned long long mant;
  if (n <= 53) {
    mant = lo << (53 - n);
  } else {
    const int s = n - 53;  // dropped bits, 1..40
    mant = (lo >> s) | (hi << (64 - s));
    const unsigned long long dropped = lo & ((1ull << s) - 1ull), half = 1ull << (s - 1);
    if (dropped > half || (dropped == half && (mant & 1ull))) {
      ++mant;
      if (mant == (1ull << 53)) {
        mant >>= 1;
        ++e;
      }
    }
  }
  return double_of_bits((neg ? (1ull << 63) : 0ull) | ((unsigned long long)(e + 1023) << 52) |
                        (mant & ((1ull << 52) - 1ull)));
}

FALCON_HD long long bits_of_double(double a) {
#ifdef __CUDA_ARCH__
  return __double_as_longlong(a);
#else
  long long b;
  memcpy(&b, &a, sizeof b);
  return b;
#endif
}

// a 2^(FB - e) truncated toward zero, as a signed integer, for |a| < 2^e
// (so below 2^FB in magnitude; FB <= 62); zero and subnormal a give 0.
// The fixed-point form of the DFT stages: every value of a butterfly at
// the scale of its largest, so sums and differences are exact integer adds.
template <int FB>
FALCON_HD long long fix_of(double a, int e) {
  const long long bits = bits_of_double(a);
  const int eb = (int)((bits >> 52) & 0x7ff);
  if (eb == 0) return 0;
  const unsigned long long m = (unsigned long long)(bits & 0xfffffffffffffLL) | (1ull << 52);
  const int sh = eb - 1075 + FB - e;  // <= FB - 53 because |a| < 2^e
  unsigned long long t;
  if (sh >= 0) t = m << sh;
  else if (sh <= -64) t = 0ull;
  else t = m >> (-sh);
  return bits < 0 ? -(long long)t : (long long)t;
}

// RN(v 2^k) for any 64-bit v (its two halves through combine_rn).
FALCON_HD double dbl_of_fix(long long v, int k) {
  return combine_rn(v >> 26, v & ((1LL << 26) - 1), k, 26);
}

// The exact integer sum_{d=A..B} q(d) 2^(W (B - d)) of the diagonal sums
// q(d) of a slice product (Horner's sum of its diagonals), two diagonals per
// 32-bit multiply-add: every |q(d)| is at most 9 x 112 x 127^2 (W = 7) or
// 10 x 272 x 63^2 (W = 6), so q(d) 2^W + q(d + 1) stays below 2^31.
template <int W, int A, int B, class Q>
FALCON_HD long long diag_sum(Q q) {
  long long s = 0;
#pragma unroll
  for (int d = A; d + 1 <= B; d += 2) s += (long long)(q(d) * (1 << W) + q(d + 1)) * (1LL << (W * (B - d - 1)));
  if constexpr (((B - A + 1) & 1) != 0) s += q(B);
  return s;
}

}  // namespace falcon
