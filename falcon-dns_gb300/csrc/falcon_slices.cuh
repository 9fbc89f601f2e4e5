// Device helpers shared by the integer-slice products (operator GEMMs in
// falcon_ozaki.cu, odd-prime DFT stages in falcon_fft.cuh): an FP64
// value cut into signed integers of a few bits relative to a power of two
// that bounds its row or column, their bf16 / fp16 encodings, the exact
// recombination, and the mma.sync used on them.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "falcon_combine.h"
#include "falcon_internal.h"

namespace falcon {
namespace {

__device__ __forceinline__ int biased_exp(double a) {
  return (int)((__double_as_longlong(a) >> 52) & 0x7ff);
}

__device__ __forceinline__ uint16_t bf16_bits_of_int(int q) {
  return __bfloat16_as_ushort(__float2bfloat16_rn((float)q));
}

// Slice formats of the operator GEMMs.  Width W bits per slice, S slices
// (MAGB = S W bits of each operand, relative to the power of two that
// bounds its row or column), the pairs s + t <= D summed per diagonal d in
// FP32, exact while K (D + 1 - ...) (2^W - 1)^2 < 2^24: W = 6 for K <= 257,
// W = 7 for K <= 112 (nine pairs per diagonal at most).  Recombination:
// sum_k a_k x_k = 2^(kH) H + 2^(kL) L with H = sum_{d<=HD} Q_d 2^(W(HD-d)),
// L = sum_{HD<d<=D} Q_d 2^(W(D-d)) (both exact in 64-bit integers) and
// kL = e_row + e_col - 2 MAGB + W (2S - 2 - D), kH = kL + W (D - HD).
template <int W> struct OzCfg;
template <> struct OzCfg<6> { static constexpr int S = 10, D = 9, HD = 4, MAGB = 60; };
template <> struct OzCfg<7> { static constexpr int S = 9, D = 8, HD = 3, MAGB = 63; };

// |a| * 2^(MAGB - e) truncated (< 2^MAGB when |a| < 2^e); zero and subnormal
// inputs give 0.
template <int MAGB>
__device__ __forceinline__ unsigned long long oz_magb(double a, int e) {
  const long long bits = __double_as_longlong(a);
  const int eb = (int)((bits >> 52) & 0x7ff);
  if (eb == 0) return 0ull;
  const unsigned long long m = (unsigned long long)(bits & 0xfffffffffffffLL) | (1ull << 52);
  const int sh = eb - 1075 + MAGB - e;  // <= MAGB - 53 because |a| < 2^e
  if (sh >= 0) return m << sh;
  if (sh <= -64) return 0ull;
  return m >> (-sh);
}

// Slice s (0 = most significant) of T in format W, with a sign, as bf16 bits.
template <int W>
__device__ __forceinline__ uint32_t oz_slice_w(unsigned long long T, bool neg, int s) {
  const int q = (int)((T >> (W * (OzCfg<W>::S - 1 - s))) & ((1u << W) - 1));
  return bf16_bits_of_int(neg ? -q : q);
}

// Slice s of two magnitudes (T0, T1 < 2^MAGB, each held as 32-bit halves
// lo:hi) in format W, as a bf16 pair with the signs sgn2 (bits 15 and 31):
// bf16(128 + q) has the bits 0x4300 + q for 0 <= q < 128, so one packed
// subtraction of 128 turns the two W-bit fields into bf16 (q0, q1) exactly.
// The same slices as oz_slice_w, except that a zero slice of a negative
// value is -0 instead of +0 (both give the same exact products and sums).
template <int W>
__device__ __forceinline__ uint32_t oz_slice_pair(uint32_t lo0, uint32_t hi0, uint32_t lo1, uint32_t hi1,
                                                  uint32_t sgn2, int s) {
  constexpr uint32_t mask = (1u << W) - 1;
  const int sh = W * (OzCfg<W>::S - 1 - s);
  uint32_t a, b;
  if (sh >= 32) {
    a = hi0 >> (sh - 32);
    b = hi1 >> (sh - 32);
  } else {
    a = __funnelshift_r(lo0, hi0, sh);
    b = __funnelshift_r(lo1, hi1, sh);
  }
  const uint32_t biased = ((a & mask) | ((b & mask) << 16)) | 0x43004300u;
  const __nv_bfloat162 v = __hsub2(*reinterpret_cast<const __nv_bfloat162*>(&biased),
                                   __floats2bfloat162_rn(128.f, 128.f));
  return *reinterpret_cast<const uint32_t*>(&v) ^ sgn2;
}

// The recombination of a slice product's two partial sums, H of the
// leading diagonals and L of the rest: RN(H 2^(k + sh) + L 2^k), each sum
// exact, one rounding: by integer instructions (combine_rn,
// falcon_combine.h) where the FP64 pipe bounds the kernel (the DFT stages),
// as two exact scalings and one FP64 add where it is idle (the
// contraction epilogues, which are bound by integer work).  The same bits.
__device__ __forceinline__ double oz_recombine_2t(long long H, long long L, int k, int sh) {
  return i64_scaled(H, k + sh) + i64_scaled(L, k);
}

// The exact integer sum of the diagonal sums: diag_sum (falcon_combine.h).
template <int W, int A, int B, class Q>
__device__ __forceinline__ long long oz_diag_sum(Q q) {
  return diag_sum<W, A, B>(q);
}

// fp16 slices of 9 bits for short sums (the DFT butterflies: at most 8
// products per output): kDftS slices of kDftW bits hold 63 bits of each
// operand, and the pairs s + t <= kDftD keep every FP32 sum exact
// (7 pairs x 8 products x 511^2 < 2^24) while the dropped pairs weigh less
// than 2^-59 of the largest product.
constexpr int kDftS = 7, kDftW = 9, kDftD = 6;

// |a| * 2^(63 - e) truncated (< 2^63 when |a| < 2^e); zero and subnormal
// inputs give 0.
__device__ __forceinline__ unsigned long long dft_mag(double a, int e) {
  const long long bits = __double_as_longlong(a);
  const int eb = (int)((bits >> 52) & 0x7ff);
  if (eb == 0) return 0ull;
  const unsigned long long m = (unsigned long long)(bits & 0xfffffffffffffLL) | (1ull << 52);
  const int sh = eb - 1012 - e;  // a = m 2^(eb-1075): T = m 2^(eb - 1075 + 63 - e), sh <= 10
  if (sh >= 0) return m << sh;
  if (sh <= -64) return 0ull;
  return m >> (-sh);
}

// Slice s (0 = most significant) of two values as an fp16 pair: fp16(1536 +
// q) has the bits 0x6600 + q for 0 <= q < 512, so q = fp16(0x6600 + q) -
// 1536 exactly; the signs (bits 15 and 31 of sgn) are applied to the result.
__device__ __forceinline__ uint32_t dft_slice2(unsigned long long tlo, unsigned long long thi, uint32_t sgn, int s) {
  const int sh = kDftW * (kDftS - 1 - s);
  const uint32_t biased = (((uint32_t)(tlo >> sh) & 511u) | (((uint32_t)(thi >> sh) & 511u) << 16)) + 0x66006600u;
  const __half2 v = __hsub2(*reinterpret_cast<const __half2*>(&biased), __floats2half2_rn(1536.f, 1536.f));
  return *reinterpret_cast<const uint32_t*>(&v) ^ sgn;
}

// The wider odd primes (h = (p-1)/2 up to 15 products per output): 8 slices
// of 8 bits (64 bits), pairs s + t <= 7 (8 pairs x 15 x 255^2 < 2^24).
constexpr int kDwS = 8, kDwW = 8, kDwD = 7;

// |a| * 2^(64 - e) truncated (< 2^64 when |a| < 2^e).
__device__ __forceinline__ unsigned long long dft_mag64(double a, int e) {
  const long long bits = __double_as_longlong(a);
  const int eb = (int)((bits >> 52) & 0x7ff);
  if (eb == 0) return 0ull;
  const unsigned long long m = (unsigned long long)(bits & 0xfffffffffffffLL) | (1ull << 52);
  const int sh = eb - 1011 - e;  // <= 11
  if (sh >= 0) return m << sh;
  if (sh <= -64) return 0ull;
  return m >> (-sh);
}

// Slice s of two 64-bit magnitudes in the 8-bit format as an fp16 pair
// (same construction as dft_slice2).
__device__ __forceinline__ uint32_t dft_slice2w(unsigned long long tlo, unsigned long long thi, uint32_t sgn, int s) {
  const int sh = kDwW * (kDwS - 1 - s);
  const uint32_t biased = (((uint32_t)(tlo >> sh) & 255u) | (((uint32_t)(thi >> sh) & 255u) << 16)) + 0x66006600u;
  const __half2 v = __hsub2(*reinterpret_cast<const __half2*>(&biased), __floats2half2_rn(1536.f, 1536.f));
  return *reinterpret_cast<const uint32_t*>(&v) ^ sgn;
}

__device__ __forceinline__ uint32_t sign2(double lo, double hi) {
  return (__double_as_longlong(lo) < 0 ? 0x8000u : 0u) | (__double_as_longlong(hi) < 0 ? 0x80000000u : 0u);
}

__device__ __forceinline__ void mma_f16(float (&c)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                        unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

}  // namespace
}  // namespace falcon
