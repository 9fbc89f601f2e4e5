// The azimuthal transforms and the nonlinear pass (Nr_maxLOOP,
// src/nonlin.F90:35-91): complex helpers, the odd-prime DFT coefficient
// tables, the FMA and tensor-core butterfly stages, the warp-per-line and
// block-per-line kernels and their launchers.  Included by one translation
// unit per largest radix class (falcon_fft7.cu, falcon_fft17.cu,
// falcon_fft31.cu), which compile in parallel; everything here has internal
// linkage, so each unit holds its own coefficient tables in constant memory
// (filled by init_dft_tables, falcon_kernels.cu, through each unit's
// init_dft_tables_<MAXP>).
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "falcon_internal.h"
#include "falcon_slices.cuh"

namespace falcon {
namespace {

// ---------------------------------------------------------------------------
// complex helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 w) {
  return make_double2(fma(a.x, w.x, -a.y * w.y), fma(a.x, w.y, a.y * w.x));
}

// ---------------------------------------------------------------------------
// Odd-prime DFT coefficient tables: kC<p>[i] = cos(2 pi i/p), kS<p>[i] =
// sin(2 pi i/p), filled from the host once per process.
// ---------------------------------------------------------------------------
template <int p> struct DftTab;
#define FALCON_DEF_TAB(p)                                                    \
  __constant__ double kC##p[p];                                              \
  __constant__ double kS##p[p];                                              \
  template <> struct DftTab<p> {                                             \
    __device__ static __forceinline__ double c(int i) { return kC##p[i]; }   \
    __device__ static __forceinline__ double s(int i) { return kS##p[i]; }   \
  };
FALCON_DEF_TAB(3)
FALCON_DEF_TAB(5)
FALCON_DEF_TAB(7)
FALCON_DEF_TAB(11)
FALCON_DEF_TAB(13)
FALCON_DEF_TAB(17)
FALCON_DEF_TAB(19)
FALCON_DEF_TAB(23)
FALCON_DEF_TAB(29)
FALCON_DEF_TAB(31)

template <int p>
static cudaError_t set_tab(const void* csym, const void* ssym) {
  double c[p], s[p];
  const double two_pi = 8.0 * atan(1.0);
  for (int i = 0; i < p; ++i) {
    c[i] = cos(two_pi * i / p);
    s[i] = sin(two_pi * i / p);
  }
  cudaError_t e = cudaMemcpyToSymbol(csym, c, sizeof(c));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(ssym, s, sizeof(s));
}

cudaError_t init_tables_here() {
  static std::atomic<bool> done[64];  // tables uploaded, per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && done[dev].load()) return cudaSuccess;
  cudaError_t e = cudaSuccess;
#define FALCON_SET(p) if (e == cudaSuccess) e = set_tab<p>(kC##p, kS##p);
  FALCON_SET(3) FALCON_SET(5) FALCON_SET(7) FALCON_SET(11) FALCON_SET(13)
  FALCON_SET(17) FALCON_SET(19) FALCON_SET(23) FALCON_SET(29) FALCON_SET(31)
#undef FALCON_SET
  // the copies may return before they land; the kernels reading the tables
  // run on non-blocking streams
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev].store(true);
  return e;
}

// Forward DFT of length p in registers: v_j <- sum_q v_q exp(-2 pi i j q/p)
// (radix 2, 4 and 6; odd primes go through dft_odd_store below).  Radix 6
// is the 6-point axis of a prime-factor plan, computed as a Good-Thomas
// 2 x 3: inputs n = (3 n1 + 2 n2) mod 6, two 3-point DFTs over n2 in the
// symmetric form of dft_odd_store (cos(2 pi/3) = -1/2 exactly), then
// y_k = W_0[k mod 3] +- W_1[k mod 3] with the sign (-1)^(k mod 2).
template <int p>
__device__ __forceinline__ void dft_small(double2 (&v)[p]) {
  if constexpr (p == 6) {
    const double c = -0.5, sn = DftTab<3>::s(1);
    double2 w0[3], w1[3];
    {
      const double2 v0 = v[0], a = cadd(v[2], v[4]), b = csub(v[2], v[4]);
      const double2 A = make_double2(fma(a.x, c, v0.x), fma(a.y, c, v0.y)), B = make_double2(b.x * sn, b.y * sn);
      w0[0] = cadd(v0, a); w0[1] = make_double2(A.x + B.y, A.y - B.x); w0[2] = make_double2(A.x - B.y, A.y + B.x);
    }
    {
      const double2 v0 = v[3], a = cadd(v[5], v[1]), b = csub(v[5], v[1]);
      const double2 A = make_double2(fma(a.x, c, v0.x), fma(a.y, c, v0.y)), B = make_double2(b.x * sn, b.y * sn);
      w1[0] = cadd(v0, a); w1[1] = make_double2(A.x + B.y, A.y - B.x); w1[2] = make_double2(A.x - B.y, A.y + B.x);
    }
    v[0] = cadd(w0[0], w1[0]); v[3] = csub(w0[0], w1[0]);
    v[4] = cadd(w0[1], w1[1]); v[1] = csub(w0[1], w1[1]);
    v[2] = cadd(w0[2], w1[2]); v[5] = csub(w0[2], w1[2]);
  } else if constexpr (p == 2) {
    double2 a = v[0], b = v[1];
    v[0] = cadd(a, b); v[1] = csub(a, b);
  } else {
    double2 t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    double2 t2 = cadd(v[1], v[3]), t3 = csub(v[1], v[3]);
    v[0] = cadd(t0, t2); v[2] = csub(t0, t2);
    v[1] = make_double2(t1.x + t3.y, t1.y - t3.x);
    v[3] = make_double2(t1.x - t3.y, t1.y + t3.x);
  }
}

// Odd-prime forward DFT in the symmetric form
//   y_0 = v_0 + sum a_q,  y_j = A_j - i B_j,  y_{p-j} = A_j + i B_j,
//   a_q = v_q + v_{p-q}, b_q = v_q - v_{p-q}, A_j = v_0 + sum a_q cos(2 pi jq/p),
//   B_j = sum b_q sin(2 pi jq/p),
// with each output pair multiplied by its twiddle (DIF) and stored as soon
// as it is formed, so only a, b stay live.
template <int p>
__device__ __forceinline__ void dft_odd_store(double2 (&v)[p], double2* __restrict__ dst, int base, int m,
                                              const double2* __restrict__ tw, int ks, bool post_tw) {
  constexpr int h = (p - 1) / 2;
  double2 a[h], b[h];
#pragma unroll
  for (int q = 1; q <= h; ++q) { a[q - 1] = cadd(v[q], v[p - q]); b[q - 1] = csub(v[q], v[p - q]); }
  const double2 v0 = v[0];
  double2 y0 = v0;
#pragma unroll
  for (int q = 0; q < h; ++q) y0 = cadd(y0, a[q]);
  dst[base] = y0;
#pragma unroll
  for (int j = 1; j <= h; ++j) {
    double2 A = v0;
    double2 Bv = make_double2(0.0, 0.0);
#pragma unroll
    for (int q = 1; q <= h; ++q) {
      const int idx = (j * q) % p;
      const double c = DftTab<p>::c(idx), s = DftTab<p>::s(idx);
      A.x = fma(a[q - 1].x, c, A.x); A.y = fma(a[q - 1].y, c, A.y);
      Bv.x = fma(b[q - 1].x, s, Bv.x); Bv.y = fma(b[q - 1].y, s, Bv.y);
    }
    double2 yj = make_double2(A.x + Bv.y, A.y - Bv.x);
    double2 yk = make_double2(A.x - Bv.y, A.y + Bv.x);
    if (post_tw) {
      yj = cmul(yj, tw[j * ks]);
      yk = cmul(yk, tw[(p - j) * ks]);
    }
    dst[base + j * m] = yj;
    dst[base + (p - j) * m] = yk;
  }
}

// One in-place stage of radix p and span m on NB (1 or 2) buffers, its
// butterflies shared by nl cooperating lanes (lane < nl).
// DIT (dif = false): twiddles exp(-2 pi i q k / (m p)) on the inputs; DIF:
// on the outputs; none for the prime-factor plan (twid = false).
// tw[k] = exp(-2 pi i k / P); stride = P / (m p).
template <int p, int NB>
__device__ __forceinline__ void fft_stage(double2* __restrict__ A, double2* __restrict__ Bf, int P, int m,
                                          int stride, const double2* __restrict__ tw, int lane, int nl, bool dif,
                                          bool twid) {
  const int mp = m * p, nb = P / p;
  const float inv_m = 1.0f / (float)m;
  for (int t = lane; t < nb; t += nl) {
    const int g = (int)(((float)t + 0.5f) * inv_m);
    const int k = t - g * m;
    const int base = g * mp + k;
    const bool tk = twid && k > 0;
    const int ks = k * stride;
    double2 va[p], vb[p];
#pragma unroll
    for (int q = 0; q < p; ++q) {
      va[q] = A[base + q * m];
      if (NB == 2) vb[q] = Bf[base + q * m];
    }
    if (tk && !dif) {
#pragma unroll
      for (int q = 1; q < p; ++q) {
        const double2 w = tw[q * ks];
        va[q] = cmul(va[q], w);
        if (NB == 2) vb[q] = cmul(vb[q], w);
      }
    }
    if constexpr (p == 2 || p == 4 || p == 6) {
      dft_small<p>(va);
      if (NB == 2) dft_small<p>(vb);
      if (tk && dif) {
#pragma unroll
        for (int q = 1; q < p; ++q) {
          const double2 w = tw[q * ks];
          va[q] = cmul(va[q], w);
          if (NB == 2) vb[q] = cmul(vb[q], w);
        }
      }
#pragma unroll
      for (int q = 0; q < p; ++q) {
        A[base + q * m] = va[q];
        if (NB == 2) Bf[base + q * m] = vb[q];
      }
    } else {
      dft_odd_store<p>(va, A, base, m, tw, ks, tk && dif);
      if (NB == 2) dft_odd_store<p>(vb, Bf, base, m, tw, ks, tk && dif);
    }
  }
}

// Generic prime radix (p <= 64) with coefficients read from the P-point
// twiddle table: exp(-2 pi i j/p) = tw[j * P/p].  Bf may be null (one buffer).
__device__ void generic_stage(double2* A, double2* Bf, int P, int p, int m, int stride,
                              const double2* tw, int lane, int nl, bool dif, bool twid) {
  const int mp = m * p, nb = P / p, tp = P / p;
  double2* B2 = Bf ? Bf : A;  // with one buffer the second transform is a repeat, not stored
  for (int t = lane; t < nb; t += nl) {
    const int g = t / m, k = t - g * m, base = g * mp + k;
    double2 va[64], vb[64], ya[64], yb[64];
    for (int q = 0; q < p; ++q) { va[q] = A[base + q * m]; vb[q] = B2[base + q * m]; }
    if (twid && !dif && k > 0)
      for (int q = 1; q < p; ++q) { double2 w = tw[q * k * stride]; va[q] = cmul(va[q], w); vb[q] = cmul(vb[q], w); }
    for (int j = 0; j < p; ++j) {
      double2 sa = make_double2(0, 0), sb = make_double2(0, 0);
      for (int q = 0; q < p; ++q) {
        double2 w = tw[((j * q) % p) * tp];
        sa = cadd(sa, cmul(va[q], w)); sb = cadd(sb, cmul(vb[q], w));
      }
      ya[j] = sa; yb[j] = sb;
    }
    if (twid && dif && k > 0)
      for (int q = 1; q < p; ++q) { double2 w = tw[q * k * stride]; ya[q] = cmul(ya[q], w); yb[q] = cmul(yb[q], w); }
    for (int q = 0; q < p; ++q) {
      A[base + q * m] = ya[q];
      if (Bf) Bf[base + q * m] = yb[q];
    }
  }
}

template <int p>
__device__ void dft_mma_stage(double2* A, double2* Bf, int P, int m, int lane, int warp, int nw);
template <int p>
__device__ void dft_mma_stage_wide(double2* A, double2* Bf, int P, int m, int lane, int warp, int nw);

// MAXP bounds the radices compiled into one kernel instance, so a plan
// with small radices is not held to the register budget of radix 31.
template <int MAXP>
__device__ __forceinline__ void run_stage(int p, bool dif, bool twid, double2* A, double2* Bf, int P, int m,
                                          int stride, const double2* tw, int lane) {
  // two buffers interleaved up to radix 7; one at a time above, to bound
  // the live registers of the butterfly
#define FALCON_CASE2(q) case q: fft_stage<q, 2>(A, Bf, P, m, stride, tw, lane, 32, dif, twid); return;
#define FALCON_CASE1(q)                                                      \
  case q:                                                                    \
    if constexpr (q <= MAXP) {                                               \
      fft_stage<q, 1>(A, nullptr, P, m, stride, tw, lane, 32, dif, twid);    \
      fft_stage<q, 1>(Bf, nullptr, P, m, stride, tw, lane, 32, dif, twid);   \
      return;                                                                \
    }                                                                        \
    break;
  if constexpr (MAXP == 31) {  // the wide primes of prime-factor plans on the tensor cores
    if (!twid && (p == 19 || p == 23 || p == 29 || p == 31)) {
      if (p == 19) dft_mma_stage_wide<19>(A, Bf, P, m, lane, 0, 1);
      else if (p == 23) dft_mma_stage_wide<23>(A, Bf, P, m, lane, 0, 1);
      else if (p == 29) dft_mma_stage_wide<29>(A, Bf, P, m, lane, 0, 1);
      else dft_mma_stage_wide<31>(A, Bf, P, m, lane, 0, 1);
      return;
    }
  }
  if constexpr (MAXP == 17) {  // plans with a prime above 17 keep the FMA butterflies
    if (!twid && (p == 11 || p == 13 || p == 17)) {
      if (p == 11) dft_mma_stage<11>(A, Bf, P, m, lane, 0, 1);
      else if (p == 13) dft_mma_stage<13>(A, Bf, P, m, lane, 0, 1);
      else dft_mma_stage<17>(A, Bf, P, m, lane, 0, 1);
      return;
    }
  }
  switch (p) {
    FALCON_CASE2(2) FALCON_CASE2(3) FALCON_CASE2(4) FALCON_CASE2(5) FALCON_CASE2(6) FALCON_CASE2(7)
    FALCON_CASE1(11) FALCON_CASE1(13) FALCON_CASE1(17)
    FALCON_CASE1(19) FALCON_CASE1(23) FALCON_CASE1(29) FALCON_CASE1(31)
    default: break;
  }
#undef FALCON_CASE1
#undef FALCON_CASE2
  generic_stage(A, Bf, P, p, m, stride, tw, lane, 32, dif, twid);
}

// One buffer, its butterflies shared by nl lanes (the block-per-line form).
template <int MAXP>
__device__ __forceinline__ void run_stage1(int p, bool dif, bool twid, double2* A, int P, int m, int stride,
                                           const double2* tw, int lane, int nl) {
#define FALCON_CASE(q)                                                   \
  case q:                                                                \
    if constexpr (q <= MAXP) {                                           \
      fft_stage<q, 1>(A, nullptr, P, m, stride, tw, lane, nl, dif, twid); \
      return;                                                            \
    }                                                                    \
    break;
  switch (p) {
    FALCON_CASE(2) FALCON_CASE(3) FALCON_CASE(4) FALCON_CASE(5) FALCON_CASE(6) FALCON_CASE(7)
    FALCON_CASE(11) FALCON_CASE(13) FALCON_CASE(17) FALCON_CASE(19) FALCON_CASE(23)
    FALCON_CASE(29) FALCON_CASE(31)
    default: break;
  }
#undef FALCON_CASE
  generic_stage(A, nullptr, P, p, m, stride, tw, lane, nl, dif, twid);
}

// Odd prime p >= 17 of a prime-factor plan (no twiddles) on both buffers
// of a block at once, the output pairs of each butterfly shared by G lanes:
// with one thread per butterfly the stage would run a few dozen long
// butterflies on a few warps.  Work items are ordered lane group first, so
// a warp's lanes share their lane group (uniform coefficient loads).  Each
// output is formed with exactly the operations of dft_odd_store, so the
// results are bit for bit those of the one-thread form.  In place: every
// item loads its inputs before any item of the round stores.
template <int p, int G>
__device__ void fft_stage_split(double2* A, double2* Bf, int P, int m, int tid, int nt) {
  constexpr int h = (p - 1) / 2;
  const int nb = P / p, mp = m * p, items = 2 * nb * G;
  const int rounds = (items + nt - 1) / nt;
  const float inv_m = 1.0f / (float)m;
  for (int rd = 0; rd < rounds; ++rd) {
    const int it = rd * nt + tid;
    const bool act = it < items;
    int jg = 0, base = 0;
    double2* buf = A;
    double2 v[p];
    if (act) {
      jg = it / (2 * nb);
      const int rem = it - jg * 2 * nb;
      const int bsel = rem >= nb;
      const int t = rem - bsel * nb;
      buf = bsel ? Bf : A;
      const int g = (int)(((float)t + 0.5f) * inv_m);
      base = g * mp + (t - g * m);
#pragma unroll
      for (int q = 0; q < p; ++q) v[q] = buf[base + q * m];
    }
    __syncthreads();
    if (act) {
      double2 a[h], b[h];
#pragma unroll
      for (int q = 1; q <= h; ++q) { a[q - 1] = cadd(v[q], v[p - q]); b[q - 1] = csub(v[q], v[p - q]); }
      const double2 v0 = v[0];
      if (jg == 0) {
        double2 y0 = v0;
#pragma unroll
        for (int q = 0; q < h; ++q) y0 = cadd(y0, a[q]);
        buf[base] = y0;
      }
      for (int j = 1 + jg; j <= h; j += G) {
        double2 Av = v0;
        double2 Bv = make_double2(0.0, 0.0);
#pragma unroll
        for (int q = 1; q <= h; ++q) {
          const int idx = (j * q) % p;
          const double c = DftTab<p>::c(idx), sn = DftTab<p>::s(idx);
          Av.x = fma(a[q - 1].x, c, Av.x); Av.y = fma(a[q - 1].y, c, Av.y);
          Bv.x = fma(b[q - 1].x, sn, Bv.x); Bv.y = fma(b[q - 1].y, sn, Bv.y);
        }
        buf[base + j * m] = make_double2(Av.x + Bv.y, Av.y - Bv.x);
        buf[base + (p - j) * m] = make_double2(Av.x - Bv.y, Av.y + Bv.x);
      }
    }
    __syncthreads();
  }
}

// Odd-prime stage (p = 11, 13, 17, so h = (p - 1)/2 <= 8) of a prime-factor
// plan on the fp16 tensor cores, in fixed point: no FP64 arithmetic.  The
// symmetric butterfly of dft_odd_store,
//   y_0 = v_0 + sum a_q,  y_j = A_j - i B_j,  y_{p-j} = A_j + i B_j,
//   A_j = v_0 + sum_q a_q cos(2 pi jq/p),  B_j = sum_q b_q sin(2 pi jq/p),
//   a_q = v_q + v_{p-q},  b_q = v_q - v_{p-q},
// with every value of a butterfly (both components) as an integer at the
// scale of its largest, 2^e: V = trunc(v 2^(kDftFB - e)), |V| < 2^58.  The
// pre-adds and the y_0 sum are then exact 64-bit integer adds (|y_0| <
// 2^63), and A_j, B_j come from one product of the block-diagonal [C 0; 0 S]
// (rows j; K = the h values a_q, then the h values b_q) with a column per
// component: one m16n8k16 MMA per slice pair takes 8 columns, 4
// butterflies x (re, im).  The coefficients (|cos|, |sin| < 1) and the
// integers 2^4 a, 2^4 b (< 2^63) are cut into kDftS = 7 signed 9-bit slices
// (fp16 holds them exactly), and the 28 pairs s + t <= 6 are summed in
// FP32: at most 8 products per output keep every sum exact (7 pairs x 8
// products x 511^2 < 2^24).  The diagonal sums give A_j - v_0 and B_j as
// exact integers H 2^36 + L in units of 2^(e - 71); v_0 and the output
// pairs A_j +- i B_j are added in those integers and each output is
// rounded once to FP64 (combine_rn).  Errors: the inputs' truncation
// (2^(e - 58) each), the dropped pairs (below 2^(e - 56) per output) and the
// final rounding; a butterfly with an Inf or NaN gives NaN.  A butterfly's
// outputs depend only on its inputs, so any tiling (warp or block form)
// gives the same bits.  Lane (g, t) of a tile holds v_q, v_{p-q} for q =
// 2t + 1, 2t + 2 and v_0 of column g, and receives A_{g+1}, B_{g+1} of
// butterfly t, re and im, from which it stores y_j and y_{p-j}.  Tiles over
// both buffers go to warps warp, warp + nw, ...; the caller synchronises
// before (inputs complete) and after (outputs stored).
constexpr int kDftFB = 58;

template <int p>
__device__ void dft_mma_stage(double2* A, double2* Bf, int P, int m, int lane, int warp, int nw) {
  constexpr int h = (p - 1) / 2;
  static_assert(h <= 8, "the block-diagonal form holds h <= 8");
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int UP = 63 - (kDftFB + 1);  // |a|, |b| < 2^(kDftFB + 1): 2^UP |a| < 2^63
  const int gid = lane >> 2, tig = lane & 3;
  const int nb = P / p, mp = m * p, nbt = 2 * nb, ntile = (nbt + 3) / 4;
  const float inv_m = 1.0f / (float)m;
  const int q1 = 2 * tig + 1, q2 = 2 * tig + 2;  // K rows 2t, 2t + 1 (a) and 2t + 8, 2t + 9 (b)
  const bool has1 = q1 <= h, has2 = q2 <= h;
  // coefficient fragments: a0 = C(row g; q1, q2), a3 = S(row g; q1, q2), j = g + 1,
  // as 63-bit fractions (every |cos|, |sin| here is below 1)
  uint32_t fc[kDftS], fs[kDftS];
  {
    const int j = gid + 1;
    double c1 = 0.0, c2 = 0.0, s1 = 0.0, s2 = 0.0;
    if (j <= h) {
      if (has1) { c1 = DftTab<p>::c((j * q1) % p); s1 = DftTab<p>::s((j * q1) % p); }
      if (has2) { c2 = DftTab<p>::c((j * q2) % p); s2 = DftTab<p>::s((j * q2) % p); }
    }
    const unsigned long long tc1 = dft_mag(c1, 0), tc2 = dft_mag(c2, 0), ts1 = dft_mag(s1, 0), ts2 = dft_mag(s2, 0);
    const uint32_t sc = sign2(c1, c2), ss = sign2(s1, s2);
#pragma unroll
    for (int sl = 0; sl < kDftS; ++sl) {
      fc[sl] = dft_slice2(tc1, tc2, sc, sl);
      fs[sl] = dft_slice2(ts1, ts2, ss, sl);
    }
  }
  for (int tile = warp; tile < ntile; tile += nw) {
    // column g: butterfly bi (over both buffers), component g & 1
    const int bi = tile * 4 + (gid >> 1), comp = gid & 1;
    double x1 = 0.0, y1 = 0.0, x2 = 0.0, y2 = 0.0, v0 = 0.0;
    double* pi = nullptr;
    if (bi < nbt) {
      const int sel = bi >= nb, t = bi - sel * nb;
      const int g = (int)(((float)t + 0.5f) * inv_m);
      pi = reinterpret_cast<double*>((sel ? Bf : A) + g * mp + (t - g * m)) + comp;
      if (has1) { x1 = pi[2 * q1 * m]; y1 = pi[2 * (p - q1) * m]; }
      if (has2) { x2 = pi[2 * q2 * m]; y2 = pi[2 * (p - q2) * m]; }
      v0 = pi[0];
    }
    // the butterfly's exponent: |v| < 2^e over its 2p values (8 lanes)
    int fb = max(max(max(biased_exp(x1), biased_exp(y1)), max(biased_exp(x2), biased_exp(y2))), biased_exp(v0));
    fb = max(fb, __shfl_xor_sync(FULL, fb, 1));
    fb = max(fb, __shfl_xor_sync(FULL, fb, 2));
    fb = max(fb, __shfl_xor_sync(FULL, fb, 4));
    const int e = fb - 1022;
    const long long X1 = fix_of<kDftFB>(x1, e), Y1 = fix_of<kDftFB>(y1, e), X2 = fix_of<kDftFB>(x2, e),
                    Y2 = fix_of<kDftFB>(y2, e), V0 = fix_of<kDftFB>(v0, e);
    const long long a1 = X1 + Y1, b1 = X1 - Y1, a2 = X2 + Y2, b2 = X2 - Y2;
    // y_0 = v_0 + sum_q a_q per component (the same sum on the four lanes)
    long long ys = a1 + a2;
    ys += __shfl_xor_sync(FULL, ys, 1);
    ys += __shfl_xor_sync(FULL, ys, 2);
    uint32_t fa[kDftS], fbq[kDftS];
    {
      const unsigned long long ta1 = (unsigned long long)(a1 < 0 ? -a1 : a1) << UP,
                               ta2 = (unsigned long long)(a2 < 0 ? -a2 : a2) << UP,
                               tb1 = (unsigned long long)(b1 < 0 ? -b1 : b1) << UP,
                               tb2 = (unsigned long long)(b2 < 0 ? -b2 : b2) << UP;
      const uint32_t sa = (a1 < 0 ? 0x8000u : 0u) | (a2 < 0 ? 0x80000000u : 0u);
      const uint32_t sb = (b1 < 0 ? 0x8000u : 0u) | (b2 < 0 ? 0x80000000u : 0u);
#pragma unroll
      for (int sl = 0; sl < kDftS; ++sl) {
        fa[sl] = dft_slice2(ta1, ta2, sa, sl);
        fbq[sl] = dft_slice2(tb1, tb2, sb, sl);
      }
    }
    __syncwarp();  // every load of the tile precedes its stores
    if (tig == 0 && pi)
      pi[0] = fb == 2047 ? __longlong_as_double(0x7ff8000000000000LL) : dbl_of_fix(V0 + ys, e - kDftFB);
    float acc[kDftD + 1][4];
#pragma unroll
    for (int d = 0; d <= kDftD; ++d)
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[d][i] = 0.f;
#pragma unroll
    for (int sl = 0; sl < kDftS; ++sl)
#pragma unroll
      for (int t = 0; t < kDftS && sl + t <= kDftD; ++t) mma_f16(acc[sl + t], fc[sl], 0u, 0u, fs[sl], fa[t], fbq[t]);
    // this lane's butterfly bo: its exponent and v_0 (lanes 8t, 8t + 4 loaded them)
    const int bo = tile * 4 + tig;
    const int eo = __shfl_sync(FULL, e, 8 * tig);
    const long long w_re = __shfl_sync(FULL, V0, 8 * tig), w_im = __shfl_sync(FULL, V0, 8 * tig + 4);
    if (gid < h && bo < nbt) {
      const int sel = bo >= nb, t = bo - sel * nb;
      const int g = (int)(((float)t + 0.5f) * inv_m);
      double2* po = (sel ? Bf : A) + g * mp + (t - g * m);
      // (A_j - v_0).re, .im, B_j.re, .im = 2^(e - 71) (H 2^36 + L),
      // H = sum_{d<=2} Q_d 512^(2-d), L = sum_{d=3..6} Q_d 512^(6-d)
      long long H[4], L[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        H[i] = ((long long)__float2int_rn(acc[0][i]) << 18) + ((long long)__float2int_rn(acc[1][i]) << 9) +
               __float2int_rn(acc[2][i]);
        L[i] = ((long long)__float2int_rn(acc[3][i]) << 27) + ((long long)__float2int_rn(acc[4][i]) << 18) +
               ((long long)__float2int_rn(acc[5][i]) << 9) + __float2int_rn(acc[6][i]);
      }
      // v_0 (units 2^(e - 58)) in the same integers: 2^13 V = (V >> 23) 2^36 + (V mod 2^23) 2^13
      const long long hr = H[0] + (w_re >> 23), lr = L[0] + ((w_re & ((1LL << 23) - 1)) << 13);
      const long long hi = H[1] + (w_im >> 23), li = L[1] + ((w_im & ((1LL << 23) - 1)) << 13);
      const int k = eo - 71;
      double2 yj = make_double2(combine_rn(hr + H[3], lr + L[3], k, 36), combine_rn(hi - H[2], li - L[2], k, 36));
      double2 yk = make_double2(combine_rn(hr - H[3], lr - L[3], k, 36), combine_rn(hi + H[2], li + L[2], k, 36));
      if (eo == 2047 - 1022) {  // Inf or NaN in the butterfly
        yj = make_double2(__longlong_as_double(0x7ff8000000000000LL), __longlong_as_double(0x7ff8000000000000LL));
        yk = yj;
      }
      const int j = gid + 1;
      po[j * m] = yj;
      po[(p - j) * m] = yk;
    }
  }
}

// Wide odd-prime stage (p = 19, 23, 29, 31: h = 9..15) of a prime-factor
// plan on the fp16 tensor cores: the fixed-point butterfly of
// dft_mma_stage (integers |V| < 2^57, |y_0| < 2^63 for h <= 15) with the
// cos and sin products as two 16 x 16 tiles (rows j, K = q, padded), 8
// signed 8-bit slices of the coefficients and of 2^6 a, 2^6 b (64 bits)
// and the 36 pairs s + t <= 7 per tile; at most 15 products per output keep
// every FP32 sum exact (8 pairs x 15 x 255^2 < 2^24).  Lane (g, t) holds
// v_q, v_{p-q} for q = 2t + 1, 2t + 2, 2t + 9, 2t + 10 of column g and
// receives A_j, B_j for j = g + 1 and g + 9 of butterfly t.
constexpr int kDwFB = 57;

template <int p>
__device__ void dft_mma_stage_wide(double2* A, double2* Bf, int P, int m, int lane, int warp, int nw) {
  constexpr int h = (p - 1) / 2;
  static_assert(h > 8 && h <= 15, "two 16 x 16 tiles");
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int UP = 64 - (kDwFB + 1);  // 2^UP |a| < 2^64
  const int gid = lane >> 2, tig = lane & 3;
  const int nb = P / p, mp = m * p, nbt = 2 * nb, ntile = (nbt + 3) / 4;
  const float inv_m = 1.0f / (float)m;
  const int qa = 2 * tig + 1;  // K rows 2t, 2t + 1 -> q = qa, qa + 1; rows 2t + 8, 2t + 9 -> q = qa + 8, qa + 9
  // coefficient fragments of the cos (C) and sin (S) tiles as 64-bit
  // fractions: per slice [0] = (j0; qa, qa+1), [1] = (j1; qa, qa+1),
  // [2] = (j0; qa+8, qa+9), [3] = (j1; qa+8, qa+9), j0 = g + 1, j1 = g + 9
  uint32_t fc[kDwS][4], fs[kDwS][4];
  {
    double c[2][4], sn[2][4];  // [row j0 / j1][q slot]
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int j = gid + 1 + 8 * r;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int q = qa + (i & 1) + 8 * (i >> 1);
        const bool ok = j <= h && q <= h;
        c[r][i] = ok ? DftTab<p>::c((j * q) % p) : 0.0;
        sn[r][i] = ok ? DftTab<p>::s((j * q) % p) : 0.0;
      }
    }
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const int r = f & 1, i0 = 2 * (f >> 1);
      const unsigned long long c0 = dft_mag64(c[r][i0], 0), c1 = dft_mag64(c[r][i0 + 1], 0);
      const unsigned long long s0 = dft_mag64(sn[r][i0], 0), s1 = dft_mag64(sn[r][i0 + 1], 0);
      const uint32_t sgc = sign2(c[r][i0], c[r][i0 + 1]), sgs = sign2(sn[r][i0], sn[r][i0 + 1]);
#pragma unroll
      for (int sl = 0; sl < kDwS; ++sl) {
        fc[sl][f] = dft_slice2w(c0, c1, sgc, sl);
        fs[sl][f] = dft_slice2w(s0, s1, sgs, sl);
      }
    }
  }
  for (int tile = warp; tile < ntile; tile += nw) {
    const int bi = tile * 4 + (gid >> 1), comp = gid & 1;
    double x[4] = {0.0, 0.0, 0.0, 0.0}, y[4] = {0.0, 0.0, 0.0, 0.0}, v0 = 0.0;
    double* pi = nullptr;
    if (bi < nbt) {
      const int sel = bi >= nb, t = bi - sel * nb;
      const int g = (int)(((float)t + 0.5f) * inv_m);
      pi = reinterpret_cast<double*>((sel ? Bf : A) + g * mp + (t - g * m)) + comp;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int q = qa + (i & 1) + 8 * (i >> 1);
        if (q <= h) { x[i] = pi[2 * q * m]; y[i] = pi[2 * (p - q) * m]; }
      }
      v0 = pi[0];
    }
    int fb = biased_exp(v0);
#pragma unroll
    for (int i = 0; i < 4; ++i) fb = max(fb, max(biased_exp(x[i]), biased_exp(y[i])));
    fb = max(fb, __shfl_xor_sync(FULL, fb, 1));
    fb = max(fb, __shfl_xor_sync(FULL, fb, 2));
    fb = max(fb, __shfl_xor_sync(FULL, fb, 4));
    const int e = fb - 1022;
    long long av[4], bv[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long long X = fix_of<kDwFB>(x[i], e), Y = fix_of<kDwFB>(y[i], e);
      av[i] = X + Y;
      bv[i] = X - Y;
    }
    const long long V0 = fix_of<kDwFB>(v0, e);
    long long ys = (av[0] + av[1]) + (av[2] + av[3]);
    ys += __shfl_xor_sync(FULL, ys, 1);
    ys += __shfl_xor_sync(FULL, ys, 2);
    __syncwarp();  // every load of the tile precedes its stores
    if (tig == 0 && pi)
      pi[0] = fb == 2047 ? __longlong_as_double(0x7ff8000000000000LL) : dbl_of_fix(V0 + ys, e - kDwFB);
    long long H[2][4], L[2][4];  // [C / S][(j0 re, j0 im, j1 re, j1 im)]: 2^(e - 71) (H 2^32 + L)
#pragma unroll
    for (int part = 0; part < 2; ++part) {
      const long long* v = part ? bv : av;
      uint32_t fx[kDwS][2];
      {
        unsigned long long t[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) t[i] = (unsigned long long)(v[i] < 0 ? -v[i] : v[i]) << UP;
        const uint32_t s01 = (v[0] < 0 ? 0x8000u : 0u) | (v[1] < 0 ? 0x80000000u : 0u);
        const uint32_t s23 = (v[2] < 0 ? 0x8000u : 0u) | (v[3] < 0 ? 0x80000000u : 0u);
#pragma unroll
        for (int sl = 0; sl < kDwS; ++sl) {
          fx[sl][0] = dft_slice2w(t[0], t[1], s01, sl);
          fx[sl][1] = dft_slice2w(t[2], t[3], s23, sl);
        }
      }
      float acc[kDwD + 1][4];
#pragma unroll
      for (int d = 0; d <= kDwD; ++d)
#pragma unroll
        for (int i = 0; i < 4; ++i) acc[d][i] = 0.f;
#pragma unroll
      for (int sl = 0; sl < kDwS; ++sl) {
        const uint32_t* f = part ? fs[sl] : fc[sl];
#pragma unroll
        for (int t = 0; t < kDwS && sl + t <= kDwD; ++t) mma_f16(acc[sl + t], f[0], f[1], f[2], f[3], fx[t][0], fx[t][1]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        long long hh = 0, ll = 0;
#pragma unroll
        for (int d = 0; d <= 3; ++d) hh = hh * 256 + __float2int_rn(acc[d][i]);
#pragma unroll
        for (int d = 4; d <= kDwD; ++d) ll = ll * 256 + __float2int_rn(acc[d][i]);
        H[part][i] = hh;
        L[part][i] = ll;
      }
    }
    const int bo = tile * 4 + tig;
    const int eo = __shfl_sync(FULL, e, 8 * tig);
    const long long w_re = __shfl_sync(FULL, V0, 8 * tig), w_im = __shfl_sync(FULL, V0, 8 * tig + 4);
    if (bo < nbt) {
      const int sel = bo >= nb, t = bo - sel * nb;
      const int g = (int)(((float)t + 0.5f) * inv_m);
      double2* po = (sel ? Bf : A) + g * mp + (t - g * m);
      // v_0 (units 2^(e - 57)) as 2^14 V = (V >> 18) 2^32 + (V mod 2^18) 2^14
      const long long vhr = w_re >> 18, vlr = (w_re & ((1LL << 18) - 1)) << 14;
      const long long vhi = w_im >> 18, vli = (w_im & ((1LL << 18) - 1)) << 14;
      const int k = eo - 71;
      const double nan = __longlong_as_double(0x7ff8000000000000LL);
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const int j = gid + 1 + 8 * r;
        if (j <= h) {
          const long long hr = H[0][2 * r] + vhr, lr = L[0][2 * r] + vlr;
          const long long hi = H[0][2 * r + 1] + vhi, li = L[0][2 * r + 1] + vli;
          double2 yj = make_double2(combine_rn(hr + H[1][2 * r + 1], lr + L[1][2 * r + 1], k, 32),
                                    combine_rn(hi - H[1][2 * r], li - L[1][2 * r], k, 32));
          double2 yk = make_double2(combine_rn(hr - H[1][2 * r + 1], lr - L[1][2 * r + 1], k, 32),
                                    combine_rn(hi + H[1][2 * r], li + L[1][2 * r], k, 32));
          if (eo == 2047 - 1022) yj = yk = make_double2(nan, nan);
          po[j * m] = yj;
          po[(p - j) * m] = yk;
        }
      }
    }
  }
}

// One stage of the block-per-line form: large odd primes of a prime-factor
// plan through fft_stage_split over the whole block, the rest per buffer
// half (run_stage1).  Called by every thread of the block.
template <int MAXP>
__device__ __forceinline__ void run_stage_block(int p, bool dif, bool twid, double2* A, double2* Bf, double2* mine,
                                                int P, int m, int stride, const double2* tw, int tid, int nt, int hl,
                                                int nl) {
  if constexpr (MAXP == 31) {
    if (!twid && (p == 19 || p == 23 || p == 29 || p == 31)) {
      if (p == 19) dft_mma_stage_wide<19>(A, Bf, P, m, tid & 31, tid >> 5, nt >> 5);
      else if (p == 23) dft_mma_stage_wide<23>(A, Bf, P, m, tid & 31, tid >> 5, nt >> 5);
      else if (p == 29) dft_mma_stage_wide<29>(A, Bf, P, m, tid & 31, tid >> 5, nt >> 5);
      else dft_mma_stage_wide<31>(A, Bf, P, m, tid & 31, tid >> 5, nt >> 5);
      __syncthreads();
      return;
    }
  }
  if constexpr (MAXP == 17) {  // plans with a prime above 17 keep the FMA butterflies
    if (!twid && (p == 11 || p == 13 || p == 17)) {
      if (p == 11) dft_mma_stage<11>(A, Bf, P, m, tid & 31, tid >> 5, nt >> 5);
      else if (p == 13) dft_mma_stage<13>(A, Bf, P, m, tid & 31, tid >> 5, nt >> 5);
      else dft_mma_stage<17>(A, Bf, P, m, tid & 31, tid >> 5, nt >> 5);
      __syncthreads();
      return;
    }
  }
  if (!twid) {
    switch (p) {
#define FALCON_SPLIT(q, g)                                  \
  case q:                                                   \
    if constexpr (q <= MAXP) {                              \
      fft_stage_split<q, g>(A, Bf, P, m, tid, nt);          \
      return;                                               \
    }                                                       \
    break;
      FALCON_SPLIT(17, 2) FALCON_SPLIT(19, 2) FALCON_SPLIT(23, 3) FALCON_SPLIT(29, 3) FALCON_SPLIT(31, 3)
#undef FALCON_SPLIT
      default: break;
    }
  }
  run_stage1<MAXP>(p, dif, twid, mine, P, m, stride, tw, hl, nl);
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Nonlinear pass (Nr_maxLOOP, src/nonlin.F90:55-86): one warp per radial
// line (r, b).  invfft of T, omega, u_phi, u_r (two complex inverse FFTs of
// length P, each carrying two real fields), the four grid products, and the
// two forward FFTs that return u_phi*T, u_r*T, u_phi*omega, u_r*omega
// truncated to modes 0..Nm and divided by P.
// ---------------------------------------------------------------------------
// A prime-factor plan of radices <= 17 reads no twiddles (its butterflies
// take their coefficients from constant memory), so its blocks carry only
// the index table and the line buffers: 3 blocks of 4 lines fit an SM.
template <int MAXP>
constexpr int nonlin_min_blocks() { return MAXP == 17 ? 3 : 1; }

template <int MAXP>
__global__ void __launch_bounds__(128, nonlin_min_blocks<MAXP>()) nonlin_kernel(NonlinArgs a) {
  extern __shared__ double2 smem[];
  const int P = a.plan.P;
  const bool no_tw = MAXP == 17 && a.plan.pfa;
  const int tw_len = no_tw ? 0 : P;
  double2* tw = smem;
  int* pos = reinterpret_cast<int*>(smem + tw_len);
  const int pos_pad = (P + 3) / 4;  // ints rounded up to double2 units (16 B)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarp = blockDim.x >> 5;
  double2* bufA = smem + tw_len + pos_pad + (size_t)warp * 2 * P;
  double2* bufB = bufA + P;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    if (!no_tw) tw[i] = a.tw[i];
    pos[i] = a.pos[i];
  }
  __syncthreads();
  const int nlines = a.R * a.B;
  const int line = blockIdx.x * nwarp + warp;
  if (line >= nlines) return;
  const int r = line / a.B, b = line - r * a.B;
  const int M = a.M, B = a.B, Nm = a.Nm;
  for (int j = lane; j < P; j += 32) { bufA[j] = make_double2(0, 0); bufB[j] = make_double2(0, 0); }
  __syncwarp();
  // Scatter conj(Z) at digit-reversed positions, Z_k = X_k + i Y_k for the
  // Hermitian spectra X, Y of two real lines (only Re of mode 0 counts, as
  // in a c2r transform).  IFFT(Z) = conj(FFT(conj(Z))).
  const size_t row = (size_t)r * M * B + b;
  for (int k = lane; k <= Nm; k += 32) {
    const size_t e = row + (size_t)k * B;
    const double2 T = a.t[e], W = a.w[e], U = a.up[e], V = a.ur[e];
    if (k == 0) {
      bufA[pos[0]] = make_double2(T.x, -W.x);
      bufB[pos[0]] = make_double2(U.x, -V.x);
    } else {
      // conj(Z_k) = (T.x - W.y, -(T.y + W.x)); conj(Z_{P-k}) = (T.x + W.y, T.y - W.x)
      bufA[pos[k]] = make_double2(T.x - W.y, -(T.y + W.x));
      bufA[pos[P - k]] = make_double2(T.x + W.y, T.y - W.x);
      bufB[pos[k]] = make_double2(U.x - V.y, -(U.y + V.x));
      bufB[pos[P - k]] = make_double2(U.x + V.y, U.y - V.x);
    }
  }
  __syncwarp();
  {  // DIT: radices processed innermost first
    int m = 1;
    for (int s = a.plan.nrad - 1; s >= 0; --s) {
      const int p = a.plan.rad[s];
      run_stage<MAXP>(p, false, !a.plan.pfa, bufA, bufB, P, m, P / (m * p), tw, lane);
      m *= p;
      __syncwarp();
    }
  }
  // Grid values: bufA = conj(t + i omg) -> t = A.x, omg = -A.y; likewise for
  // (u_phi, u_r) in bufB.  Products, in natural order for the DIF.
  double urmax = 0.0, upmax = 0.0;
  const bool want_max = a.umax != nullptr;
  for (int j = lane; j < P; j += 32) {
    const double2 za = bufA[j], zb = bufB[j];
    const double tt = za.x, om = -za.y, up = zb.x, ur = -zb.y;
    bufA[j] = make_double2(up * tt, ur * tt);
    bufB[j] = make_double2(up * om, ur * om);
    if (want_max) {  // FP64 max instructions only when the CFL inputs are read
      urmax = fmax(urmax, fabs(ur));
      upmax = fmax(upmax, fabs(up));
    }
  }
  __syncwarp();
  {  // DIF: outermost radix first
    int m = P;
    for (int s = 0; s < a.plan.nrad; ++s) {
      const int p = a.plan.rad[s];
      m /= p;
      run_stage<MAXP>(p, true, !a.plan.pfa, bufA, bufB, P, m, P / (m * p), tw, lane);
      __syncwarp();
    }
  }
  // Split the two-for-one spectra: X_k = (Z_k + conj Z_{P-k})/2,
  // Y_k = (Z_k - conj Z_{P-k})/(2i), then divide by P.
  const double s = 0.5 / (double)P;
  for (int k = lane; k <= Nm; k += 32) {
    const size_t e = row + (size_t)k * B;
    const double2 za = bufA[pos[k]], ca = bufA[pos[k == 0 ? 0 : P - k]];
    const double2 zb = bufB[pos[k]], cb = bufB[pos[k == 0 ? 0 : P - k]];
    a.ntp[e] = make_double2((za.x + ca.x) * s, (za.y - ca.y) * s);
    a.ntr[e] = make_double2((za.y + ca.y) * s, (ca.x - za.x) * s);
    a.nwp[e] = make_double2((zb.x + cb.x) * s, (zb.y - cb.y) * s);
    a.nwr[e] = make_double2((zb.y + cb.y) * s, (cb.x - zb.x) * s);
  }
  if (a.umax) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      urmax = fmax(urmax, __shfl_xor_sync(0xffffffffu, urmax, o));
      upmax = fmax(upmax, __shfl_xor_sync(0xffffffffu, upmax, o));
    }
    if (lane == 0) {
      a.umax[2 * ((size_t)r * B + b)] = urmax;
      a.umax[2 * ((size_t)r * B + b) + 1] = upmax;
    }
  }
}

// Block-per-line form of the same pass, for launches with too few radial
// lines to fill the GPU at one warp per line (one instance, or a small
// group): the (T, omega) and (u_phi, u_r) transforms run on the two halves of
// the block, each spread over S warps, with block barriers between stages.
// Same arithmetic per element as nonlin_kernel (bit-identical results).
template <int MAXP, int S>
__global__ void __launch_bounds__(64 * S) nonlin_line_kernel(NonlinArgs a) {
  extern __shared__ double2 smem[];
  __shared__ double red[2][2 * S];
  const int P = a.plan.P;
  double2* tw = smem;
  int* pos = reinterpret_cast<int*>(smem + P);
  const int pos_pad = (P + 3) / 4;
  double2* bufA = smem + P + pos_pad;
  double2* bufB = bufA + P;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int nl = 32 * S, half = tid / nl, hl = tid - half * nl;
  double2* mine = half ? bufB : bufA;
  for (int i = tid; i < P; i += nt) {
    tw[i] = a.tw[i];
    pos[i] = a.pos[i];
    bufA[i] = make_double2(0, 0);
    bufB[i] = make_double2(0, 0);
  }
  __syncthreads();
  const int line = blockIdx.x;
  const int r = line / a.B, b = line - r * a.B;
  const int M = a.M, B = a.B, Nm = a.Nm;
  const size_t row = (size_t)r * M * B + b;
  for (int k = tid; k <= Nm; k += nt) {
    const size_t e = row + (size_t)k * B;
    const double2 T = a.t[e], W = a.w[e], U = a.up[e], V = a.ur[e];
    if (k == 0) {
      bufA[pos[0]] = make_double2(T.x, -W.x);
      bufB[pos[0]] = make_double2(U.x, -V.x);
    } else {
      bufA[pos[k]] = make_double2(T.x - W.y, -(T.y + W.x));
      bufA[pos[P - k]] = make_double2(T.x + W.y, T.y - W.x);
      bufB[pos[k]] = make_double2(U.x - V.y, -(U.y + V.x));
      bufB[pos[P - k]] = make_double2(U.x + V.y, U.y - V.x);
    }
  }
  __syncthreads();
  {
    int m = 1;
    for (int s = a.plan.nrad - 1; s >= 0; --s) {
      const int p = a.plan.rad[s];
      run_stage_block<MAXP>(p, false, !a.plan.pfa, bufA, bufB, mine, P, m, P / (m * p), tw, tid, nt, hl, nl);
      m *= p;
    }
  }
  double urmax = 0.0, upmax = 0.0;
  const bool want_max = a.umax != nullptr;
  for (int j = tid; j < P; j += nt) {
    const double2 za = bufA[j], zb = bufB[j];
    const double tt = za.x, om = -za.y, up = zb.x, ur = -zb.y;
    bufA[j] = make_double2(up * tt, ur * tt);
    bufB[j] = make_double2(up * om, ur * om);
    if (want_max) {  // FP64 max instructions only when the CFL inputs are read
      urmax = fmax(urmax, fabs(ur));
      upmax = fmax(upmax, fabs(up));
    }
  }
  __syncthreads();
  {
    int m = P;
    for (int s = 0; s < a.plan.nrad; ++s) {
      const int p = a.plan.rad[s];
      m /= p;
      run_stage_block<MAXP>(p, true, !a.plan.pfa, bufA, bufB, mine, P, m, P / (m * p), tw, tid, nt, hl, nl);
    }
  }
  const double sc = 0.5 / (double)P;
  for (int k = tid; k <= Nm; k += nt) {
    const size_t e = row + (size_t)k * B;
    const double2 za = bufA[pos[k]], ca = bufA[pos[k == 0 ? 0 : P - k]];
    const double2 zb = bufB[pos[k]], cb = bufB[pos[k == 0 ? 0 : P - k]];
    a.ntp[e] = make_double2((za.x + ca.x) * sc, (za.y - ca.y) * sc);
    a.ntr[e] = make_double2((za.y + ca.y) * sc, (ca.x - za.x) * sc);
    a.nwp[e] = make_double2((zb.x + cb.x) * sc, (zb.y - cb.y) * sc);
    a.nwr[e] = make_double2((zb.y + cb.y) * sc, (cb.x - zb.x) * sc);
  }
  if (a.umax) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      urmax = fmax(urmax, __shfl_xor_sync(0xffffffffu, urmax, o));
      upmax = fmax(upmax, __shfl_xor_sync(0xffffffffu, upmax, o));
    }
    const int w = tid >> 5;
    if ((tid & 31) == 0) { red[0][w] = urmax; red[1][w] = upmax; }
    __syncthreads();
    if (tid == 0) {
      for (int i = 1; i < 2 * S; ++i) { urmax = fmax(urmax, red[0][i]); upmax = fmax(upmax, red[1][i]); }
      a.umax[2 * ((size_t)r * B + b)] = urmax;
      a.umax[2 * ((size_t)r * B + b) + 1] = upmax;
    }
  }
}

static int nonlin_warps(int P, bool no_tw, int* smem_bytes) {
  int dev = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const int fixed = ((no_tw ? 0 : P) + (P + 3) / 4) * 16;
  int w = 4;
  while (w > 1 && fixed + w * 2 * P * 16 > maxsm) --w;
  *smem_bytes = fixed + w * 2 * P * 16;
  return w;
}

template <int MAXP, int S>
static cudaError_t launch_nonlin_line(const NonlinArgs& a, cudaStream_t s) {
  const int P = a.plan.P;
  const int smem = (P + (P + 3) / 4 + 2 * P) * 16;
  cudaError_t e = cudaFuncSetAttribute(nonlin_line_kernel<MAXP, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  nonlin_line_kernel<MAXP, S><<<a.R * a.B, 64 * S, smem, s>>>(a);
  return cudaGetLastError();
}

// Resident warps per SM of the warp-per-line form (w warps a block, smem
// bytes) and of the block-per-line form with 8 warps a line, from the
// occupancy calculator; memoised per (form, P).
template <int MAXP>
static bool line_form_holds_more_warps(int P, int w, int smem) {
  struct Memo { int P, w, smem; bool line; };
  thread_local std::vector<Memo> memo;
  for (const Memo& m : memo)
    if (m.P == P && m.w == w && m.smem == smem) return m.line;
  const int smem_line = (P + (P + 3) / 4 + 2 * P) * 16;
  int nb_warp = 0, nb_line = 0;
  bool line = false;
  if (cudaFuncSetAttribute(nonlin_kernel<MAXP>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) == cudaSuccess &&
      cudaFuncSetAttribute(nonlin_line_kernel<MAXP, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_line) ==
          cudaSuccess &&
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb_warp, nonlin_kernel<MAXP>, 32 * w, smem) == cudaSuccess &&
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb_line, nonlin_line_kernel<MAXP, 4>, 256, smem_line) ==
          cudaSuccess)
    line = nb_line * 8 > nb_warp * w;
  memo.push_back(Memo{P, w, smem, line});
  return line;
}

// Lines that one warp each cannot spread over the GPU (fewer than two per
// SM) go to the block-per-line form: 8 warps per line up to one line per
// SM, 4 up to two.  So do long lines whose warp-per-line blocks (a whole
// line per warp in shared memory) would leave fewer warps on an SM than the
// block-per-line form (Np = 1023, 1536: 3-4 against 16 warps per SM).
template <int MAXP>
static cudaError_t launch_nonlin_t(const NonlinArgs& a, cudaStream_t s) {
  int dev = 0, nsm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int nlines = a.R * a.B;
  if (nlines <= nsm) return launch_nonlin_line<MAXP, 4>(a, s);
  if (nlines <= 2 * nsm) return launch_nonlin_line<MAXP, 2>(a, s);
  int smem = 0;
  const int w = nonlin_warps(a.plan.P, MAXP == 17 && a.plan.pfa, &smem);
  if (line_form_holds_more_warps<MAXP>(a.plan.P, w, smem)) return launch_nonlin_line<MAXP, 4>(a, s);
  cudaError_t e = cudaFuncSetAttribute(nonlin_kernel<MAXP>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const int grid = (nlines + w - 1) / w;
  nonlin_kernel<MAXP><<<grid, 32 * w, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace
}  // namespace falcon
