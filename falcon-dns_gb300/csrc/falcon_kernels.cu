// sm_103a kernels of the FAlCon-DNS time step (FP64 throughout).
//
// On GB300 the FP64 FMA pipe (~1.2 TFLOP/s measured) is ~30x slower than
// HBM relative to the bytes these kernels move, so every kernel here is
// bound by FP64 issue, not memory: the code minimises FP64 instructions
// (two-for-one real transforms, symmetric odd-prime butterflies with
// constant-bank coefficients, register-tiled DFMA GEMMs) and keeps the
// non-FP64 instruction count per FMA below one.
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "falcon_internal.h"
#include "falcon_slices.cuh"

namespace falcon {

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

cudaError_t init_dft_tables() {
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

cudaError_t launch_nonlin(const NonlinArgs& a, cudaStream_t s) {
  int maxp = 0;
  for (int i = 0; i < a.plan.nrad; ++i) maxp = a.plan.rad[i] > maxp ? a.plan.rad[i] : maxp;
  if (maxp <= 7) return launch_nonlin_t<7>(a, s);
  if (maxp <= 17) return launch_nonlin_t<17>(a, s);
  return launch_nonlin_t<31>(a, s);
}

// ---------------------------------------------------------------------------
// Register-tiled FP64 GEMM, Y = alpha * A * X (A column-major, rows x K).
// A block covers NCOL columns (64, 32 or 16) and nw * RG * RPT rows, RG =
// 64 / NCOL: lane = (row group rg, column pair cp) with NCOL / 2 column
// pairs, so warp w owns rows [row0 + (w*RG + rg)*RPT, +RPT) and columns
// n0 + 2*cp + {0,1}.  Narrow tiles keep the lanes busy when a batch entry
// has few columns (per-mode solves of small groups).  K is staged in chunks
// of 16 through shared memory; the last chunk runs only its valid length.
// Every output accumulates over k in ascending order with FMAs, whatever
// the tile, so results do not depend on the launch shape.
// ---------------------------------------------------------------------------
constexpr int kKC = 16;

// Asynchronous 8-byte global -> shared copy (cp.async); a masked element is
// written as zero without reading global memory.
__device__ __forceinline__ void cp_async8(double* dst, const double* src, bool valid) {
  const unsigned saddr = (unsigned)__cvta_generic_to_shared(dst);
  const int sz = valid ? 8 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(saddr), "l"(src), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <int RPT, int NCOL>
__global__ void __launch_bounds__(512) gemm_tile_kernel(GemmArgs g) {
  constexpr int RG = 64 / NCOL, CP = NCOL / 2;
  extern __shared__ __align__(16) double gsm[];
  const int nw = blockDim.x >> 5;
  const int rows_blk = nw * RG * RPT;
  const int stage = kKC * (rows_blk + NCOL);   // one buffer: A [kKC][rows_blk], X [kKC][NCOL]
  const int z = blockIdx.z;
  const double* A = g.A + (size_t)z * g.sA;
  const double* X = g.X + (size_t)z * g.sX;
  double* Y = g.Y + (size_t)z * g.sY;
  const int n0 = blockIdx.x * NCOL;
  const int row0 = blockIdx.y * rows_blk;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rg = lane / CP, cp = lane - rg * CP;
  const int rw = (warp * RG + rg) * RPT;  // first row of this thread within the block
  double acc[RPT][2];
#pragma unroll
  for (int i = 0; i < RPT; ++i) { acc[i][0] = 0.0; acc[i][1] = 0.0; }
  const int nthr = blockDim.x;
  // Double-buffered K chunks: the copies of chunk c+1 are in flight while
  // chunk c is multiplied, so the memory latency is hidden even when a
  // small grid leaves no other blocks to switch to.
  auto issue = [&](int k0, double* buf) {
    const int kc = min(kKC, g.K - k0);
    const int na = kc * rows_blk, nx = kc * NCOL;
    for (int idx = threadIdx.x; idx < na + nx; idx += nthr) {
      if (idx < na) {
        const int kk = idx / rows_blk, rr = idx - kk * rows_blk, row = row0 + rr;
        const bool ok = row < g.rows;
        cp_async8(buf + idx, ok ? A + (size_t)(k0 + kk) * g.lda + row : A, ok);
      } else {
        const int j = idx - na, kk = j / NCOL, c = j - kk * NCOL, n = n0 + c;
        const bool ok = n < g.N;
        cp_async8(buf + kKC * rows_blk + j, ok ? X + (size_t)(k0 + kk) * g.ldx + n : X, ok);
      }
    }
    cp_async_commit();
  };
  issue(0, gsm);
  int cur = 0;
  for (int k0 = 0; k0 < g.K; k0 += kKC) {
    const int kc = min(kKC, g.K - k0);
    const bool more = k0 + kKC < g.K;
    if (more) {
      issue(k0 + kKC, gsm + (cur ^ 1) * stage);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const double* As = gsm + cur * stage;
    const double* Xs = As + kKC * rows_blk;
    const double* Aw = As + rw;
    if (kc == kKC) {
#pragma unroll
      for (int kk = 0; kk < kKC; ++kk) {
        const double2 xv = *reinterpret_cast<const double2*>(&Xs[kk * NCOL + 2 * cp]);
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
          const double av = Aw[kk * rows_blk + i];
          acc[i][0] = fma(av, xv.x, acc[i][0]);
          acc[i][1] = fma(av, xv.y, acc[i][1]);
        }
      }
    } else {
      for (int kk = 0; kk < kc; ++kk) {
        const double2 xv = *reinterpret_cast<const double2*>(&Xs[kk * NCOL + 2 * cp]);
#pragma unroll
        for (int i = 0; i < RPT; ++i) {
          const double av = Aw[kk * rows_blk + i];
          acc[i][0] = fma(av, xv.x, acc[i][0]);
          acc[i][1] = fma(av, xv.y, acc[i][1]);
        }
      }
    }
    __syncthreads();  // every thread is done with this buffer before it is refilled
    cur ^= 1;
  }
  const int n = n0 + 2 * cp;
#pragma unroll
  for (int i = 0; i < RPT; ++i) {
    const int row = row0 + rw + i;
    if (row < g.rows) {
      double* yp = &Y[(size_t)row * g.ldy + n];
      if (n + 1 < g.N && (reinterpret_cast<uintptr_t>(yp) & 15) == 0) {
        *reinterpret_cast<double2*>(yp) = make_double2(g.alpha * acc[i][0], g.alpha * acc[i][1]);
      } else if (n + 1 < g.N) {
        // odd leading dimension or offset: two 8-byte stores
        yp[0] = g.alpha * acc[i][0];
        yp[1] = g.alpha * acc[i][1];
      } else if (n < g.N) {
        Y[(size_t)row * g.ldy + n] = g.alpha * acc[i][0];
      }
    }
  }
}

// Small-N form (N <= 8 columns per batch entry): one thread per output row.
template <int NC>
__global__ void __launch_bounds__(32) dfma_gemv_kernel(GemmArgs g) {
  extern __shared__ double xs[];  // K x NC
  const int z = blockIdx.y;
  const double* A = g.A + (size_t)z * g.sA;
  const double* X = g.X + (size_t)z * g.sX;
  double* Y = g.Y + (size_t)z * g.sY;
  // the block's X panel, eight loads in flight per thread
  const int nthr = blockDim.x, nx = g.K * NC;
  for (int b0 = 0; b0 < nx; b0 += 8 * nthr) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = b0 + u * nthr + (int)threadIdx.x;
      const int k = idx / NC, c = idx - k * NC;
      v[u] = (idx < nx && c < g.N) ? X[(size_t)k * g.ldx + c] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int idx = b0 + u * nthr + (int)threadIdx.x;
      if (idx < nx) xs[idx] = v[u];
    }
  }
  __syncthreads();
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= g.rows) return;
  double acc[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc[c] = 0.0;
  // A loads issued eight at a time ahead of their FMAs (k order kept)
  int k = 0;
  for (; k + 8 <= g.K; k += 8) {
    double av[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) av[u] = A[(size_t)(k + u) * g.lda + row];
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[c] = fma(av[u], xs[(k + u) * NC + c], acc[c]);
  }
  for (; k < g.K; ++k) {
    const double av = A[(size_t)k * g.lda + row];
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] = fma(av, xs[k * NC + c], acc[c]);
  }
#pragma unroll
  for (int c = 0; c < NC; ++c)
    if (c < g.N) Y[(size_t)row * g.ldy + c] = g.alpha * acc[c];
}

template <int RPT, int NCOL>
static cudaError_t launch_tile(const GemmArgs& g, int nw, int row_blocks, cudaStream_t s) {
  // two K-chunk buffers; above 48 KB the kernel is opted in once per device
  static std::atomic<bool> opted[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (!(dev >= 0 && dev < 64 && opted[dev].load())) {
    const cudaError_t e = cudaFuncSetAttribute(gemm_tile_kernel<RPT, NCOL>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) opted[dev].store(true);
  }
  dim3 grid((g.N + NCOL - 1) / NCOL, row_blocks, g.batch);
  const size_t smem = (size_t)2 * kKC * (nw * (64 / NCOL) * RPT + NCOL) * sizeof(double);
  gemm_tile_kernel<RPT, NCOL><<<grid, 32 * nw, smem, s>>>(g);
  return cudaGetLastError();
}

// Launch shape from a cost model of the FP64 pipe: a block's work is
// rows_blk x NCOL per k; blocks spread evenly over the SMs, so an SM runs
// ceil(blocks / nsm) of them; an SM with fewer than 4 resident warps leaves
// FP64 units of its sub-partitions idle.  The cheapest (NCOL, row blocks
// rb, warps nw, rows per thread rpt) wins, ties going to deeper register
// tiles; extra row blocks (each re-stages the X panel) and single-row
// threads carry a small penalty.
struct TileShape { int ncol, rb, nw, rpt; };
static TileShape pick_shape(const GemmArgs& g, int nsm) {
  TileShape best{64, 1, 8, 1};
  double bcost = 1e300;
  int brpt = 0;
  for (int ncol = 16; ncol <= 64; ncol *= 2) {
    if (g.fma_ncol && ncol != g.fma_ncol) continue;
    const int rg = 64 / ncol, maxr = (ncol == 64) ? 16 : 8;
    const long cb = (long)((g.N + ncol - 1) / ncol) * g.batch;
    for (int rb = 1; rb <= 16; ++rb)
      for (int nw = 2; nw <= 16; ++nw)
        for (int rpt = 1; rpt <= maxr; ++rpt) {
          const int rows_blk = nw * rg * rpt;
          if ((long)rb * rows_blk < g.rows) continue;
          if ((long)(rb - 1) * rows_blk >= g.rows) continue;   // no empty row block
          if (rows_blk > 256) continue;                         // two K buffers <= 80 KB
          const long blocks = cb * rb;
          const long waves = (blocks + nsm - 1) / nsm;
          const long occ = std::max(1, std::min(48 / nw, 5));
          const double wps = (double)nw * (double)std::min(waves, occ);
          const double eff = std::min(1.0, wps / 4.0);
          const double cost = (double)waves * rows_blk * ncol / eff * (1.0 + 0.02 * (rb - 1)) *
                              (rpt == 1 ? 1.1 : 1.0);
          if (cost < bcost * (1.0 - 1e-12) || (cost <= bcost * (1.0 + 1e-12) && rpt > brpt)) {
            bcost = cost; brpt = rpt; best = {ncol, rb, nw, rpt};
          }
        }
  }
  return best;
}

template <int NCOL>
static cudaError_t launch_ncol(const GemmArgs& g, const TileShape& t, cudaStream_t s) {
  switch (t.rpt) {
    case 1: return launch_tile<1, NCOL>(g, t.nw, t.rb, s);
    case 2: return launch_tile<2, NCOL>(g, t.nw, t.rb, s);
    case 3: return launch_tile<3, NCOL>(g, t.nw, t.rb, s);
    case 4: return launch_tile<4, NCOL>(g, t.nw, t.rb, s);
    case 5: return launch_tile<5, NCOL>(g, t.nw, t.rb, s);
    case 6: return launch_tile<6, NCOL>(g, t.nw, t.rb, s);
    case 7: return launch_tile<7, NCOL>(g, t.nw, t.rb, s);
    case 8: return launch_tile<8, NCOL>(g, t.nw, t.rb, s);
    default: break;
  }
  if constexpr (NCOL == 64) {
    switch (t.rpt) {
      case 9: return launch_tile<9, 64>(g, t.nw, t.rb, s);
      case 10: return launch_tile<10, 64>(g, t.nw, t.rb, s);
      case 11: return launch_tile<11, 64>(g, t.nw, t.rb, s);
      case 12: return launch_tile<12, 64>(g, t.nw, t.rb, s);
      case 13: return launch_tile<13, 64>(g, t.nw, t.rb, s);
      case 14: return launch_tile<14, 64>(g, t.nw, t.rb, s);
      case 15: return launch_tile<15, 64>(g, t.nw, t.rb, s);
      default: return launch_tile<16, 64>(g, t.nw, t.rb, s);
    }
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_gemm(const GemmArgs& g, cudaStream_t s) {
  if (g.rows <= 0 || g.N <= 0 || g.batch <= 0) return cudaSuccess;
  if (g.oz_s) return launch_oz_gemm(g, s);
  if (g.N <= 8) {
    // one warp of rows per block, so small problems spread over the SMs
    dim3 grid((g.rows + 31) / 32, g.batch);
    const size_t sm = (size_t)g.K * 8 * sizeof(double);
    if (g.N <= 2) dfma_gemv_kernel<2><<<grid, 32, (size_t)g.K * 2 * sizeof(double), s>>>(g);
    else if (g.N <= 4) dfma_gemv_kernel<4><<<grid, 32, (size_t)g.K * 4 * sizeof(double), s>>>(g);
    else dfma_gemv_kernel<8><<<grid, 32, sm, s>>>(g);
    return cudaGetLastError();
  }
  static int nsm_dev[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  int nsm = (dev >= 0 && dev < 64) ? nsm_dev[dev] : 0;
  if (nsm == 0) {
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 152;
    if (dev >= 0 && dev < 64) nsm_dev[dev] = nsm;
  }
  // shapes are memoised per (rows, N, batch, SM count, column width asked
  // for): the search runs on the host once per problem size
  struct Memo { int rows, N, batch, nsm, ncol; TileShape t; };
  thread_local std::unordered_map<unsigned long long, Memo> memo;
  // (a hash; the entry is checked against the full sizes)
  const unsigned long long key = (unsigned long long)(g.rows & 0xfff) | ((unsigned long long)(g.N & 0xffffff) << 12) |
                                 ((unsigned long long)(g.batch & 0xffff) << 36) |
                                 ((unsigned long long)(nsm & 0x3ff) << 52) |
                                 ((unsigned long long)(g.fma_ncol == 0 ? 0 : g.fma_ncol == 16 ? 1 : g.fma_ncol == 32 ? 2 : 3)
                                  << 62);
  auto it = memo.find(key);
  TileShape t;
  if (it != memo.end() && it->second.rows == g.rows && it->second.N == g.N && it->second.batch == g.batch &&
      it->second.nsm == nsm && it->second.ncol == g.fma_ncol) {
    t = it->second.t;
  } else {
    t = pick_shape(g, nsm);
    memo[key] = Memo{g.rows, g.N, g.batch, nsm, g.fma_ncol, t};
  }
  if (t.ncol == 16) return launch_ncol<16>(g, t, s);
  if (t.ncol == 32) return launch_ncol<32>(g, t, s);
  return launch_ncol<64>(g, t, s);
}

// ---------------------------------------------------------------------------
// IMEX right-hand sides (rhs_construct_temp / _vort / _uphi_bar,
// src/rhs_create.F90:24-385), one thread per (r, m, b).
// ---------------------------------------------------------------------------
// The FP64 pipe bounds this kernel (~35 FP64 instructions per element
// against ~20 bytes of HBM traffic per instruction's worth of time), so the
// weights are folded once per thread (c_exp = dt w_exp) and every sum is a
// chain of FMAs.
__global__ void imex_rhs_kernel(RhsArgs a) {
  const unsigned B = (unsigned)a.B, M = (unsigned)a.M;
  const size_t total = (size_t)a.R * M * B;
  const double dt = a.dt;
  double c_exp[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) c_exp[i] = dt * a.w_exp[i];
  const double c_cn = (1.0 - a.w_imp[0]) * dt;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t rm = e / B;
    const unsigned b = (unsigned)(e - rm * B);
    const unsigned r = (unsigned)(rm / M), m = (unsigned)(rm - (size_t)r * M);
    const double ir = a.inv_r[r];
    const double dm = (double)(int)m, dmir = dm * ir;
    // upFR_prev = upFR after the nonlinear pass (src/steptime.F90:212), for
    // the u_phi balance of the diagnostics
    if (m == 0 && a.up0_prev) a.up0_prev[(size_t)r * B + b] = a.up[e].x;
    // explicit (advective) term of T: i m r^-1 (uphi T) + d(ur T)/dr + r^-1 (ur T)
    {
      const double2 p = a.ntp[e], q = a.ntr[e], dq = a.dntr[e];
      const double2 nt = make_double2(fma(-dmir, p.y, fma(ir, q.x, dq.x)), fma(dmir, p.x, fma(ir, q.y, dq.y)));
      a.nt_new[e] = nt;
      double2 rhs;
      if (a.scheme_cn) {
        const double2 T = a.th[0][e], L = a.lt[e];
        const double c = c_cn * a.inv_pr[b], k2 = dm * dm * a.inv_r2[r];
        rhs = make_double2(fma(c, fma(-k2, T.x, L.x), T.x), fma(c, fma(-k2, T.y, L.y), T.y));
      } else {
        const double2 h0 = a.th[0][e];
        rhs = make_double2(a.w_imp[0] * h0.x, a.w_imp[0] * h0.y);
        for (int i = 1; i < a.n_imp; ++i) {
          const double2 h = a.th[i][e];
          rhs.x = fma(a.w_imp[i], h.x, rhs.x); rhs.y = fma(a.w_imp[i], h.y, rhs.y);
        }
      }
      rhs.x = fma(-c_exp[0], nt.x, rhs.x); rhs.y = fma(-c_exp[0], nt.y, rhs.y);
      for (int i = 1; i < a.n_exp; ++i) {
        const double2 h = a.nth[i][e];
        rhs.x = fma(-c_exp[i], h.x, rhs.x); rhs.y = fma(-c_exp[i], h.y, rhs.y);
      }
      if (r == 0) rhs = make_double2(m == 0 ? 1.0 : 0.0, 0.0);
      if (r == (unsigned)a.R - 1) rhs = make_double2(0.0, 0.0);
      a.rhs_t[e] = rhs;
    }
    if (m > 0) {
      const double2 p = a.nwp[e], q = a.nwr[e], dq = a.dnwr[e];
      const double2 nw = make_double2(fma(-dmir, p.y, fma(ir, q.x, dq.x)), fma(dmir, p.x, fma(ir, q.y, dq.y)));
      a.nw_new[e] = nw;
      double2 rhs;
      if (a.scheme_cn) {
        const double2 W = a.wh[0][e], L = a.lw[e], To = a.th[0][e];
        const double k2 = dm * dm * a.inv_r2[r];
        const double bc = a.ra_pr[b] * dt * 0.5 * dmir;  // old-T half of the CN buoyancy
        rhs = make_double2(fma(bc, To.y, fma(c_cn, fma(-k2, W.x, L.x), W.x)),
                           fma(-bc, To.x, fma(c_cn, fma(-k2, W.y, L.y), W.y)));
      } else {
        const double2 h0 = a.wh[0][e];
        rhs = make_double2(a.w_imp[0] * h0.x, a.w_imp[0] * h0.y);
        for (int i = 1; i < a.n_imp; ++i) {
          const double2 h = a.wh[i][e];
          rhs.x = fma(a.w_imp[i], h.x, rhs.x); rhs.y = fma(a.w_imp[i], h.y, rhs.y);
        }
      }
      rhs.x = fma(-c_exp[0], nw.x, rhs.x); rhs.y = fma(-c_exp[0], nw.y, rhs.y);
      for (int i = 1; i < a.n_exp; ++i) {
        const double2 h = a.nwh[i][e];
        rhs.x = fma(-c_exp[i], h.x, rhs.x); rhs.y = fma(-c_exp[i], h.y, rhs.y);
      }
      if (r == 0 || r == (unsigned)a.R - 1) rhs = make_double2(0.0, 0.0);
      a.rhs_w[e] = rhs;
    } else {
      // mean azimuthal flow: rhs_construct_uphi_bar
      const size_t rb = (size_t)r * B + b;
      const double urom = a.nwr[e].x;  // mode-0 coefficient of ur*omg = its azimuthal mean
      a.urom_new[rb] = urom;
      double rhs;
      if (a.scheme_cn) {
        const double u = a.ubh[0][rb];
        const double lu = a.lu0[rb].x;
        rhs = fma(c_cn, fma(-a.inv_r2[r], u, lu), u);
      } else {
        rhs = a.w_imp[0] * a.ubh[0][rb];
        for (int i = 1; i < a.n_imp; ++i) rhs = fma(a.w_imp[i], a.ubh[i][rb], rhs);
      }
      rhs = fma(-c_exp[0], urom, rhs);
      for (int i = 1; i < a.n_exp; ++i) rhs = fma(-c_exp[i], a.uromh[i][rb], rhs);
      if (r == 0 || r == (unsigned)a.R - 1) rhs = 0.0;
      a.rhs_w[e] = make_double2(rhs, 0.0);
    }
  }
}

static int ew_grid(size_t n) {
  size_t g = (n + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  return (int)(g ? g : 1);
}

cudaError_t launch_imex_rhs(const RhsArgs& a, cudaStream_t s) {
  imex_rhs_kernel<<<ew_grid((size_t)a.R * a.M * a.B), 256, 0, s>>>(a);
  return cudaGetLastError();
}

__global__ void add_buoyancy_kernel(int R, int M, int B, const double* inv_r, const double* ra_pr,
                                    double scale, const double2* t_new, double2* rhs_w, double2* buo_out) {
  const size_t total = (size_t)R * M * B;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(e % B);
    const size_t rm = e / B;
    const int m = (int)(rm % M);
    const int r = (int)(rm / M);
    if (m == 0) continue;
    const double2 T = t_new[e];
    const double f = (double)m * inv_r[r];
    // buoyancy term -(Ra/Pr) i m r^-1 T
    const double2 bu = make_double2(ra_pr[b] * f * T.y, -ra_pr[b] * f * T.x);
    if (buo_out) buo_out[e] = bu;
    if (rhs_w && r > 0 && r < R - 1) {
      double2 v = rhs_w[e];
      v.x += scale * bu.x; v.y += scale * bu.y;
      rhs_w[e] = v;
    }
  }
}

cudaError_t launch_add_buoyancy(int R, int M, int B, const double* inv_r, const double* ra_pr,
                                double scale, const double2* t_new, double2* rhs_w, double2* buo_out,
                                cudaStream_t s) {
  add_buoyancy_kernel<<<ew_grid((size_t)R * M * B), 256, 0, s>>>(R, M, B, inv_r, ra_pr, scale, t_new,
                                                                  rhs_w, buo_out);
  return cudaGetLastError();
}

// u_r = i m r^-1 psi (m >= 1); mode 0: u_phi = uphi_bar, omega = uphi_bar/r +
// d uphi_bar/dr, u_r = 0 (src/fourierloop.F90:267-315).
__global__ void post_w_kernel(int R, int M, int B, const double* inv_r, const double2* psi, double2* ur,
                              double2* up, double2* w, const double* ub, double* ubar_new) {
  const size_t total = (size_t)R * M * B;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(e % B);
    const size_t rm = e / B;
    const int m = (int)(rm % M);
    const int r = (int)(rm / M);
    if (m > 0) {
      const double2 ps = psi[e];
      const double f = (double)m * inv_r[r];
      ur[e] = make_double2(-f * ps.y, f * ps.x);
    } else {
      const double u = ub[(size_t)r * 2 * B + 2 * b];
      const double du = ub[(size_t)(R + r) * 2 * B + 2 * b];
      up[e] = make_double2(u, 0.0);
      ur[e] = make_double2(0.0, 0.0);
      w[e] = make_double2(u * inv_r[r] + du, 0.0);
      if (ubar_new) ubar_new[(size_t)r * B + b] = u;
    }
  }
}

cudaError_t launch_post_w(int R, int M, int B, const double* inv_r, const double2* psi, double2* ur,
                          double2* up, double2* w, const double* ub, double* ubar_new, cudaStream_t s) {
  post_w_kernel<<<ew_grid((size_t)R * M * B), 256, 0, s>>>(R, M, B, inv_r, psi, ur, up, w, ub, ubar_new);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// IMEXRK stage right-hand side (Get_stage_var, src/fourierloop_imexrk.F90:
// 214-354): Y0 + dt * (sum_i aD(s,i) F_d(i) + aA(s,i) F_a(i)) [+ buoyancy].
// The buoyancy of the current stage is added after the temperature solve.
// ---------------------------------------------------------------------------
__global__ void stage_rhs_kernel(StageArgs a) {
  const size_t total = (size_t)a.R * a.M * a.B;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(e % a.B);
    const size_t rm = e / a.B;
    const int m = (int)(rm % a.M);
    const int r = (int)(rm / a.M);
    const double dt = a.dt;
    {
      double2 fd = make_double2(0, 0), fa = make_double2(0, 0);
      for (int i = 0; i < a.st; ++i) {
        const double2 q = a.fdt[i][e];
        fd.x += a.aD[i] * q.x; fd.y += a.aD[i] * q.y;
      }
      for (int i = 0; i < a.st; ++i) {
        const double2 q = a.fat[i][e];
        fa.x += a.aA[i] * q.x; fa.y += a.aA[i] * q.y;
      }
      const double2 y0 = a.t0[e];
      double2 rhs = make_double2(y0.x + dt * (fd.x + fa.x), y0.y + dt * (fd.y + fa.y));
      if (r == 0) rhs = make_double2(m == 0 ? 1.0 : 0.0, 0.0);
      if (r == a.R - 1) rhs = make_double2(0.0, 0.0);
      a.rhs_t[e] = rhs;
    }
    double2 fd = make_double2(0, 0), fa = make_double2(0, 0), fb = make_double2(0, 0);
    for (int i = 0; i < a.st; ++i) {
      const double2 q = a.fdw[i][e];
      fd.x += a.aD[i] * q.x; fd.y += a.aD[i] * q.y;
    }
    for (int i = 0; i < a.st; ++i) {
      const double2 q = a.faw[i][e];
      fa.x += a.aA[i] * q.x; fa.y += a.aA[i] * q.y;
    }
    if (m == 0) {
      const double y0 = a.u0[(size_t)r * a.B + b];
      double rhs = y0 + dt * (fd.x + fa.x);
      if (r == 0 || r == a.R - 1) rhs = 0.0;
      a.rhs_w[e] = make_double2(rhs, 0.0);
    } else {
      for (int i = 0; i < a.st; ++i) {
        const double2 q = a.buo[i][e];
        const double c = a.buo_imp ? a.aD[i] : a.aA[i];
        fb.x += c * q.x; fb.y += c * q.y;
      }
      const double2 y0 = a.w0[e];
      double2 rhs = make_double2(y0.x + dt * (fd.x + fa.x + fb.x), y0.y + dt * (fd.y + fa.y + fb.y));
      if (r == 0 || r == a.R - 1) rhs = make_double2(0.0, 0.0);
      a.rhs_w[e] = rhs;
    }
  }
}

cudaError_t launch_stage_rhs(const StageArgs& a, cudaStream_t s) {
  stage_rhs_kernel<<<ew_grid((size_t)a.R * a.M * a.B), 256, 0, s>>>(a);
  return cudaGetLastError();
}

// Stage derivatives (RHS_construct_stage, src/fourierloop_imexrk.F90:403-497
// with src/rhs_create_imexrk.F90): advective -N, diffusive L f, and the
// stage-1 buoyancy.
__global__ void stage_deriv_kernel(StageArgs a) {
  const size_t total = (size_t)a.R * a.M * a.B;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total;
       e += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(e % a.B);
    const size_t rm = e / a.B;
    const int m = (int)(rm % a.M);
    const int r = (int)(rm / a.M);
    const double ir = a.inv_r[r], ir2 = a.inv_r2[r];
    const double dm = (double)m, mm = dm * dm;
    {
      const double2 p = a.ntp[e], q = a.ntr[e], dq = a.dntr[e];
      a.fat_out[e] = make_double2(-(-dm * ir * p.y + dq.x + ir * q.x), -(dm * ir * p.x + dq.y + ir * q.y));
      const double2 T = a.t[e], L = a.lt[e];
      const double ip = a.inv_pr[b];
      a.fdt_out[e] = make_double2(ip * (L.x - mm * ir2 * T.x), ip * (L.y - mm * ir2 * T.y));
    }
    if (m == 0) {
      const size_t rb = (size_t)r * a.B + b;
      a.faw_out[e] = make_double2(-a.nwr[e].x, 0.0);
      const double u = a.up[e].x;
      a.fdw_out[e] = make_double2(a.lu0[rb].x - ir2 * u, 0.0);
    } else {
      const double2 p = a.nwp[e], q = a.nwr[e], dq = a.dnwr[e];
      a.faw_out[e] = make_double2(-(-dm * ir * p.y + dq.x + ir * q.x), -(dm * ir * p.x + dq.y + ir * q.y));
      const double2 W = a.w[e], L = a.lw[e];
      a.fdw_out[e] = make_double2(L.x - mm * ir2 * W.x, L.y - mm * ir2 * W.y);
      if (a.buo_out) {
        const double2 T = a.t[e];
        const double f = dm * ir;
        a.buo_out[e] = make_double2(a.ra_pr[b] * f * T.y, -a.ra_pr[b] * f * T.x);
      }
    }
  }
}

cudaError_t launch_stage_deriv(const StageArgs& a, cudaStream_t s) {
  stage_deriv_kernel<<<ew_grid((size_t)a.R * a.M * a.B), 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Layout transforms and small helpers
// ---------------------------------------------------------------------------
__global__ void scatter_instance_kernel(int R, int M, int B, int b, const double2* src, double2* dst) {
  const int n = R * M;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int r = i / M, m = i - r * M;  // src index m + M r (Fortran (M,R))
    dst[((size_t)r * M + m) * B + b] = src[i];
  }
}
__global__ void gather_instance_kernel(int R, int M, int B, int b, const double2* src, double2* dst) {
  const int n = R * M;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int r = i / M, m = i - r * M;
    dst[i] = src[((size_t)r * M + m) * B + b];
  }
}
cudaError_t launch_scatter_instance(int R, int M, int B, int b, const double2* src, double2* dst,
                                    cudaStream_t s) {
  scatter_instance_kernel<<<ew_grid((size_t)R * M), 256, 0, s>>>(R, M, B, b, src, dst);
  return cudaGetLastError();
}
// All B columns at once: src holds the B instances' Fortran (M, R) arrays
// back to back in slot order; the slot index runs fastest over the threads
// so the stores to the batched (R, M, B) layout are coalesced.
__global__ void scatter_columns_kernel(int R, int M, int B, const double2* __restrict__ src,
                                      double2* __restrict__ dst) {
  const size_t rm = (size_t)R * M, n = rm * B;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t e = i / B;  // r * M + m
    const int b = (int)(i - e * B);
    dst[i] = src[(size_t)b * rm + e];
  }
}
cudaError_t launch_scatter_columns(int R, int M, int B, const double2* src, double2* dst, cudaStream_t s) {
  scatter_columns_kernel<<<ew_grid((size_t)R * M * B), 256, 0, s>>>(R, M, B, src, dst);
  return cudaGetLastError();
}
cudaError_t launch_gather_instance(int R, int M, int B, int b, const double2* src, double2* dst,
                                   cudaStream_t s) {
  gather_instance_kernel<<<ew_grid((size_t)R * M), 256, 0, s>>>(R, M, B, b, src, dst);
  return cudaGetLastError();
}
__global__ void extract_mode0_kernel(int R, int M, int B, const double2* src, double* dst) {
  const int n = R * B;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int r = i / B, b = i - r * B;
    dst[i] = src[(size_t)r * M * B + b].x;
  }
}
cudaError_t launch_extract_mode0(int R, int M, int B, const double2* src, double* dst, cudaStream_t s) {
  extract_mode0_kernel<<<ew_grid((size_t)R * B), 256, 0, s>>>(R, M, B, src, dst);
  return cudaGetLastError();
}

// dgetrs 'N' (src/algebra_lapack.F90:36-37) for many systems: row
// interchanges, unit-lower forward substitution, upper back substitution,
// in the column order of the reference BLAS dtrsm.  One warp per right-hand
// side; the column updates are spread over the lanes.
__global__ void getrs_kernel(int n, int nsys, int nrhs, const double* lu, const int* ipiv, double* b) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= nsys * nrhs) return;
  const int sys = warp / nrhs;
  const double* A = lu + (size_t)sys * n * n;
  const int* pv = ipiv + (size_t)sys * n;
  double* x = b + (size_t)warp * n;
  if (lane == 0)
    for (int i = 0; i < n; ++i) {
      const int p = pv[i] - 1;
      if (p != i) { const double t = x[i]; x[i] = x[p]; x[p] = t; }
    }
  __syncwarp();
  for (int j = 0; j < n; ++j) {
    const double xj = x[j];
    __syncwarp();
    if (xj != 0.0)
      for (int i = j + 1 + lane; i < n; i += 32) x[i] -= xj * A[(size_t)j * n + i];
    __syncwarp();
  }
  for (int j = n - 1; j >= 0; --j) {
    double xj = x[j];
    __syncwarp();
    if (xj != 0.0) {
      xj = xj / A[(size_t)j * n + j];
      __syncwarp();
      if (lane == 0) x[j] = xj;
      for (int i = lane; i < j; i += 32) x[i] -= xj * A[(size_t)j * n + i];
    }
    __syncwarp();
  }
}

cudaError_t launch_getrs_batched(int n, int nsys, int nrhs, const double* lu, const int* ipiv,
                                 double* b, cudaStream_t s) {
  const int warps = nsys * nrhs;
  const int threads = 128;
  const int grid = (warps * 32 + threads - 1) / threads;
  getrs_kernel<<<grid, threads, 0, s>>>(n, nsys, nrhs, lu, ipiv, b);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// FP64 FMA throughput (the roofline denominator of every kernel above).
// ---------------------------------------------------------------------------
__global__ void fp64_peak_kernel(double* out, int iters, double a, double c) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x0 = fma(x0, a, c); x1 = fma(x1, a, c); x2 = fma(x2, a, c); x3 = fma(x3, a, c);
      x4 = fma(x4, a, c); x5 = fma(x5, a, c); x6 = fma(x6, a, c); x7 = fma(x7, a, c);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

double measure_fp64_peak() {
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = nsm * 4, threads = 256, iters = 200;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fp64_peak_kernel<<<blocks, threads>>>(out, 20, 1.0000001, 1e-9);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    fp64_peak_kernel<<<blocks, threads>>>(out, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
  return flops / (best * 1e-3) / 1e9;
}

}  // namespace falcon

namespace falcon {

// out[c][i] = sum_k A[i*n + k] * in[c][k] for complex columns (A real,
// row-major n x n): the Chebyshev transforms as dense operators.
__global__ void apply_cols_kernel(int n, int ncol, const double* A, const double2* in, double2* out) {
  const int c = blockIdx.y;
  const double2* x = in + (size_t)c * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double sr = 0.0, si = 0.0;
    for (int k = 0; k < n; ++k) {
      const double a = A[(size_t)i * n + k];
      const double2 v = x[k];
      sr = fma(a, v.x, sr);
      si = fma(a, v.y, si);
    }
    out[(size_t)c * n + i] = make_double2(sr, si);
  }
}

cudaError_t launch_apply_cols(int n, int ncol, const double* A, const double2* in, double2* out, cudaStream_t s) {
  dim3 grid((n + 127) / 128, ncol);
  apply_cols_kernel<<<grid, 128, 0, s>>>(n, ncol, A, in, out);
  return cudaGetLastError();
}

// dst[row][j] = map[j] >= 0 ? src[row][map[j]] : 0 (instance-column remap of
// a [rows][B] array, elements of `ew` doubles).
__global__ void remap_cols_kernel(const double* src, double* dst, size_t rows, int bs, int bd, int ew,
                                  const int* map) {
  const size_t total = rows * (size_t)bd * ew;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int q = (int)(i % ew);
    const size_t rj = i / ew;
    const int j = (int)(rj % bd);
    const size_t row = rj / bd;
    const int sj = map[j];
    dst[i] = (sj >= 0 && src) ? src[(row * bs + sj) * ew + q] : 0.0;
  }
}

cudaError_t launch_remap_cols(const double* src, double* dst, size_t rows, int bs, int bd, int ew, const int* map,
                              cudaStream_t s) {
  const size_t total = rows * (size_t)bd * ew;
  size_t g = (total + 255) / 256;
  if (g > 152 * 64) g = 152 * 64;
  if (g == 0) g = 1;
  remap_cols_kernel<<<(int)g, 256, 0, s>>>(src, dst, rows, bs, bd, ew, map);
  return cudaGetLastError();
}

}  // namespace falcon

namespace falcon {

// Column b of a [rows][B] array (ew doubles per element): dst = src, or 0
// when src is null.  Touches only that column.
__global__ void col_op_kernel(const double* src, double* dst, size_t rows, int B, int b, int ew) {
  const size_t total = rows * ew;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t row = i / ew;
    const int q = (int)(i % ew);
    const size_t e = (row * B + b) * ew + q;
    dst[e] = src ? src[e] : 0.0;
  }
}

cudaError_t launch_col_op(const double* src, double* dst, size_t rows, int B, int b, int ew, cudaStream_t s) {
  size_t g = (rows * ew + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  if (g == 0) g = 1;
  col_op_kernel<<<(int)g, 256, 0, s>>>(src, dst, rows, B, b, ew);
  return cudaGetLastError();
}

}  // namespace falcon

namespace falcon {

// FP64 tensor-core (mma.sync m8n8k4 f64) throughput, measured to decide
// between DMMA and DFMA for the per-mode contractions.
__global__ void dmma_peak_kernel(double* out, int iters) {
  const double a = threadIdx.x * 1e-3, b = 1.0 - a;
  double c[4][2];
#pragma unroll
  for (int j = 0; j < 4; ++j) { c[j][0] = 0.0; c[j][1] = 0.0; }
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                     : "+d"(c[j][0]), "+d"(c[j][1]) : "d"(a), "d"(b));
    }
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 4; ++j) s += c[j][0] + c[j][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

double measure_fp64_mma_peak() {
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = nsm * 4, threads = 128, iters = 100;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  dmma_peak_kernel<<<blocks, threads>>>(out, 10);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    dmma_peak_kernel<<<blocks, threads>>>(out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  const double flops = 2.0 * 8 * 8 * 4 * 16 * 4 * (double)iters * blocks * (threads / 32);
  return flops / (best * 1e-3) / 1e9;
}

}  // namespace falcon

// ---------------------------------------------------------------------------
// Allocation-free nonlinear pass.
//
// falcon_nonlin_dev builds its FFT tables (P twiddles, P digit-reversal
// positions) in device memory it allocates per call.  Some callers must not
// have the library allocate: hosts that own every byte of device memory
// through their own pre-sized pool (the way the serving loop budgets HBM per
// request) and cannot let a library grow the footprint behind their back,
// and hosts stepping in tight loops where a cudaMalloc/cudaFree pair would
// synchronise the device on every call.  For them the tables live in the
// fixed file-scope array below, sized for Np_max = 3*Nm_max <= 4096.
// ---------------------------------------------------------------------------
namespace falcon {

constexpr int kNoAllocMaxP = 4096;
// twiddles (kNoAllocMaxP double2) followed by positions (kNoAllocMaxP int):
// 80 KiB, held by every GPU that loads the library until the process exits.
constexpr size_t kNoAllocScratchBytes = (size_t)kNoAllocMaxP * (sizeof(double2) + sizeof(int));
static __device__ __align__(256) unsigned char g_nonlin_scratch[kNoAllocScratchBytes];

// Per-device address of g_nonlin_scratch (host code may not use the symbol
// itself as a device pointer), looked up once per device under a
// std::once_flag, so host threads making their first call together do not
// race on it.
static std::once_flag g_scratch_once[64];
static void* g_scratch_addr[64] = {nullptr};

// Host staging of the tables: filled and copied under the mutex.  A copy from
// pageable host memory has consumed its source when cudaMemcpyAsync returns,
// so the buffer is free again once the copies are issued.
static std::mutex g_noalloc_host_mu;
static double2 g_noalloc_tw_h[kNoAllocMaxP];
static int g_noalloc_pos_h[kNoAllocMaxP];

}  // namespace falcon

extern "C" const char* falcon_last_error(void);
namespace falcon { int set_error_message(const char* msg); }

// Same computation, device layout and bits as falcon_nonlin_dev, without any
// device allocation: the FFT tables are built on the host by the same code
// as the allocating form (fft_tables_host) and copied into a fixed static
// device array.
//  - Asynchronous on `stream`: the call returns once the table copies and
//    the kernel are queued (the table copies, from pageable host memory,
//    wait for earlier work on the stream).  Synchronise the stream before
//    reading the outputs; a kernel fault is reported there, not in the
//    return code.  (falcon_nonlin_dev synchronises before it returns.)
//  - The first call on a device looks up that device's address of the array
//    (cudaGetSymbolAddress, with the device current, once per device); make
//    that first call before any stream capture on that device.
//  - Every call overwrites the whole table region it uses, so no state
//    carries over between calls; but all calls on a device share the one
//    array, so calls whose kernels overlap on the GPU (different streams, or
//    host threads) race on it and must be serialised by the caller.
//  - Limit: Np_max = 3*nm <= 4096 (nm <= 1365); larger sizes return
//    FALCON_EINVAL (-1).
extern "C" int falcon_nonlin_noalloc_dev(int nr, int nm, int nb, const double* t_dev, const double* omg_dev,
                                         const double* up_dev, const double* ur_dev, double* uphi_t_dev,
                                         double* ur_t_dev, double* uphi_omg_dev, double* ur_omg_dev,
                                         void* stream) {
  using namespace falcon;
  if (nr < 1 || nm < 1 || nb < 1) { set_error_message("falcon_nonlin_noalloc_dev: invalid sizes"); return -1; }
  const int P = 3 * nm;
  if (P > kNoAllocMaxP) {
    set_error_message("falcon_nonlin_noalloc_dev: Np_max = 3*Nm_max exceeds the 4096-point scratch limit");
    return -1;
  }
  FftPlan plan{};
  if (make_fft_plan(P, &plan) != 0) {
    set_error_message("falcon_nonlin_noalloc_dev: 3*Nm_max has a prime factor above 64");
    return -1;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) { set_error_message("falcon_nonlin_noalloc_dev: no current device"); return -2; }
  std::call_once(g_scratch_once[dev], [dev] {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_nonlin_scratch) == cudaSuccess) g_scratch_addr[dev] = ptr;
  });
  if (!g_scratch_addr[dev]) {
    set_error_message("falcon_nonlin_noalloc_dev: cudaGetSymbolAddress failed on this device");
    return -2;
  }
  e = init_dft_tables();
  if (e != cudaSuccess) { set_error_message(cudaGetErrorString(e)); return -2; }
  double2* tw = reinterpret_cast<double2*>(g_scratch_addr[dev]);
  int* pos = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(g_scratch_addr[dev]) +
                                    (size_t)kNoAllocMaxP * sizeof(double2));
  cudaStream_t s = (cudaStream_t)stream;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_host_mu);
    fft_tables_host(plan, g_noalloc_tw_h, g_noalloc_pos_h);
    e = cudaMemcpyAsync(tw, g_noalloc_tw_h, sizeof(double2) * (size_t)P, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(pos, g_noalloc_pos_h, sizeof(int) * (size_t)P, cudaMemcpyHostToDevice, s);
  }
  if (e != cudaSuccess) { set_error_message(cudaGetErrorString(e)); return -2; }
  NonlinArgs a{};
  a.R = nr; a.M = nm + 1; a.B = nb; a.Nm = nm;
  a.plan = plan; a.tw = tw; a.pos = pos;
  a.t = reinterpret_cast<const double2*>(t_dev); a.w = reinterpret_cast<const double2*>(omg_dev);
  a.up = reinterpret_cast<const double2*>(up_dev); a.ur = reinterpret_cast<const double2*>(ur_dev);
  a.ntp = reinterpret_cast<double2*>(uphi_t_dev); a.ntr = reinterpret_cast<double2*>(ur_t_dev);
  a.nwp = reinterpret_cast<double2*>(uphi_omg_dev); a.nwr = reinterpret_cast<double2*>(ur_omg_dev);
  e = launch_nonlin(a, s);
  if (e != cudaSuccess) { set_error_message(cudaGetErrorString(e)); return -2; }
  return 0;
}

namespace falcon {

// writeKE_spectral (src/output.F90:122-324) for every instance of a group,
// one block per instance.  wq[r] is the radInt functional (src/integ.F90:
// 36-76) written as weights on the values: radInt(f) = sum_r wq[r] f(r).
// d1_0 / d1_R are rows 0 and R-1 of the physical d/dr matrix (Nusselt from
// dT0/dr at the walls, src/output.F90:259-263).  tprev is the temperature of
// the last nonlinear pass, which the reference multiplies with the current
// u_r for the buoyancy power (src/output.F90:211, :302).  Output per
// instance (8 doubles): ke, ke_r, ke_phi, ke_upbar, nu_top, nu_bot, vis, buo.
// Phase 1, one block per radial row r and 32 instance columns: threads
// (tx, ty) take column tx and the modes m = ty (mod 8), so every load of a
// warp is one coalesced run of 32 columns.  Per (r, b) it writes the
// radially weighted sums (k = 0..6) and the unweighted u_phi power (k = 7)
// to part[(k R + r) B + b].
__global__ void __launch_bounds__(256) diag_rows_kernel(DiagArgs a) {
  const int r = blockIdx.x, tx = threadIdx.x, ty = threadIdx.y;
  const int R = a.R, M = a.M, B = a.B;
  const int b = blockIdx.y * 32 + tx;
  __shared__ double part[8][4][33];
  double ur2 = 0.0, up2 = 0.0, w2 = 0.0, urt = 0.0;
  if (b < B) {
    for (int m = ty; m < M; m += 8) {
      const size_t e = ((size_t)r * M + m) * B + b;
      const double2 u = a.ur[e], v = a.up[e], o = a.w[e], tp = a.tprev[e];
      ur2 += u.x * u.x + u.y * u.y;
      up2 += v.x * v.x + v.y * v.y;
      if (m == 0) {
        w2 += o.x * o.x - o.y * o.y;
        urt += u.x * tp.x;
      } else {
        w2 += 2.0 * (o.x * o.x + o.y * o.y);
        urt += 2.0 * (u.x * tp.x + u.y * tp.y);
      }
    }
  }
  part[ty][0][tx] = ur2; part[ty][1][tx] = up2; part[ty][2][tx] = w2; part[ty][3][tx] = urt;
  __syncthreads();
  if (ty != 0 || b >= B) return;
  for (int y = 1; y < 8; ++y) {
    ur2 += part[y][0][tx]; up2 += part[y][1][tx]; w2 += part[y][2][tx]; urt += part[y][3][tx];
  }
  const double q = a.wq[r];
  const size_t e0 = ((size_t)r * M) * B + b;
  const double u0 = a.up[e0].x, t0 = a.t[e0].x;
  double* P = a.part + (size_t)r * B + b;
  const size_t ks = (size_t)R * B;
  P[0 * ks] = q * ur2;
  P[1 * ks] = q * up2;
  P[2 * ks] = q * u0 * u0;
  P[3 * ks] = q * w2;
  P[4 * ks] = q * urt;
  P[5 * ks] = a.d1_0[r] * t0;
  P[6 * ks] = a.d1_R[r] * t0;
  P[7 * ks] = up2;
}

// Phase 2, one warp per instance: lane l sums the radial rows l, l + 32,
// ..., then a fixed shuffle tree; then the eight diagnostics of
// writeKE_spectral / Nusselt (8 doubles per instance).
__global__ void diag_sum_kernel(DiagArgs a) {
  const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  const int R = a.R, B = a.B;
  if (b >= B) return;
  const size_t ks = (size_t)R * B;
  double t[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int r = lane; r < R; r += 32)
#pragma unroll
    for (int k = 0; k < 7; ++k) t[k] += a.part[k * ks + (size_t)r * B + b];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < 7; ++k) t[k] += __shfl_xor_sync(0xffffffffu, t[k], o);
  if (lane != 0) return;
  const double s_in = a.part[7 * ks + b], s_out = a.part[7 * ks + (size_t)(R - 1) * B + b];
  const double two_pi = 2.0 * a.pi;
  double* o = a.out + (size_t)b * 8;
  o[0] = two_pi * (t[0] + t[1]);
  o[1] = two_pi * t[0];
  o[2] = two_pi * t[1];
  o[3] = two_pi * t[2];
  o[4] = t[6] / a.nu_top_den;
  o[5] = t[5] / a.nu_bot_den;
  o[6] = two_pi * t[3] - (a.mbc_sf ? (4.0 * a.pi * 2.0 * s_out - 4.0 * a.pi * 2.0 * s_in) : 0.0);
  o[7] = two_pi * a.ra_pr[b] * t[4];
}

cudaError_t launch_diagnostics(const DiagArgs& a, cudaStream_t s) {
  diag_rows_kernel<<<dim3(a.R, (a.B + 31) / 32), dim3(32, 8), 0, s>>>(a);
  diag_sum_kernel<<<(a.B + 3) / 4, 128, 0, s>>>(a);
  return cudaGetLastError();
}

// calculate_spectra (src/output.F90:327-355) of every instance, one thread
// per (mode, instance): 4 pi radInt of |ur_m ur_m + up_m up_m| (complex
// squares, as the reference forms them) and of |T_m|; wq are the radInt
// weights on the values.  Output [b][m].
__global__ void spectra_kernel(int R, int M, int B, const double2* t, const double2* ur, const double2* up,
                               const double* wq, double four_pi, double* ke, double* ts) {
  const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)M * B) return;
  const int m = (int)(idx / B), b = (int)(idx - (long)m * B);
  double sk = 0.0, st = 0.0;
  for (int r = 0; r < R; ++r) {
    const size_t e = ((size_t)r * M + m) * B + b;
    const double2 u = ur[e], v = up[e], T = t[e];
    const double ar = u.x * u.x - u.y * u.y, ai = u.x * u.y + u.y * u.x;
    const double br = v.x * v.x - v.y * v.y, bi = v.x * v.y + v.y * v.x;
    sk += wq[r] * hypot(ar + br, ai + bi);
    st += wq[r] * hypot(T.x, T.y);
  }
  ke[(size_t)b * M + m] = four_pi * sk;
  ts[(size_t)b * M + m] = four_pi * st;
}

cudaError_t launch_spectra(int R, int M, int B, const double2* t, const double2* ur, const double2* up,
                           const double* wq, double four_pi, double* ke, double* ts, cudaStream_t s) {
  spectra_kernel<<<ew_grid((size_t)M * B), 256, 0, s>>>(R, M, B, t, ur, up, wq, four_pi, ke, ts);
  return cudaGetLastError();
}

// The u_phi balance of writeKE_spectral (src/output.F90:145-228), one thread
// per (radius, instance): d(up_0)/dt against the value at the start of the
// step (up0_prev), the advection -(ur d(up)/dr + ur up / r) summed over
// modes as the reference forms it (the m = 0 product, conjugate pairs for
// m >= 1; real parts), and the diffusion d2 up_0/dr2 + (d up_0/dr) / r -
// up_0 / r^2 = (Lp up_0) - up_0 / r^2.  d1up = d(up)/dr of every mode.
// Output [b][r][3].
__global__ void upbalance_kernel(int R, int M, int B, const double2* ur, const double2* up, const double2* d1up,
                                 const double* up0_prev, const double* Lp, const double* inv_r,
                                 const double* inv_r2, double dt, double* out) {
  const long idx = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (idx >= (long)R * B) return;
  const int r = (int)(idx / B), b = (int)(idx - (long)r * B);
  double p = 0.0, q = 0.0;
  for (int m = 0; m < M; ++m) {
    const size_t e = ((size_t)r * M + m) * B + b;
    const double2 u = ur[e], w = up[e], dw = d1up[e];
    if (m == 0) {
      p += u.x * w.x - u.y * w.y;
      q += u.x * dw.x - u.y * dw.y;
    } else {
      p += 2.0 * (u.x * w.x + u.y * w.y);
      q += 2.0 * (u.x * dw.x + u.y * dw.y);
    }
  }
  const size_t e0 = ((size_t)r * M) * B + b;
  const double u0 = up[e0].x;
  double lap = 0.0;
  for (int k = 0; k < R; ++k) lap += Lp[r + (size_t)R * k] * up[((size_t)k * M) * B + b].x;
  double* o = out + ((size_t)b * R + r) * 3;
  o[0] = (u0 - up0_prev[(size_t)r * B + b]) / dt;
  o[1] = -(q + inv_r[r] * p);
  o[2] = lap - inv_r2[r] * u0;
}

cudaError_t launch_upbalance(int R, int M, int B, const double2* ur, const double2* up, const double2* d1up,
                             const double* up0_prev, const double* Lp, const double* inv_r, const double* inv_r2,
                             double dt, double* out, cudaStream_t s) {
  upbalance_kernel<<<ew_grid((size_t)R * B), 256, 0, s>>>(R, M, B, ur, up, d1up, up0_prev, Lp, inv_r, inv_r2, dt,
                                                          out);
  return cudaGetLastError();
}

}  // namespace falcon

namespace falcon {

// Assembly_stage for schemes that are not stiffly accurate
// (src/fourierloop_imexrk.F90:499-651), elementwise part: y_n = y_0 +
// dt sum_i (bA_i F_a(i) + bD_i F_d(i)) for T, uphi_bar (m = 0) and the
// interior vorticity (m >= 1, with the buoyancy under bD), then the psi
// Poisson right-hand side -omega (zero boundary rows) into rhs_w.
__global__ void assembly_kernel(AsmArgs a) {
  const size_t total = (size_t)a.R * a.M * a.B;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(e % a.B);
    const size_t rm = e / a.B;
    const int m = (int)(rm % a.M);
    const int r = (int)(rm / a.M);
    double2 f = make_double2(0.0, 0.0);
    for (int i = 0; i < a.ns; ++i) {
      const double2 qa = a.fat[i][e], qd = a.fdt[i][e];
      f.x = f.x + a.bA[i] * qa.x + a.bD[i] * qd.x;
      f.y = f.y + a.bA[i] * qa.y + a.bD[i] * qd.y;
    }
    double2 t = a.t0[e];
    t.x = t.x + a.dt * f.x;
    t.y = t.y + a.dt * f.y;
    if (r == 0) t = make_double2(m == 0 ? 1.0 : 0.0, 0.0);
    if (r == a.R - 1) t = make_double2(0.0, 0.0);
    a.t0[e] = t;
    if (m == 0) {
      double fu = 0.0;
      for (int i = 0; i < a.ns; ++i) fu = fu + a.bA[i] * a.faw[i][e].x + a.bD[i] * a.fdw[i][e].x;
      const size_t rb = (size_t)r * a.B + b;
      double u = a.u0[rb] + a.dt * fu;
      if (r == 0 || r == a.R - 1) u = 0.0;
      a.u0[rb] = u;
      a.rhs_w[e] = make_double2(0.0, 0.0);
    } else {
      double2 w = a.w0[e];
      if (r > 0 && r < a.R - 1) {
        double2 g = make_double2(0.0, 0.0);
        for (int i = 0; i < a.ns; ++i) {
          const double2 qa = a.faw[i][e], qd = a.fdw[i][e], qb = a.buo[i][e];
          g.x = g.x + a.bA[i] * qa.x + a.bD[i] * qd.x + a.bD[i] * qb.x;
          g.y = g.y + a.bA[i] * qa.y + a.bD[i] * qd.y + a.bD[i] * qb.y;
        }
        w.x = w.x + a.dt * g.x;
        w.y = w.y + a.dt * g.y;
        a.w0[e] = w;
        a.rhs_w[e] = make_double2(-1.0 * w.x, -1.0 * w.y);
      } else {
        a.rhs_w[e] = make_double2(0.0, 0.0);
      }
    }
  }
}

// After the psi solve: u_r = i m psi/r (m >= 1); mode 0: omega = ubar/r +
// d ubar/dr, u_phi = ubar, u_r = 0 (src/fourierloop_imexrk.F90:556-572).
__global__ void assembly_post_kernel(int R, int M, int B, const double* inv_r, const double2* psi,
                                     const double* u0, const double* du0, double2* ur, double2* up, double2* w0) {
  const size_t total = (size_t)R * M * B;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(e % B);
    const size_t rm = e / B;
    const int m = (int)(rm % M);
    const int r = (int)(rm / M);
    if (m > 0) {
      const double2 ps = psi[e];
      const double f = 1.0 * (double)m * inv_r[r];
      ur[e] = make_double2(-f * ps.y, f * ps.x);
    } else {
      const size_t rb = (size_t)r * B + b;
      const double u = u0[rb];
      up[e] = make_double2(u, 0.0);
      ur[e] = make_double2(0.0, 0.0);
      w0[e] = make_double2(u * inv_r[r] + du0[rb], 0.0);
    }
  }
}

cudaError_t launch_assembly(const AsmArgs& a, cudaStream_t s) {
  size_t n = (size_t)a.R * a.M * a.B;
  size_t g = (n + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  assembly_kernel<<<(int)(g ? g : 1), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_assembly_post(int R, int M, int B, const double* inv_r, const double2* psi, const double* u0,
                                 const double* du0, double2* ur, double2* up, double2* w0, cudaStream_t s) {
  size_t n = (size_t)R * M * B;
  size_t g = (n + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  assembly_post_kernel<<<(int)(g ? g : 1), 256, 0, s>>>(R, M, B, inv_r, psi, u0, du0, ur, up, w0);
  return cudaGetLastError();
}

}  // namespace falcon
