// FP64 GEMM Y = alpha * A * X on the bf16 tensor cores (mma.sync m16n8k16,
// FP32 accumulation) by exact integer slicing (the Ozaki scheme).
//
// On GB300 the FP64 pipe (~1.2 TFLOP/s) is ~500x slower than bf16 MMA
// (~600 TFLOP/s measured for mma.sync), and DMMA shares the FP64 rate.  So
// the operator contractions of the time step run as integer products:
//   - A row i with |a| < 2^e_i and an X column n with |x| < 2^f_n are cut
//     into S signed W-bit integers (exact in bf16):
//       a = 2^e_i sum_s alpha_s 2^(-W(s+1)),  x = 2^f_n sum_t beta_t 2^(-W(t+1)),
//     dropping bits below 2^(e - S W);
//   - P_st = sum_k alpha_s beta_t is exact in FP32, and so is
//     Q_d = sum_{s+t=d} P_st for d <= D, one FP32 register set per d: with
//     W = 6, S = 10, D = 9 for K <= 257 (10 pairs x 257 x 63^2 < 2^24), with
//     W = 7, S = 9, D = 8 for K <= 112 (9 x 112 x 127^2 < 2^24; 45 pairs
//     instead of 55).  The pairs s + t > D weigh less than 2^-56 of
//     max|A_ik| max|X_kn| per product;
//   - Y = 2^kH H + 2^kL L, H and L the high and low diagonals combined
//     exactly in 64-bit integers, scaled exactly through their bits and
//     added once in FP64 (OzCfg in falcon_slices.cuh).
// The error is of the order of K 2^-56 max_k|A_ik| max_k|X_kn|, the level of
// an FP64 GEMM's rounding; each output depends only on its own row and
// column, and every FP32 sum is exact, so results do not depend on the
// launch shape or on the other columns of the batch.
//
// The operators are constant: their slices are made once (launch_oz_slice_rows)
// when an operator set is built.  X is sliced per contraction into slice
// planes (launch_oz_slice_cols); contractions sharing one X reuse them.
#include <cuda_bf16.h>
#include <stdint.h>

#include <atomic>

#include "falcon_internal.h"
#include "falcon_slices.cuh"

namespace falcon {

namespace {

}  // namespace

// One thread per (entry, row): the row exponent, then the slices of each
// element (format W).  Layout [nb][S][KP/8][rowsP][8]: element (row r, k)
// of a slice plane at ((k/8) rowsP + r) 8 + k%8, so that 8 consecutive k
// of a row are 16 contiguous bytes and a k group of all rows is one
// contiguous block (the tile shape both tensor-core kernels stage).  The
// caller zeroes S (padding rows and K columns stay zero).
template <int W>
__global__ void oz_slice_rows_kernel(const double* A, long lda, long sA, int rows, int K, int nb, uint16_t* S,
                                     int* ex, int rowsP, int KP) {
  using C = OzCfg<W>;
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= (long)nb * rows) return;
  const int z = (int)(t / rows), r = (int)(t - (long)z * rows);
  const double* a = A + (size_t)z * sA + r;
  int mx = 0;
  for (int k = 0; k < K; ++k) mx = max(mx, biased_exp(a[(size_t)k * lda]));
  const int e = mx - 1022;  // |a| < 2^e for every entry of the row
  ex[(size_t)z * rowsP + r] = mx ? e : 0;
  uint16_t* s0 = S + (size_t)z * C::S * rowsP * KP + (size_t)r * 8;
  const size_t sls = (size_t)rowsP * KP;
  for (int k = 0; k < K; ++k) {
    const double v = a[(size_t)k * lda];
    const unsigned long long T = mx ? oz_magb<C::MAGB>(v, e) : 0ull;
    const size_t at = (size_t)(k >> 3) * rowsP * 8 + (k & 7);
#pragma unroll
    for (int sl = 0; sl < C::S; ++sl) s0[sl * sls + at] = (uint16_t)oz_slice_w<W>(T, v < 0, sl);
  }
}

cudaError_t launch_oz_slice_rows(const double* A, long lda, long sA, int rows, int K, int nb, uint16_t* S, int* ex,
                                 int rowsP, int KP, int w, cudaStream_t s) {
  const long n = (long)nb * rows;
  if (n <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((n + 127) / 128);
  if (w == 7) oz_slice_rows_kernel<7><<<grid, 128, 0, s>>>(A, lda, sA, rows, K, nb, S, ex, rowsP, KP);
  else oz_slice_rows_kernel<6><<<grid, 128, 0, s>>>(A, lda, sA, rows, K, nb, S, ex, rowsP, KP);
  return cudaGetLastError();
}

// Column slices of X: block (64 columns, batch entry); the column
// exponent from four strided partial maxima, then every (k, column) element
// cut into its slices (format W), written slice plane by slice plane
// (coalesced along the columns).
template <int W>
__global__ void __launch_bounds__(256) oz_slice_cols_kernel(const double* X, long ldx, long sX, int K, int N,
                                                            uint16_t* Xs, int* cexp, int KP, int Np) {
  using C = OzCfg<W>;
  __shared__ int ex[4][64];
  const int c = threadIdx.x & 63, kq = threadIdx.x >> 6;
  const int z = blockIdx.y, n = blockIdx.x * 64 + c;
  const double* Xz = X + (size_t)z * sX;
  int mx = 0;
  if (n < N)
    for (int k = kq; k < K; k += 4) mx = max(mx, biased_exp(Xz[(size_t)k * ldx + n]));
  ex[kq][c] = mx;
  __syncthreads();
  const int fb = max(max(ex[0][c], ex[1][c]), max(ex[2][c], ex[3][c]));
  if (kq == 0 && n < Np) cexp[(size_t)z * Np + n] = fb;
  if (n >= Np) return;
  uint16_t* xz = Xs + (size_t)z * C::S * KP * Np;
  for (int k = kq; k < KP; k += 4) {
    unsigned long long T = 0ull;
    bool neg = false;
    if (k < K && n < N && fb > 0) {
      const double v = Xz[(size_t)k * ldx + n];
      T = oz_magb<C::MAGB>(v, fb - 1022);
      neg = __double_as_longlong(v) < 0;
    }
#pragma unroll
    for (int sl = 0; sl < C::S; ++sl) xz[((size_t)sl * KP + k) * Np + n] = (uint16_t)oz_slice_w<W>(T, neg, sl);
  }
}

cudaError_t launch_oz_slice_cols(const double* X, long ldx, long sX, int K, int N, int batch, uint16_t* Xs,
                                 int* cexp, int KP, int Np, int w, cudaStream_t s) {
  if (N <= 0 || batch <= 0) return cudaSuccess;
  dim3 grid((Np + 63) / 64, batch);
  if (w == 7) oz_slice_cols_kernel<7><<<grid, 256, 0, s>>>(X, ldx, sX, K, N, Xs, cexp, KP, Np);
  else oz_slice_cols_kernel<6><<<grid, 256, 0, s>>>(X, ldx, sX, K, N, Xs, cexp, KP, Np);
  return cudaGetLastError();
}

namespace {

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned saddr = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(saddr), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}
__device__ __forceinline__ void ldsm_x2t(unsigned (&r)[2], const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(a));
}

}  // namespace

// Tiled slice GEMM (format W, OzCfg<W>).  Block: MT row tiles (16 rows) x
// NQ column groups (16 columns), each (row tile, column group) taken by
// 2 / NT warps of NT 16x8 tiles each; K in chunks of 16 staged in shared
// memory by cp.async two chunks deep (slices of A and X for all S slices of
// the chunk); fragments by ldmatrix from padded rows (48 and NQ*32+16 bytes:
// conflict-free).  Per chunk a warp does the slice-pair products s + t <= D
// (55 for W = 6, 45 for W = 7) on each of its tiles.  NT = 1 halves the
// accumulator registers (D + 1 diagonals x 4 per tile), so twice the warps
// fit on an SM.
// FX: the block cuts its own X columns (all of K, from the FP64 operand)
// into slice planes resident in shared memory, with the column exponents,
// instead of reading planes made by oz_slice_cols_kernel: the same slices,
// one launch and the planes' HBM round trip fewer.
template <int MT, int NQ, int NT, int MINB, int W, bool FX>
__global__ void __launch_bounds__(32 * MT * NQ * (2 / NT), MINB) oz_mma_kernel(GemmArgs q) {
  using C = OzCfg<W>;
  constexpr int SPLIT = 2 / NT;  // warps per (row tile, column group)
  constexpr int AROW = 24, XROW = NQ * 16 + 8;           // padded row lengths (bf16)
  constexpr int CW = NQ * 16;                            // columns of the block
  constexpr int ASTAGE = C::S * MT * 16 * AROW, XSTAGE = FX ? 0 : C::S * 16 * XROW;
  extern __shared__ __align__(16) uint16_t oz_panel[];   // [2][ASTAGE + XSTAGE] (+ FX: planes, exponents)
  const int z = blockIdx.z;
  const int col0 = blockIdx.x * CW, row0b = blockIdx.y * MT * 16;
  const uint16_t* Az = q.oz_s + (size_t)z * q.oz_sz + (size_t)(q.oz_row0 + row0b) * 8;
  const size_t aslice = (size_t)q.oz_rowsP * q.oz_KP;
  const uint16_t* Xz = FX ? nullptr : q.oz_xs + (size_t)z * C::S * q.oz_KP * q.oz_Np + col0;
  const size_t xslice = (size_t)q.oz_KP * q.oz_Np;
  const int tid = threadIdx.x, nthr = 32 * MT * NQ * SPLIT;
  uint16_t* xres = oz_panel + 2 * (ASTAGE + XSTAGE);                          // FX: [S][KP][XROW]
  int* cex_s = reinterpret_cast<int*>(xres + (FX ? (size_t)C::S * q.oz_KP * XROW : 0));  // FX: [CW]
  auto stage = [&](int k0, int buf) {
    uint16_t* Ap = oz_panel + buf * (ASTAGE + XSTAGE);
    uint16_t* Xp = Ap + ASTAGE;
    for (int i = tid; i < C::S * MT * 16 * 2; i += nthr) {        // A: (slice, row, half)
      const int h = i & 1, rr = (i >> 1) % (MT * 16), sl = (i >> 1) / (MT * 16);
      cp_async16(Ap + (sl * MT * 16 + rr) * AROW + 8 * h,
                 Az + sl * aslice + ((size_t)((k0 >> 3) + h) * q.oz_rowsP + rr) * 8);
    }
    if constexpr (!FX) {
      for (int i = tid; i < C::S * 16 * 2 * NQ; i += nthr) {      // X: (slice, k, 8-column chunk)
        const int cq = i % (2 * NQ), kk = (i / (2 * NQ)) % 16, sl = i / (2 * NQ * 16);
        cp_async16(Xp + (sl * 16 + kk) * XROW + 8 * cq, Xz + sl * xslice + (size_t)(k0 + kk) * q.oz_Np + 8 * cq);
      }
    }
    cp_commit();
  };
  const int warp = tid >> 5, lane = tid & 31, gid = lane >> 2, tig = lane & 3;
  const int wm = warp % MT, wr = warp / MT, wn = wr / SPLIT, nt0 = (wr % SPLIT) * NT;
  float acc[C::D + 1][NT][4];
#pragma unroll
  for (int d = 0; d <= C::D; ++d)
#pragma unroll
    for (int nt = 0; nt < NT; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[d][nt][i] = 0.f;
  const int nk = q.oz_KP / 16;
  stage(0, 0);
  if constexpr (FX) {
    // thread (row group g, column c): rows k = g, g + ng, ... of column c
    constexpr int NG = 32 * MT * NQ * SPLIT / CW;
    int* pmax = cex_s + CW;  // [NG][CW]
    const int c = tid % CW, g = tid / CW, n = col0 + c;
    const double* xc = q.X + (size_t)z * q.sX + n;
    int mx = 0;
    if (n < q.N)
      for (int k = g; k < q.K; k += NG) mx = max(mx, biased_exp(xc[(size_t)k * q.ldx]));
    pmax[g * CW + c] = mx;
    __syncthreads();
    int fb = 0;
    for (int j = 0; j < NG; ++j) fb = max(fb, pmax[j * CW + c]);
    if (g == 0) cex_s[c] = fb;
    for (int k = g; k < q.oz_KP; k += NG) {
      unsigned long long T = 0ull;
      bool neg = false;
      if (k < q.K && n < q.N && fb > 0) {
        const double v = xc[(size_t)k * q.ldx];
        T = oz_magb<C::MAGB>(v, fb - 1022);
        neg = __double_as_longlong(v) < 0;
      }
#pragma unroll
      for (int sl = 0; sl < C::S; ++sl) xres[((size_t)sl * q.oz_KP + k) * XROW + c] = (uint16_t)oz_slice_w<W>(T, neg, sl);
    }
  }
  for (int kc = 0; kc < nk; ++kc) {
    if (kc + 1 < nk) {
      stage((kc + 1) * 16, (kc + 1) & 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    const uint16_t* Ap = oz_panel + (kc & 1) * (ASTAGE + XSTAGE);
    // X rows of this chunk: slice t at Xp + t * xts (16 rows of XROW)
    const uint16_t* Xp = FX ? xres + (size_t)kc * 16 * XROW : Ap + ASTAGE;
    const size_t xts = FX ? (size_t)q.oz_KP * XROW : (size_t)16 * XROW;
    unsigned bf[C::S][NT][2];
#pragma unroll
    for (int t = 0; t < C::S; ++t)
#pragma unroll
      for (int nt = 0; nt < NT; ++nt)
        ldsm_x2t(bf[t][nt], Xp + t * xts + (lane & 15) * XROW + wn * 16 + (nt0 + nt) * 8);
#pragma unroll
    for (int sl = 0; sl < C::S; ++sl) {
      unsigned af[4];
      ldsm_x4(af, Ap + (sl * MT * 16 + wm * 16 + (lane & 15)) * AROW + (lane >> 4) * 8);
#pragma unroll
      for (int t = 0; t < C::S && sl + t <= C::D; ++t)
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) mma_bf16(acc[sl + t][nt], af[0], af[1], af[2], af[3], bf[t][nt][0], bf[t][nt][1]);
    }
    __syncthreads();  // every warp is done with this buffer before it is refilled
  }
  // recombination: Y = 2^kH H + 2^kL L (OzCfg), exact scalings and one FP64 add
  const bool scale_y = q.alpha != 1.0;  // one FP64 compare, not one per output
  const int* aex = q.oz_ex + (size_t)z * q.oz_rowsP + q.oz_row0;
  const int* cex = FX ? cex_s - col0 : q.oz_cexp + (size_t)z * q.oz_Np;
  double* Y = q.Y + (size_t)z * q.sY;
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) {
    const int n = col0 + wn * 16 + (nt0 + nt) * 8 + tig * 2;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = row0b + wm * 16 + gid + 8 * h;
      if (r >= q.rows || n >= q.N) continue;
      const int er = aex[r];
      double out[2];
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int i = 2 * h + j;
        auto qd = [&](int d) { return __float2int_rn(acc[d][nt][i]); };
        const long long H = oz_diag_sum<W, 0, C::HD>(qd), L = oz_diag_sum<W, C::HD + 1, C::D>(qd);
        const int fb = cex[n + j];
        const int kL = er + (fb - 1022) - 2 * C::MAGB + W * (2 * C::S - 2 - C::D);
        double y = fb > 0 ? oz_recombine_2t(H, L, kL, W * (C::D - C::HD)) : 0.0;
        if (fb == 2047) y = __longlong_as_double(0x7ff8000000000000LL);  // Inf or NaN in the column
        out[j] = scale_y ? q.alpha * y : y;
      }
      double* yp = Y + (size_t)r * q.ldy + n;
      if (n + 1 < q.N) {
        if ((reinterpret_cast<uintptr_t>(yp) & 15) == 0) {
          *reinterpret_cast<double2*>(yp) = make_double2(out[0], out[1]);
        } else {
          yp[0] = out[0];
          yp[1] = out[1];
        }
      } else {
        yp[0] = out[0];
      }
    }
  }
}

template <int MT, int NQ, int NT, int MINB, int W, bool FX>
static cudaError_t launch_oz_w(const GemmArgs& g, cudaStream_t s) {
  constexpr int S = OzCfg<W>::S, XROW = NQ * 16 + 8;
  constexpr int NG = 32 * MT * NQ * (2 / NT) / (NQ * 16);
  const size_t smem =
      FX ? 2 * (size_t)S * MT * 16 * 24 * sizeof(uint16_t) + (size_t)S * g.oz_KP * XROW * sizeof(uint16_t) +
               (size_t)(NQ * 16) * (1 + NG) * sizeof(int)
         : 2 * ((size_t)S * MT * 16 * 24 + (size_t)S * 16 * XROW) * sizeof(uint16_t);
  if (smem > 227 * 1024) return cudaErrorInvalidValue;
  static std::atomic<bool> opted[64];  // opted in to the largest shared memory, per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (!(dev >= 0 && dev < 64 && opted[dev].load())) {
    const cudaError_t e = cudaFuncSetAttribute(oz_mma_kernel<MT, NQ, NT, MINB, W, FX>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) opted[dev].store(true);
  }
  dim3 grid((g.N + NQ * 16 - 1) / (NQ * 16), (g.rows + MT * 16 - 1) / (MT * 16), g.batch);
  oz_mma_kernel<MT, NQ, NT, MINB, W, FX><<<grid, 32 * MT * NQ * (2 / NT), smem, s>>>(g);
  return cudaGetLastError();
}

template <int MT, int NQ, int NT = 2, int MINB = 1, bool FX = false>
static cudaError_t launch_oz_mt(const GemmArgs& g, cudaStream_t s) {
  return g.oz_w == 7 ? launch_oz_w<MT, NQ, NT, MINB, 7, FX>(g, s) : launch_oz_w<MT, NQ, NT, MINB, 6, FX>(g, s);
}

cudaError_t launch_oz_gemm(const GemmArgs& g, cudaStream_t s) {
  if (g.rows <= 0 || g.N <= 0 || g.batch <= 0) return cudaSuccess;
  const bool fx = oz_fused_x(g.rows, g.N, g.batch);
  if (g.K > 257 || g.oz_KP < g.K || (!fx && (!g.oz_xs || (g.oz_Np % 32) != 0)) || (g.oz_w != 6 && g.oz_w != 7) ||
      (g.oz_w == 7 && g.oz_KP > 112))
    return cudaErrorInvalidValue;
  // Row tiles per block: all of them up to 8 (one column group of 16, so
  // the operator panel is staged once for every row of the block), else the
  // fewest balanced blocks of at most 4 tiles with two column groups.
  const int rt = (g.rows + 15) / 16;
  if (rt >= 5 && rt <= 8) {
    switch (rt) {
      case 5: return fx ? launch_oz_mt<5, 1, 1, 2, true>(g, s) : launch_oz_mt<5, 1, 1, 2, false>(g, s);
      case 6: return fx ? launch_oz_mt<6, 1, 1, 1, true>(g, s) : launch_oz_mt<6, 1, 1, 1, false>(g, s);
      case 7: return fx ? launch_oz_mt<7, 1, 1, 1, true>(g, s) : launch_oz_mt<7, 1, 1, 1, false>(g, s);
      default: return fx ? launch_oz_mt<8, 1, 1, 1, true>(g, s) : launch_oz_mt<8, 1, 1, 1, false>(g, s);
    }
  }
  const int groups = (rt + 3) / 4, mt = (rt + groups - 1) / groups;
  const bool wide = g.N > 16;
  switch (mt) {
    case 1: return wide ? launch_oz_mt<1, 2>(g, s) : launch_oz_mt<1, 1>(g, s);
    case 2: return wide ? launch_oz_mt<2, 2>(g, s) : launch_oz_mt<2, 1>(g, s);
    case 3: return wide ? launch_oz_mt<3, 2>(g, s) : launch_oz_mt<3, 1>(g, s);
    default: return wide ? launch_oz_mt<4, 2>(g, s) : launch_oz_mt<4, 1>(g, s);
  }
}

}  // namespace falcon
