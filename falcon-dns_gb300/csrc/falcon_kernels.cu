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
// The nonlinear pass and its tables live in falcon_fft.cuh, compiled once
// per largest radix class (7, 17, 31) in its own translation unit.
// ---------------------------------------------------------------------------
cudaError_t init_dft_tables_7();
cudaError_t init_dft_tables_17();
cudaError_t init_dft_tables_31();
cudaError_t launch_nonlin_7(const NonlinArgs& a, cudaStream_t s);
cudaError_t launch_nonlin_17(const NonlinArgs& a, cudaStream_t s);
cudaError_t launch_nonlin_31(const NonlinArgs& a, cudaStream_t s);

cudaError_t init_dft_tables() {
  cudaError_t e = init_dft_tables_7();
  if (e == cudaSuccess) e = init_dft_tables_17();
  if (e == cudaSuccess) e = init_dft_tables_31();
  return e;
}

cudaError_t launch_nonlin(const NonlinArgs& a, cudaStream_t s) {
  int maxp = 0;
  for (int i = 0; i < a.plan.nrad; ++i) maxp = a.plan.rad[i] > maxp ? a.plan.rad[i] : maxp;
  if (maxp <= 7) return launch_nonlin_7(a, s);
  if (maxp <= 17) return launch_nonlin_17(a, s);
  return launch_nonlin_31(a, s);
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
