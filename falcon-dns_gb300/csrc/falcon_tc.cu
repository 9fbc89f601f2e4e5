// FP64 operator contractions Y = alpha A X on the 5th-generation tensor
// cores (tcgen05, accumulators in tensor memory) by exact integer slicing,
// with the same slice formats and recombination as oz_mma_kernel
// (falcon_ozaki.cu, OzCfg in falcon_slices.cuh): every FP32 sum of slice
// products is exact, so both kernels give the same bits.
//
// Tile: 128 operator rows (the MMA's M) x 24 X columns.  Per slice diagonal
// d = s + t one FP32 accumulator of 128 x 24 in tensor memory, the S
// diagonals side by side (diagonal d at column 24 d of its buffer), and two
// such buffers (columns 0 and 256), so the epilogue of one tile runs while
// the next tile multiplies.  Per 16-wide K chunk and operator slice s the
// MMA warp issues ONE tcgen05.mma.kind::f16 (bf16 in, FP32 accumulate): A_s
// against the X slices 0..S-1-s laid side by side along N, whose products
// land exactly on the diagonals s..S-1 (N rounded up to a multiple of 16;
// the extra columns' products fall in a spill strip after the last
// diagonal).  The operator slice is read from shared memory once per chunk.
//
// Operands in shared memory, no swizzle, K-major core matrices (8 rows x
// 16 bytes):
//  - A, the operator slices made once per operator set (layout
//    [nb][S][KP/8][rowsP][8], launch_oz_slice_rows): one TMA tensor copy per
//    K chunk brings all S slices of a 128-row tile.  When the whole K fits
//    in the stage ring (KP <= 80 for 7-bit slices) a tile's operator stays
//    resident while the CTA walks its column tiles;
//  - X: four producer warps read the FP64 columns (kept in registers), take
//    each column's exponent over all of K and cut the values into slices
//    directly in shared memory (no slice planes in HBM), two slices per
//    packed bf16 subtraction.
// Warp roles (448 threads, one CTA per SM, persistent over a contiguous
// range of (entry, row tile, column tile) work items):
//   0-7   epilogue: tcgen05.ld of the diagonals (warp w reads tensor-memory
//         lanes 32 (w%4).. = operator rows, half w/4 of the columns), exact
//         recombination, FP64 stores;
//   8-11  X producers;
//   12    tensor-memory allocation and the operator's TMA copies (lane 0);
//   13    MMA issue (lane 0).
// Every wait on an mbarrier is bounded: after ~1 s a wait sets an error
// word in global memory and the CTA's abort flag, and every role leaves
// its loop; the MMA warp waits (bounded) for its own products and the TMA
// warp for its own copies before the tensor memory is freed.  Waiting
// threads sleep in hardware (try_wait with a suspend-time hint).
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>

#include "falcon_internal.h"
#include "falcon_slices.cuh"
#include "falcon_tc.h"

namespace falcon {
namespace {

constexpr long long kSpinCycles = 2000000000LL;  // ~1 s at 2 GHz

template <int W>
struct TcCfg {
  static constexpr int S = OzCfg<W>::S, D = OzCfg<W>::D, HD = OzCfg<W>::HD, MAGB = OzCfg<W>::MAGB;
  static constexpr int BM = kTcBM, BN = kTcBN, BK = 16;
  static constexpr int NA = (W == 7) ? 5 : 3;  // operator stages (16 k each)
  static constexpr int NX = 4;                 // X stages
  static constexpr int A_SLICE = BM * BK * 2;  // 4096 bytes: 2 k groups x 128 rows x 16 B
  static constexpr int A_STAGE = S * A_SLICE;
  // X stage: [k group (2)][column group (XCOLS / 8)][8 columns][16 B]
  static constexpr int XCOLS = tc_x_cols(S);
  static constexpr int XGROUPS = XCOLS / 8;
  static constexpr uint32_t XLBO = tc_x_lbo(S);  // between the two k groups
  static constexpr int X_STAGE = 2 * XGROUPS * 128;
  static constexpr int OFF_A = 0;
  static constexpr int OFF_X = NA * A_STAGE;
  static constexpr int OFF_CEX = OFF_X + NX * X_STAGE;  // int [4][BN] column exponents
  static constexpr int OFF_PM = OFF_CEX + 4 * BN * 4;   // int [4][BN] partial maxima
  static constexpr int NBAR = 2 * NA + 2 * NX + 4 + 8 + 1;
  static constexpr int OFF_BAR = OFF_PM + 4 * BN * 4;
  static constexpr int OFF_MISC = OFF_BAR + NBAR * 8;   // tensor-memory address, abort flag, producer flags
  static constexpr int BYTES = OFF_MISC + 16;
  static constexpr int SMEM = BYTES + 1024;             // + alignment of the base to 1 KiB
  static constexpr uint32_t TMEM_COLS = 512;
  static_assert(S * BN + 8 <= kTcAccStride && 2 * kTcAccStride <= (int)TMEM_COLS, "accumulator buffers");
  static_assert(tc_mma_n(S, 0) <= 256, "MMA N");
  static_assert(SMEM <= 227 * 1024, "shared memory");
};

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(su32(b)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(su32(b)),
               "r"(bytes)
               : "memory");
}
// try_wait with a suspend-time hint: the thread sleeps in hardware until the
// phase completes or ~20 us pass, so waiting warps take no issue slots from
// the producer and epilogue warps on their sub-partition.
__device__ __forceinline__ bool mbar_try_sleep(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity), "r"(20000u)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of parity `parity`; false when the CTA aborts
// (this wait timed out, or another role's did).
__device__ __noinline__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag, int* err, int code) {
  const long long t0 = clock64();
  while (!mbar_try_sleep(b, parity)) {
    if (*abort_flag) return false;
    if (clock64() - t0 > kSpinCycles) {
      *abort_flag = 1;
      atomicCAS(err, 0, code);
      return false;
    }
  }
  return true;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void named_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }

__device__ __forceinline__ void tma_load_5d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                            int c3, int c4) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6, "
      "%7}], [%2];" ::"r"(su32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(su32(bar)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4)
      : "memory");
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void tc_commit(uint64_t* b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(b)) : "memory");
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, uint32_t (&r)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// The work item of linear tile index t: entry z, row tile mt, column tile nt.
struct TileIdx {
  int z, mt, nt;
};
__device__ __forceinline__ TileIdx tile_of(long t, int n_mt, int n_nt) {
  TileIdx r;
  r.nt = (int)(t % n_nt);
  const long zm = t / n_nt;
  r.mt = (int)(zm % n_mt);
  r.z = (int)(zm / n_mt);
  return r;
}

template <int W>
__global__ void __launch_bounds__(448, 1) tc_gemm_kernel(const __grid_constant__ CUtensorMap amap, const TcArgs q) {
  using C = TcCfg<W>;
  extern __shared__ uint8_t tc_smem_raw[];
  uint8_t* sm = tc_smem_raw + ((1024 - (su32(tc_smem_raw) & 1023)) & 1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + C::OFF_BAR);
  uint64_t* full_a = bars;
  uint64_t* empty_a = full_a + C::NA;
  uint64_t* full_x = empty_a + C::NA;
  uint64_t* empty_x = full_x + C::NX;
  uint64_t* acc_full = empty_x + C::NX;  // [2]
  uint64_t* acc_empty = acc_full + 2;    // [2]
  uint64_t* cex_full = acc_empty + 2;    // [4]
  uint64_t* cex_empty = cex_full + 4;    // [4]
  uint64_t* drain = cex_empty + 4;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + C::OFF_MISC);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(sm + C::OFF_MISC + 4);
  int* cex_ring = reinterpret_cast<int*>(sm + C::OFF_CEX);
  int* pm = reinterpret_cast<int*>(sm + C::OFF_PM);

  if (tid == 0) {
    for (int i = 0; i < C::NA; ++i) { mbar_init(&full_a[i], 1); mbar_init(&empty_a[i], 1); }
    for (int i = 0; i < C::NX; ++i) { mbar_init(&full_x[i], kTcProducers); mbar_init(&empty_x[i], 1); }
    for (int i = 0; i < 2; ++i) { mbar_init(&acc_full[i], 1); mbar_init(&acc_empty[i], kTcEpilogue); }
    for (int i = 0; i < 4; ++i) { mbar_init(&cex_full[i], kTcProducers); mbar_init(&cex_empty[i], kTcEpilogue); }
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // the X stages' padding columns (read only by the rounded-up MMAs, whose
  // products there land in the spill strip) hold zeros
  if constexpr (C::XCOLS > C::S * C::BN)
    for (int i = tid; i < C::NX * 2 * (C::XCOLS - C::S * C::BN) * 4; i += blockDim.x) {
      const int words = (C::XCOLS - C::S * C::BN) * 4;  // 32-bit words of the padding per k group
      const int st = i / (2 * words), kg = (i / words) % 2, w = i % words;
      reinterpret_cast<uint32_t*>(sm + C::OFF_X + st * C::X_STAGE + kg * C::XGROUPS * 128 +
                                  C::S * C::BN * 16)[w] = 0u;
    }
  if (warp == kTcWarpTma) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)),
                 "r"(C::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  const int n_nt = (q.N + C::BN - 1) / C::BN, n_mt = (q.rows + C::BM - 1) / C::BM;
  const long T = (long)q.batch * n_mt * n_nt;
  const long t_begin = T * blockIdx.x / gridDim.x, t_end = T * (blockIdx.x + 1) / gridDim.x;
  const int nk = q.KP / C::BK;
  const bool resident = nk <= C::NA;
  const uint32_t sm_base = su32(sm);

  if (warp < kTcEpilogue / 32) {
    // ---------------- epilogue ----------------
    // warp (q, h): tensor-memory lanes 32q..32q+31 (operator rows), columns
    // 12h..12h+11 of the tile; waits are taken by lane 0 and broadcast, so a
    // warp leaves together (tcgen05.ld is warp-collective)
    const int qd = warp & 3, half = warp >> 2;
    const bool scale_y = q.alpha != 1.0;  // one FP64 compare, not one per output
    long u = 0;
    for (long t = t_begin; t < t_end; ++t, ++u) {
      const TileIdx ti = tile_of(t, n_mt, n_nt);
      const int buf = (int)(u & 1);
      int ok = 1;
      if (lane == 0)
        ok = mbar_wait(&acc_full[buf], (uint32_t)((u >> 1) & 1), abort_flag, q.err, 1) &&
             mbar_wait(&cex_full[u & 3], (uint32_t)((u >> 2) & 1), abort_flag, q.err, 2);
      ok = __shfl_sync(0xffffffffu, ok, 0);
      __syncwarp();
      if (!ok) break;
      tc_fence_after();
      const int* cex = cex_ring + (u & 3) * C::BN;
      const int r = ti.mt * C::BM + qd * 32 + lane;
      const bool valid = r < q.rows;
      int er = 0;
      double* yrow = nullptr;
      if (valid) {
        int o = 0;
        while (o + 1 < q.nout && r >= q.rend[o]) ++o;
        const int r0 = o ? q.rend[o - 1] : 0;
        er = q.aex[(size_t)ti.z * q.rowsP + r];
        yrow = q.Y[o] + (size_t)ti.z * q.sY + (size_t)(r - r0) * q.ldy;
      }
      const int n0 = ti.nt * C::BN;
      const uint32_t lane_addr = tmem + ((uint32_t)(qd * 32) << 16) + (uint32_t)(buf * kTcAccStride);
#pragma unroll 1
      for (int c0 = half * (C::BN / 2); c0 < (half + 1) * (C::BN / 2); c0 += 4) {
        uint32_t v[C::D + 1][4];
#pragma unroll
        for (int d = 0; d <= C::D; ++d) tmem_ld4(lane_addr + (uint32_t)(d * C::BN + c0), v[d]);
        tmem_wait_ld();
#pragma unroll
        for (int d = 0; d <= C::D; ++d)
#pragma unroll
          for (int j = 0; j < 4; ++j) asm volatile("" : "+r"(v[d][j]));
        if (valid) {
          double out[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            auto qd = [&](int d) { return __float2int_rn(__uint_as_float(v[d][j])); };
            const long long H = oz_diag_sum<W, 0, C::HD>(qd), L = oz_diag_sum<W, C::HD + 1, C::D>(qd);
            const int fb = cex[c0 + j];
            const int kL = er + (fb - 1022) - 2 * C::MAGB + W * (2 * C::S - 2 - C::D);
            double y = fb > 0 ? oz_recombine_2t(H, L, kL, W * (C::D - C::HD)) : 0.0;
            if (fb == 2047) y = __longlong_as_double(0x7ff8000000000000LL);  // Inf or NaN in the column
            out[j] = scale_y ? q.alpha * y : y;
          }
          const int n = n0 + c0;
          double* yp = yrow + n;
          if (n + 4 <= q.N && (reinterpret_cast<uintptr_t>(yp) & 15) == 0) {
            *reinterpret_cast<double2*>(yp) = make_double2(out[0], out[1]);
            *reinterpret_cast<double2*>(yp + 2) = make_double2(out[2], out[3]);
          } else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
              if (n + j < q.N) yp[j] = out[j];
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&acc_empty[buf]);
      mbar_arrive(&cex_empty[u & 3]);
    }
  } else if (warp < (kTcEpilogue + kTcProducers) / 32) {
    // ---------------- X producers ----------------
    // Thread (column n, k group kg, half h) owns the values k = 16 c + 8 kg +
    // 4 h + i (i < 4) of its column: it reads them once per tile (the first
    // RC chunks stay in registers), takes the column exponent with its three
    // partners, then cuts them into slices chunk by chunk (8 bytes per
    // slice).  Waits are taken by thread 0 and passed on through prod_ok
    // (two slots by wait parity) at a named barrier, so the producers always
    // leave together and the named barriers stay matched.
    constexpr int RC = 9;  // K up to 144 (Nr = 129) held in registers
    const int tp = tid - kTcEpilogue;
    volatile int* prod_ok = reinterpret_cast<volatile int*>(sm + C::OFF_MISC + 8);
    const bool act = tp < 4 * C::BN;
    const int hq = tp / (2 * C::BN), rem = tp % (2 * C::BN), kg = rem / C::BN, n = rem % C::BN;
    const int part = kg * 2 + hq;  // partner index for the column maximum
    long xc = 0, u = 0, nw = 0;
    bool stop = false;
    for (long t = t_begin; t < t_end && !stop; ++t, ++u) {
      const TileIdx ti = tile_of(t, n_mt, n_nt);
      const int n0 = ti.nt * C::BN, nn = n0 + n;
      const double* Xz = q.X + (size_t)ti.z * q.sX;
      const bool col = act && nn < q.N;
      double v[RC][4];
      int mx = 0;
#pragma unroll
      for (int c = 0; c < RC; ++c)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int k = c * C::BK + kg * 8 + hq * 4 + i;
          v[c][i] = (col && c < nk && k < q.K) ? Xz[(size_t)k * q.ldx + nn] : 0.0;
        }
      for (int c = RC; c < nk; ++c)
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int k = c * C::BK + kg * 8 + hq * 4 + i;
          if (col && k < q.K) mx = max(mx, biased_exp(Xz[(size_t)k * q.ldx + nn]));
        }
#pragma unroll
      for (int c = 0; c < RC; ++c)
#pragma unroll
        for (int i = 0; i < 4; ++i) mx = max(mx, biased_exp(v[c][i]));
      if (tp == 0)
        prod_ok[nw & 1] = mbar_wait(&cex_empty[u & 3], (uint32_t)(((u >> 2) & 1) ^ 1), abort_flag, q.err, 3) ? 1 : 0;
      if (act) pm[part * C::BN + n] = mx;
      named_sync(1, kTcProducers);
      if (!prod_ok[(nw++) & 1]) break;
      int* cex = cex_ring + (u & 3) * C::BN;
      const int fb = act ? max(max(pm[n], pm[C::BN + n]), max(pm[2 * C::BN + n], pm[3 * C::BN + n])) : 0;
      if (tp < C::BN) cex[tp] = fb;
      mbar_arrive(&cex_full[u & 3]);
      auto produce = [&](const double (&vals)[4]) -> bool {
        const long j = xc++;
        const int st = (int)(j % C::NX);
        if (tp == 0)
          prod_ok[nw & 1] = mbar_wait(&empty_x[st], (uint32_t)(((j / C::NX) & 1) ^ 1), abort_flag, q.err, 4) ? 1 : 0;
        named_sync(1, kTcProducers);
        if (!prod_ok[(nw++) & 1]) return false;
        if (act) {
          uint32_t lo[4], hi[4], sg[2];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const unsigned long long Tm = fb > 0 ? oz_magb<C::MAGB>(vals[i], fb - 1022) : 0ull;
            lo[i] = (uint32_t)Tm;
            hi[i] = (uint32_t)(Tm >> 32);
          }
#pragma unroll
          for (int p = 0; p < 2; ++p)
            sg[p] = (__double_as_longlong(vals[2 * p]) < 0 ? 0x8000u : 0u) |
                    (__double_as_longlong(vals[2 * p + 1]) < 0 ? 0x80000000u : 0u);
          uint8_t* xs = sm + C::OFF_X + st * C::X_STAGE + (kg * C::XGROUPS + n / 8) * 128 + (n % 8) * 16 + hq * 8;
#pragma unroll
          for (int s = 0; s < C::S; ++s) {
            const uint32_t w0 = oz_slice_pair<W>(lo[0], hi[0], lo[1], hi[1], sg[0], s);
            const uint32_t w1 = oz_slice_pair<W>(lo[2], hi[2], lo[3], hi[3], sg[1], s);
            *reinterpret_cast<uint2*>(xs + s * (C::BN / 8) * 128) = make_uint2(w0, w1);
          }
        }
        fence_async_smem();
        mbar_arrive(&full_x[st]);
        return true;
      };
#pragma unroll
      for (int c = 0; c < RC; ++c)
        if (c < nk && !stop && !produce(v[c])) stop = true;
      for (int c = RC; c < nk && !stop; ++c) {
        double w4[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int k = c * C::BK + kg * 8 + hq * 4 + i;
          w4[i] = (col && k < q.K) ? Xz[(size_t)k * q.ldx + nn] : 0.0;
        }
        if (!produce(w4)) stop = true;
      }
    }
  } else if (warp == kTcWarpTma) {
    // ---------------- operator TMA copies ----------------
    if (lane == 0) {
      long ac = 0;
      long last = -1;  // item (z, mt) of the previous tile
      long issued = 0;
      for (long t = t_begin; t < t_end && !*abort_flag; ++t) {
        const TileIdx ti = tile_of(t, n_mt, n_nt);
        const long item = (long)ti.z * n_mt + ti.mt;
        if (resident && item == last) continue;
        last = item;
        for (int c = 0; c < nk; ++c) {
          const long j = ac++;
          const int st = (int)(j % C::NA);
          if (!mbar_wait(&empty_a[st], (uint32_t)(((j / C::NA) & 1) ^ 1), abort_flag, q.err, 5)) break;
          mbar_expect_tx(&full_a[st], (uint32_t)C::A_STAGE);
          tma_load_5d(sm + C::OFF_A + st * C::A_STAGE, &amap, &full_a[st], 0, q.row0 + ti.mt * C::BM, 2 * c, 0,
                      q.z0 + ti.z);
          issued = ac;
        }
      }
      // wait for the copies this thread issued (bounded), so none is in
      // flight when the CTA ends
      for (long j = (issued > C::NA ? issued - C::NA : 0); j < issued; ++j) {
        const long long t0 = clock64();
        while (!mbar_try_sleep(&full_a[j % C::NA], (uint32_t)((j / C::NA) & 1)) && clock64() - t0 < kSpinCycles) {
        }
      }
    }
  } else {
    // ---------------- MMA issue ----------------
    if (lane == 0) {
      long ac = 0, xc = 0, u = 0, abase = 0;
      long last = -1;
      bool any = false;
      for (long t = t_begin; t < t_end; ++t, ++u) {
        const TileIdx ti = tile_of(t, n_mt, n_nt);
        const long item = (long)ti.z * n_mt + ti.mt;
        const bool first_of_item = item != last;
        last = item;
        bool last_of_item = true;
        if (t + 1 < t_end) {
          const TileIdx tn = tile_of(t + 1, n_mt, n_nt);
          last_of_item = ((long)tn.z * n_mt + tn.mt) != item;
        }
        if (resident && first_of_item) {
          abase = ac;
          ac += nk;
        }
        const int buf = (int)(u & 1);
        if (u > 1 && !mbar_wait(&acc_empty[buf], (uint32_t)(((u - 2) >> 1) & 1), abort_flag, q.err, 6)) break;
        tc_fence_after();
        const uint32_t acc_base = tmem + (uint32_t)(buf * kTcAccStride);
        bool ok = true;
        for (int c = 0; c < nk && ok; ++c) {
          const long ja = resident ? abase + c : ac++;
          const int sa = (int)(ja % C::NA);
          if ((!resident || first_of_item) &&
              !mbar_wait(&full_a[sa], (uint32_t)((ja / C::NA) & 1), abort_flag, q.err, 7)) {
            ok = false;
            break;
          }
          const long jx = xc++;
          const int sx = (int)(jx % C::NX);
          if (!mbar_wait(&full_x[sx], (uint32_t)((jx / C::NX) & 1), abort_flag, q.err, 8)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a_stage = sm_base + C::OFF_A + sa * C::A_STAGE;
          const uint64_t bdesc = tc_smem_desc(sm_base + C::OFF_X + sx * C::X_STAGE, C::XLBO, kTcSbo);
          // operator slice s against the X slices 0..S-1-s side by side:
          // products on the diagonals s..S-1 (s = 0 writes every diagonal
          // fresh in the first chunk of a tile; the rest accumulate)
#pragma unroll 1
          for (int s = 0; s < C::S; ++s)
            tc_mma(acc_base + (uint32_t)(s * C::BN), tc_smem_desc(a_stage + s * C::A_SLICE, kTcALbo, kTcSbo), bdesc,
                   tc_idesc_bf16(C::BM, tc_mma_n(C::S, s)), (c > 0 || s > 0) ? 1u : 0u);
          any = true;
          tc_commit(&empty_x[sx]);
          if (!resident || last_of_item) tc_commit(&empty_a[sa]);
        }
        if (!ok) break;
        tc_commit(&acc_full[buf]);
      }
      // wait for every product this thread issued (bounded) before the
      // tensor memory is freed
      if (any) {
        tc_commit(drain);
        const long long t0 = clock64();
        while (!mbar_try_sleep(drain, 0) && clock64() - t0 < kSpinCycles) {
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kTcWarpTma) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::TMEM_COLS) : "memory");
  }
}

static __device__ int g_tc_err;
std::once_flag g_tc_err_once[64];
int* g_tc_err_addr[64];

int* tc_err_ptr(int dev) {
  std::call_once(g_tc_err_once[dev], [dev] {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_tc_err) == cudaSuccess) g_tc_err_addr[dev] = static_cast<int*>(p);
  });
  return g_tc_err_addr[dev];
}

template <int W>
cudaError_t launch_tc_w(const TcArgs& a, const CUtensorMap& map, cudaStream_t s) {
  using C = TcCfg<W>;
  static std::atomic<bool> opted[64];
  int dev = 0, nsm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!opted[dev].load()) {
    e = cudaFuncSetAttribute(tc_gemm_kernel<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    if (e != cudaSuccess) return e;
    opted[dev].store(true);
  }
  e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  TcArgs q = a;
  q.err = tc_err_ptr(dev);
  if (!q.err) return cudaErrorInvalidSymbol;
  const long T = (long)q.batch * ((q.rows + C::BM - 1) / C::BM) * ((q.N + C::BN - 1) / C::BN);
  const int grid = (int)(T < nsm ? T : nsm);
  tc_gemm_kernel<W><<<grid, kTcThreads, C::SMEM, s>>>(map, q);
  return cudaGetLastError();
}

}  // namespace

int tc_make_operator_map(CUtensorMap* map, const uint16_t* slices, int nb, int S, int KP, int rowsP) {
  using Encode = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static Encode encode = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult st;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &st) ==
            cudaSuccess &&
        st == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<Encode>(fn);
  });
  if (!encode || !slices || KP % 16 != 0 || rowsP < kTcBM || nb < 1 || (reinterpret_cast<uintptr_t>(slices) & 15))
    return -1;
  // [nb][S][KP/8][rowsP][8] bf16 bits: dims innermost first
  const cuuint64_t dims[5] = {8, (cuuint64_t)rowsP, (cuuint64_t)(KP / 8), (cuuint64_t)S, (cuuint64_t)nb};
  const cuuint64_t strides[4] = {16, (cuuint64_t)rowsP * 16, (cuuint64_t)rowsP * KP * 2,
                                 (cuuint64_t)S * rowsP * KP * 2};
  const cuuint32_t box[5] = {8, (cuuint32_t)kTcBM, 2, (cuuint32_t)S, 1};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 5, const_cast<uint16_t*>(slices), dims, strides, box,
                            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -2;
}

int tc_stage_layout_check(int w, int KP) {
  // every descriptor of the kernel stays inside its shared-memory stage and
  // every accumulator inside its tensor-memory buffer: decode start,
  // leading and stride offsets back from the encodings and bound the last
  // byte of the last core matrix an MMA reads
  auto last_byte = [](uint64_t d, int row_groups, int k_groups) -> long {
    const long start = (long)(d & 0x3FFF) << 4, lbo = (long)((d >> 16) & 0x3FFF) << 4,
               sbo = (long)((d >> 32) & 0x3FFF) << 4;
    return start + (row_groups - 1) * sbo + (k_groups - 1) * lbo + 127;
  };
  const int S = tc_slices(w), NA = w == 7 ? 5 : 3, NX = 4;
  const long a_slice = kTcBM * 16 * 2;
  const long a_stage = S * a_slice;
  const long x_stage = 2L * tc_x_cols(S) * 16;
  const long off_x = NA * a_stage;
  if (KP % 16 != 0 || KP > 272) return -1;
  if (S * kTcBN + 8 > kTcAccStride || 2 * kTcAccStride > 512) return -4;
  for (int st = 0; st < NA; ++st)
    for (int s = 0; s < S; ++s) {
      const uint64_t d = tc_smem_desc((uint32_t)(st * a_stage + s * a_slice), kTcALbo, kTcSbo);
      if (last_byte(d, kTcBM / 8, 2) >= (st * a_stage + (s + 1) * a_slice)) return -2;
    }
  for (int st = 0; st < NX; ++st)
    for (int s = 0; s < S; ++s) {
      const int n = tc_mma_n(S, s);
      if (n % 16 != 0 || n > 256 || n > tc_x_cols(S) || s * kTcBN + n > kTcAccStride) return -4;
      const uint64_t d = tc_smem_desc((uint32_t)(off_x + st * x_stage), tc_x_lbo(S), kTcSbo);
      if (last_byte(d, n / 8, 2) >= off_x + (st + 1) * x_stage) return -3;
    }
  return 0;
}

cudaError_t launch_tc_gemm(const TcArgs& a, const CUtensorMap& map, cudaStream_t s) {
  if (a.rows <= 0 || a.N <= 0 || a.batch <= 0) return cudaSuccess;
  if (a.K > 257 || a.KP < a.K || (a.KP % 16) != 0 || (a.w != 6 && a.w != 7) || (a.w == 7 && a.KP > 112) ||
      a.nout < 1 || a.nout > 4 || a.rend[a.nout - 1] != a.rows)
    return cudaErrorInvalidValue;
  return a.w == 7 ? launch_tc_w<7>(a, map, s) : launch_tc_w<6>(a, map, s);
}

int tc_error_read_and_clear() {
  int v = 0;
  if (cudaMemcpyFromSymbol(&v, g_tc_err, sizeof(int)) != cudaSuccess) return -1;
  if (v) {
    const int z = 0;
    cudaMemcpyToSymbol(g_tc_err, &z, sizeof(int));
  }
  return v;
}

}  // namespace falcon
