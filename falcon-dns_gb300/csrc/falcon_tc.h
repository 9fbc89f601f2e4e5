// Interface of the tcgen05 operator contraction (falcon_tc.cu) and the
// encodings of its shared-memory matrix and instruction descriptors and of
// its operand layouts, shared by the kernel, its host launcher and the
// host-side checks.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace falcon {

constexpr int kTcBM = 128;  // operator rows per tile (the MMA's M)
constexpr int kTcBN = 24;   // X columns per tile (one slice's share of the MMA's N)
constexpr int kTcAccStride = 256;  // tensor-memory columns between the two accumulator buffers
constexpr int kTcEpilogue = 256;   // epilogue threads (warps 0-7)
constexpr int kTcProducers = 128;  // X producer threads (warps 8-11)
constexpr int kTcWarpTma = 12;     // tensor-memory allocation and operator copies
constexpr int kTcThreads = 448;    // + the MMA warp (13)

// Slices per operand (S) of the 7-bit and 6-bit formats (OzCfg); the
// diagonals d = s + t run 0..S-1.
__host__ __device__ constexpr int tc_slices(int w) { return w == 7 ? 9 : 10; }
// N of the MMA of operator slice s: the X slices 0..S-1-s side by side
// (24 columns each), rounded up to a multiple of 16 (the extra columns'
// products land in a spill strip of the accumulator buffer).
__host__ __device__ constexpr int tc_mma_n(int S, int s) { return ((S - s) * kTcBN + 15) / 16 * 16; }
// Columns of an X stage: every slice's 24 columns, rounded up to a
// multiple of 16 (zero padding read only by the rounded MMAs).
__host__ __device__ constexpr int tc_x_cols(int S) { return (S * kTcBN + 15) / 16 * 16; }

// Shared-memory layouts (no swizzle, K-major, core matrix = 8 rows x 16 B
// stored as 128 contiguous bytes): the operator stage holds per slice two
// k groups of 128 rows (stride-dimension offset 128 B between 8-row
// groups, leading-dimension offset 2048 B between the k groups); the X
// stage holds two k groups of all slices' columns side by side, slice t's
// column n at stage column 24 t + n (128 B between 8-column groups,
// tc_x_cols(S) x 16 B between the k groups).
constexpr uint32_t kTcSbo = 128;
constexpr uint32_t kTcALbo = kTcBM * 16;
__host__ __device__ constexpr uint32_t tc_x_lbo(int S) { return (uint32_t)tc_x_cols(S) * 16; }

// Shared-memory matrix descriptor of tcgen05.mma: start address, leading
// and stride byte offsets (each >> 4, 14 bits), descriptor version 1 (bits
// 46-47), base offset 0, no swizzle (bits 61-63 = 0).
__host__ __device__ constexpr uint64_t tc_smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of tcgen05.mma.kind::f16: D format FP32 (bits
// 4-5 = 1), A and B bf16 (bits 7-9 = 1, 10-12 = 1), no negation, both
// K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Y_o[z][row - rstart_o][n] = alpha sum_k A_z[row0 + row][k] X_z[k][n] for
// the rows of output o (rows [rend[o-1], rend[o]), up to 4 outputs).
struct TcArgs {
  const double* X;
  long ldx, sX;        // X[z sX + k ldx + n]
  int K, KP, N, batch, rows, w;
  int nout;
  int rend[4];
  double* Y[4];
  long ldy, sY;        // Y_o[z sY + r ldy + n]
  double alpha;
  const int* aex;      // row exponents of batch entry 0, row 0 of this contraction; stride rowsP per entry
  int rowsP;
  int row0, z0;        // tensor-map coordinates of this contraction's first row and entry
  int* err;            // error word (set by the launcher)
};

// Tensor map of an operator's slices [nb][S][KP/8][rowsP][8] (bf16 bits)
// for the copies of the kernel (box: 8 k x 128 rows x 2 k groups x S
// slices x 1 entry).  Host.
int tc_make_operator_map(CUtensorMap* map, const uint16_t* slices, int nb, int S, int KP, int rowsP);
// Every descriptor of the kernel's stage layout stays inside its stage and
// every accumulator inside the allocated tensor memory (0, or < 0).  Host.
int tc_stage_layout_check(int w, int KP);
cudaError_t launch_tc_gemm(const TcArgs& a, const CUtensorMap& map, cudaStream_t s);
// The kernels' error word (a wait that timed out: 1-8), read and cleared.
int tc_error_read_and_clear();

}  // namespace falcon
