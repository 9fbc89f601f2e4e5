// Device construction of the implicit operators (mat_build*, dgetrf, dgetrs
// and chebinvtran of src/mat_assembly.F90, src/algebra_lapack.F90,
// src/chebyshev_fftw.F90), one operator set per (Nr, Nm, mBC, scheme, dt, Pr).
//
// Each mode's matrix is assembled on the device, factorised by one block in
// LAPACK's unblocked dgetf2 order (first maximal pivot, reciprocal scaling,
// rank-1 updates without contraction) and solved against unit right-hand
// sides in dgetrs order, so the inverse columns are the ones the reference's
// own dgetrs returns.  The coupled psi-omega operator AF is factorised whole
// (2R x 2R, in the reference's boundary-row order), not through a block
// elimination: the Chebyshev Laplacian is conditioned like R^4 and another
// elimination order would round differently from the reference.
#include <math.h>

#include "falcon_internal.h"

namespace falcon {

// Entries (i, j) of the R x R mode-m matrices, column-major, from t, D, D2
// (column-major R x R), written for modes m0 .. m0+nmodes-1.
//   kind 0: AT     = C [t - w dt/Pr L_m] with T boundary rows (mat_build)
//   kind 4: LAPpsi = C [L_m] with psi = 0 rows               (mat_build_rk)
// End columns are halved; L_m = r^-1 D + D2 - m^2 r^-2 t.
__global__ void assemble_kernel(int kind, int R, int m0, int nmodes, const double* t, const double* D,
                                const double* D2, const double* inv_r, const double* inv_r2, double wdt,
                                double inv_pr, double C, double* out) {
  const size_t per = (size_t)R * R;
  const size_t total = per * nmodes;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int mi = (int)(e / per);
    const size_t ij = e - (size_t)mi * per;
    const int j = (int)(ij / R), i = (int)(ij - (size_t)j * R);
    const double n = (double)(m0 + mi);
    const double nn = n * n;
    const size_t q = i + (size_t)R * j;
    const double L = __dadd_rn(__dadd_rn(__dmul_rn(inv_r[i], D[q]), D2[q]), -__dmul_rn(__dmul_rn(nn, inv_r2[i]), t[q]));
    const bool bc = (i == 0 || i == R - 1);
    double v;
    if (kind == 0) v = bc ? t[q] : __dadd_rn(t[q], -__dmul_rn(__dmul_rn(wdt, inv_pr), L));
    else v = bc ? t[q] : L;
    if (j == 0 || j == R - 1) v = __dmul_rn(0.5, v);
    out[e] = __dmul_rn(C, v);
  }
}

// AF (2R x 2R, column-major) of src/mat_assembly.F90:303-345 for modes
// m0 .. m0+nmodes-1:  [[L_m, t], [0, t - w dt L_m]] with the psi = 0 rows
// and the psi-derivative rows (dpsi/dr = 0 for no-slip, d2psi/dr2 - r^-1
// dpsi/dr = 0 for stress-free) at the ends of one block each; the IMEXRK
// build (mat_build_irk) puts the derivative rows in the upper block, the
// multistep build in the lower one.  End columns of both blocks are halved.
__global__ void assemble_af_kernel(int R, int m0, int nmodes, int mbc, int irk, const double* t, const double* D,
                                   const double* D2, const double* inv_r, const double* inv_r2, double wdt,
                                   double C, double* out) {
  const int R2 = 2 * R;
  const size_t per = (size_t)R2 * R2;
  const size_t total = per * nmodes;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int mi = (int)(e / per);
    const size_t ij = e - (size_t)mi * per;
    const int gj = (int)(ij / R2), gi = (int)(ij - (size_t)gj * R2);
    const int bi = gi >= R, bj = gj >= R;
    const int i = gi - bi * R, j = gj - bj * R;
    const double n = (double)(m0 + mi);
    const double nn = n * n;
    const size_t q = i + (size_t)R * j;
    const double L = __dadd_rn(__dadd_rn(__dmul_rn(inv_r[i], D[q]), D2[q]), -__dmul_rn(__dmul_rn(nn, inv_r2[i]), t[q]));
    const bool bc = (i == 0 || i == R - 1);
    double v;
    if (!bc) {
      if (!bi) v = bj ? t[q] : L;
      else v = bj ? __dadd_rn(t[q], -__dmul_rn(wdt, L)) : 0.0;
    } else if (bj) {
      v = 0.0;
    } else {
      const bool deriv = irk ? (bi == 0) : (bi == 1);
      v = deriv ? (mbc == 0 ? D[q] : __dadd_rn(D2[q], -__dmul_rn(inv_r[i], D[q]))) : t[q];
    }
    if (j == 0 || j == R - 1) v = __dmul_rn(0.5, v);
    out[e] = __dmul_rn(C, v);
  }
}

constexpr int kMaxLu = 520;  // largest order factorised (2 Nr_max for Nr_max <= 257)

// dgetrs 'N' on nrhs right-hand sides stored row-major (n x nrhs) in place,
// with the LU factors `a` (column-major n x n) and 0-based pivots `piv`: row
// interchanges, unit-lower forward, upper backward; the right-hand sides are
// independent columns, one thread each (threads tid of nt).
__device__ void dgetrs_rows(int n, const double* a, const int* piv, double* X, int nrhs, int tid, int nt) {
  for (int c = tid; c < nrhs; c += nt) {
    for (int i = 0; i < n; ++i) {
      const int p = piv[i];
      if (p != i) {
        const double tmp = X[(size_t)i * nrhs + c];
        X[(size_t)i * nrhs + c] = X[(size_t)p * nrhs + c];
        X[(size_t)p * nrhs + c] = tmp;
      }
    }
    for (int j = 0; j < n; ++j) {
      const double bj = X[(size_t)j * nrhs + c];
      if (bj != 0.0)
        for (int i = j + 1; i < n; ++i)
          X[(size_t)i * nrhs + c] = __dadd_rn(X[(size_t)i * nrhs + c], -__dmul_rn(bj, a[i + (size_t)n * j]));
    }
    for (int j = n - 1; j >= 0; --j) {
      double bj = X[(size_t)j * nrhs + c];
      if (bj != 0.0) {
        bj = bj / a[j + (size_t)n * j];
        X[(size_t)j * nrhs + c] = bj;
        for (int i = 0; i < j; ++i)
          X[(size_t)i * nrhs + c] = __dadd_rn(X[(size_t)i * nrhs + c], -__dmul_rn(bj, a[i + (size_t)n * j]));
      }
    }
  }
}

// One block per matrix: dgetf2 on the n x n column-major matrix (in shared
// memory when SMEM, else in place in global memory, where it stays L1/L2
// resident), then dgetrs 'N' on nrhs right-hand sides stored row-major
// (n x nrhs) in place.  info[b] = 0, or j+1 at the first zero pivot (INFO).
template <bool SMEM>
__global__ void __launch_bounds__(512) lu_solve_kernel(int n, double* mats, size_t mstride, double* rhs,
                                                       size_t rstride, int nrhs, int* info) {
  extern __shared__ double sm_a[];
  __shared__ double red_v[16];
  __shared__ int red_i[16];
  __shared__ int s_piv;
  __shared__ double s_pv;
  __shared__ int s_piv_all[kMaxLu];
  const int b = blockIdx.x;
  double* A = mats + (size_t)b * mstride;
  double* X = rhs + (size_t)b * rstride;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  double* a = SMEM ? sm_a : A;
  if (SMEM) {
    for (int e = tid; e < n * n; e += nt) a[e] = A[e];
    __syncthreads();
  }
  int first_zero = 0;
  for (int j = 0; j < n; ++j) {
    // pivot: first index of the largest |a(i, j)|, i >= j (idamax)
    double best = -1.0;
    int bi = n;
    for (int i = j + tid; i < n; i += nt) {
      const double v = fabs(a[i + (size_t)n * j]);
      if (v > best || (v == best && i < bi)) { best = v; bi = i; }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, best, off);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) { red_v[warp] = best; red_i[warp] = bi; }
    __syncthreads();
    if (tid == 0) {
      double bv = red_v[0];
      int bb = red_i[0];
      for (int w = 1; w < nw; ++w)
        if (red_v[w] > bv || (red_v[w] == bv && red_i[w] < bb)) { bv = red_v[w]; bb = red_i[w]; }
      if (bb >= n) bb = j;  // column without a comparable entry (NaN): keep the diagonal
      s_piv = bb;
      s_piv_all[j] = bb;
      s_pv = a[bb + (size_t)n * j];
    }
    __syncthreads();
    // the pivot value is read once by thread 0 before any row swap, so every
    // thread takes the same branch below (the barrier inside stays uniform)
    const int p = s_piv;
    const double pv = s_pv;
    if (pv != 0.0) {
      if (p != j)
        for (int k = tid; k < n; k += nt) {
          const double tmp = a[j + (size_t)n * k];
          a[j + (size_t)n * k] = a[p + (size_t)n * k];
          a[p + (size_t)n * k] = tmp;
        }
      __syncthreads();
      if (fabs(pv) >= 2.2250738585072014e-308) {
        const double rp = 1.0 / pv;
        for (int i = j + 1 + tid; i < n; i += nt) a[i + (size_t)n * j] = __dmul_rn(a[i + (size_t)n * j], rp);
      } else {
        for (int i = j + 1 + tid; i < n; i += nt) a[i + (size_t)n * j] = a[i + (size_t)n * j] / pv;
      }
    } else if (first_zero == 0) {
      first_zero = j + 1;
    }
    __syncthreads();
    for (int k = j + 1 + warp; k < n; k += nw) {
      const double akj = a[j + (size_t)n * k];
      if (akj != 0.0)
        for (int i = j + 1 + lane; i < n; i += 32)
          a[i + (size_t)n * k] = __dadd_rn(a[i + (size_t)n * k], -__dmul_rn(a[i + (size_t)n * j], akj));
    }
    __syncthreads();
  }
  if (tid == 0 && info) info[b] = first_zero;
  dgetrs_rows(n, a, s_piv_all, X, nrhs, tid, nt);
}

// Unit right-hand sides, row-major (n x nrhs) per batch entry: column c has
// its one at row off + c (off = 0: the identity; off = R with n = 2R: the
// vorticity block [0; I] of AF).
__global__ void unit_rhs_kernel(int n, int nrhs, int off, int nb, double* out) {
  const size_t per = (size_t)n * nrhs, total = per * nb;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t ij = e % per;
    out[e] = ((ij / nrhs) == (ij % nrhs) + (size_t)off) ? 1.0 : 0.0;
  }
}

static int ew_blocks(size_t n) {
  size_t g = (n + 255) / 256;
  if (g > 152 * 64) g = 152 * 64;
  return (int)(g ? g : 1);
}

cudaError_t launch_assemble(int kind, int R, int m0, int nmodes, const double* t, const double* D, const double* D2,
                            const double* inv_r, const double* inv_r2, double wdt, double inv_pr, double C,
                            double* out, cudaStream_t s) {
  if (kind != 0 && kind != 4) return cudaErrorInvalidValue;
  assemble_kernel<<<ew_blocks((size_t)R * R * nmodes), 256, 0, s>>>(kind, R, m0, nmodes, t, D, D2, inv_r, inv_r2, wdt,
                                                                    inv_pr, C, out);
  return cudaGetLastError();
}

cudaError_t launch_assemble_af(int R, int m0, int nmodes, int mbc, int irk, const double* t, const double* D,
                               const double* D2, const double* inv_r, const double* inv_r2, double wdt, double C,
                               double* out, cudaStream_t s) {
  assemble_af_kernel<<<ew_blocks((size_t)4 * R * R * nmodes), 256, 0, s>>>(R, m0, nmodes, mbc, irk, t, D, D2, inv_r,
                                                                           inv_r2, wdt, C, out);
  return cudaGetLastError();
}

// Shared-memory form up to 160 x 160 (200 KB); larger orders factorise in
// place in global memory (the matrices are overwritten).
// The solve phase of lu_solve_kernel for factors made elsewhere (a host's
// own dgetrf): one block per matrix, factors (column-major n x n, stride
// mstride; in shared memory when SMEM) and 1-based pivots (stride pstride)
// as LAPACK returns them, right-hand sides row-major (n x nrhs) in place.
// The pivots were checked to lie in [1, n] on the host.
template <bool SMEM>
__global__ void __launch_bounds__(512) getrs_rows_kernel(int n, const double* lus, size_t mstride, const int* ipivs,
                                                         size_t pstride, double* rhs, size_t rstride, int nrhs) {
  extern __shared__ double sm_f[];
  __shared__ int s_piv[kMaxLu];
  const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const double* A = lus + (size_t)b * mstride;
  for (int i = tid; i < n; i += nt) s_piv[i] = ipivs[(size_t)b * pstride + i] - 1;
  if (SMEM)
    for (int e = tid; e < n * n; e += nt) sm_f[e] = A[e];
  __syncthreads();
  dgetrs_rows(n, SMEM ? sm_f : A, s_piv, rhs + (size_t)b * rstride, nrhs, tid, nt);
}

cudaError_t launch_getrs_rows(int n, int nb, const double* lu, size_t mstride, const int* ipiv, size_t pstride,
                              double* rhs, size_t rstride, int nrhs, cudaStream_t s) {
  if (n > kMaxLu) return cudaErrorInvalidValue;
  const size_t smem = sizeof(double) * (size_t)n * n;
  if (smem <= 160 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(getrs_rows_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    getrs_rows_kernel<true><<<nb, 512, smem, s>>>(n, lu, mstride, ipiv, pstride, rhs, rstride, nrhs);
  } else {
    getrs_rows_kernel<false><<<nb, 512, 0, s>>>(n, lu, mstride, ipiv, pstride, rhs, rstride, nrhs);
  }
  return cudaGetLastError();
}

cudaError_t launch_lu_solve(int n, int nb, double* mats, size_t mstride, double* rhs, size_t rstride, int nrhs,
                            int* info, cudaStream_t s) {
  if (n < 1 || n > kMaxLu) return cudaErrorInvalidValue;
  if (nb <= 0) return cudaSuccess;
  const size_t smem = (size_t)n * n * sizeof(double);
  if (n <= 160) {
    cudaError_t e = cudaFuncSetAttribute(lu_solve_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    lu_solve_kernel<true><<<nb, 512, smem, s>>>(n, mats, mstride, rhs, rstride, nrhs, info);
  } else {
    lu_solve_kernel<false><<<nb, 512, 0, s>>>(n, mats, mstride, rhs, rstride, nrhs, info);
  }
  return cudaGetLastError();
}

cudaError_t launch_unit_rhs(int n, int nrhs, int off, int nb, double* out, cudaStream_t s) {
  unit_rhs_kernel<<<ew_blocks((size_t)n * nrhs * nb), 256, 0, s>>>(n, nrhs, off, nb, out);
  return cudaGetLastError();
}

}  // namespace falcon
