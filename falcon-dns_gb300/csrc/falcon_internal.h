// Internal interfaces between the host runtime (falcon_host.cpp) and the
// sm_103a kernels (falcon_kernels.cu, falcon_fft.cuh, ...).  Not part of the C ABI.
//
// Device layout of every complex field of a group of B instances that share
// (Nr, Nm): X[r][m][b] (instance fastest), one double2 per element, so that
//  - a radial operator (R x R) applied to all modes and instances is one
//    GEMM with K = R and N = 2*M*B contiguous columns, and
//  - a per-mode operator applied to all instances of a mode is a GEMM whose
//    2*B columns are contiguous.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace falcon {

constexpr int kMaxRadix = 16;     // stages of a mixed-radix FFT plan
constexpr int kMaxStages = 8;     // IMEXRK stages supported (KC885 has 8)

// Plan of the azimuthal transform of length P = 3*Nm.  Two forms:
//  - pfa = 1 (P square-free, prime factors <= 31): Good-Thomas prime-factor
//    mapping; the stages are twiddle-free DFTs along the axes of a
//    rad[0] x rad[1] x ... array (row-major, last axis contiguous) and the
//    spectrum sits at pos[k] = sum_d ((k cinv[d]) mod rad[d]) stride[d],
//    cinv[d] = (P/rad[d])^-1 mod rad[d];
//  - pfa = 0: mixed-radix Cooley-Tukey, in-place DIT/DIF with twiddles and
//    the spectrum at the digit-reversed positions pos[k].
struct FftPlan {
  int P;
  int nrad;
  int pfa;
  int rad[kMaxRadix];   // radices / axis sizes, outermost first
  int cinv[kMaxRadix];
};

// Builds the plan for length P (host).  Returns 0, or -1 when P has a prime
// factor above 64 or more than kMaxRadix factors.
inline int make_fft_plan(int P, FftPlan* plan) {
  FftPlan f{};
  f.P = P;
  int primes[64], np = 0, n = P;
  for (int q = 2; q * q <= n; ++q)
    while (n % q == 0) { if (np < 64) primes[np++] = q; n /= q; }
  if (n > 1 && np < 64) primes[np++] = n;
  bool squarefree = true, small = true;
  for (int i = 0; i < np; ++i) {
    if (i > 0 && primes[i] == primes[i - 1]) squarefree = false;
    if (primes[i] > 31) small = false;
    if (primes[i] > 64) return -1;
  }
  if (squarefree && small && np <= kMaxRadix) {
    // 2 x 3 as one axis of 6 (its butterfly a Good-Thomas 2 x 3 in
    // registers, dft_small<6>): one pass over the line in shared memory
    // fewer, the same FP64 operations
    bool has2 = false, has3 = false;
    for (int i = 0; i < np; ++i) { has2 = has2 || primes[i] == 2; has3 = has3 || primes[i] == 3; }
    if (has2 && has3) {
      int j = 0;
      for (int i = 0; i < np; ++i)
        if (primes[i] == 2) primes[j++] = 6;
        else if (primes[i] != 3) primes[j++] = primes[i];
      np = j;
    }
    f.pfa = 1;
    f.nrad = np;
    for (int i = 0; i < np; ++i) {
      const int Nd = primes[i], a = (P / Nd) % Nd;
      int c = 1;
      while ((a * c) % Nd != 1 % Nd) ++c;  // modular inverse, Nd <= 31 (gcd(a, Nd) = 1)
      f.rad[i] = Nd;
      f.cinv[i] = (Nd == 1) ? 0 : c;
    }
  } else {
    int k = 0;
    n = P;
    while (n % 4 == 0 && k < kMaxRadix) { f.rad[k++] = 4; n /= 4; }
    while (n % 2 == 0 && k < kMaxRadix) { f.rad[k++] = 2; n /= 2; }
    for (int q = 3; q * q <= n && k < kMaxRadix; q += 2)
      while (n % q == 0 && k < kMaxRadix) { f.rad[k++] = q; n /= q; }
    if (n > 1) {
      if (k >= kMaxRadix) return -1;
      f.rad[k++] = n;
    }
    if (n > 1 && n > 64) return -1;
    f.nrad = k;
  }
  *plan = f;
  return 0;
}

// Position of spectral index k in the transform's work array.
#ifdef __CUDACC__
__host__ __device__
#endif
inline int fft_position(const FftPlan& f, int k) {
  int span = f.P, pp = 0;
  if (f.pfa) {
    for (int i = 0; i < f.nrad; ++i) {
      span /= f.rad[i];
      pp += ((int)(((long long)k * f.cinv[i]) % f.rad[i])) * span;
    }
  } else {
    int x = k;
    for (int i = 0; i < f.nrad; ++i) {
      const int d = x % f.rad[i];
      x /= f.rad[i];
      span /= f.rad[i];
      pp += d * span;
    }
  }
  return pp;
}

// Tables of the transform of length plan.P, built on the host (falcon_host.cpp):
// tw[k] = exp(-2 pi i k/P) from the host's cos/sin and pos[k] =
// fft_position(plan, k).  Every entry point that runs the nonlinear pass
// takes its tables from here, so they all use the same bits.
void fft_tables_host(const FftPlan& plan, double2* tw, int* pos);

// Arguments of the nonlinear-pass kernel (Nr_maxLOOP, src/nonlin.F90:35-91).
struct NonlinArgs {
  int R, M, B, Nm;
  FftPlan plan;
  const double2* tw;    // exp(-2 pi i k/P), k < P
  const int* pos;       // digit-reversal positions, P entries
  const double2 *t, *w, *up, *ur;        // inputs  [r][m][b]
  double2 *ntp, *ntr, *nwp, *nwr;        // outputs [r][m][b]
  double* umax;                          // optional [r][b][2]: max|ur|, max|uphi|
};

// Y[row][n] = alpha * sum_k A[k*lda + row] * X[k*ldx + n] for
// row < rows, n < N, with a batch index z applying the strides sA, sX, sY.
struct GemmArgs {
  const double* A; long lda;
  const double* X; long ldx;
  double* Y; long ldy;
  int K, rows, N;
  long sA, sX, sY;
  int batch;
  double alpha;
  // Optional exact-slice copy of A for the tensor-core path (launch_gemm
  // uses it when set): slices of batch entry z at oz_s + z*oz_sz, row
  // exponents at oz_ex + z*oz_rowsP, this GEMM's first operator row oz_row0.
  const uint16_t* oz_s;
  const int* oz_ex;
  long oz_sz;
  int oz_rowsP, oz_KP, oz_row0;
  int oz_w;  // slice format (bits per slice) of A and X: 6 or 7
  // slices of X made by launch_oz_slice_cols: [batch][S][oz_KP][oz_Np]
  // bf16 and column exponents [batch][oz_Np]
  const uint16_t* oz_xs;
  const int* oz_cexp;
  int oz_Np;
  // tensor map (CUtensorMap) of the whole slice array of the operator and
  // this GEMM's first batch entry in it, for the tcgen05 kernel
  const void* oz_tmap;
  int oz_z0;
  // FP64 FMA tiles (no slice view): 0 = the tile shape of the cost model,
  // 16 / 32 / 64 = the cost model's best shape of that column width (every
  // shape sums each output over k in the same order: the same bits)
  int fma_ncol;
};

// ---- FP64 GEMM on bf16 tensor cores by exact slicing (falcon_ozaki.cu) ----
// An FP64 operand row (or column) with |a| < 2^e is cut into S signed
// integers of W bits, a = 2^e sum_s q_s 2^(-W (s+1)) up to 2^(e - S W).
// Slice products are exact in bf16 x bf16 -> FP32 and their sums stay
// below 2^24 (exact); the pairs s + t <= D are summed per s + t and
// recombined in 64-bit integers and one FP64 add.  Formats: W = 6 (S = 10,
// D = 9) for K <= 257, W = 7 (S = 9, D = 8) for K <= 112 (OzCfg in
// falcon_slices.cuh).  kOzS is the largest slice count (buffer sizes).
constexpr int kOzS = 10;
inline int oz_width_for(int KP) { return KP <= 112 ? 7 : 6; }
// Contractions of operators of 5 to 8 row tiles (65 <= rows <= 128) with
// few columns in all (N x batch <= 16384: one instance, small groups) take a
// kernel that slices its X columns itself: one launch fewer per contraction
// where launches dominate.  Larger ones read slice planes made once by
// launch_oz_slice_cols (shared by the contractions of one X), which costs
// less than slicing in every block.
inline bool oz_fused_x(int rows, int N, int batch) {
  const int rt = (rows + 15) / 16;
  return rt >= 5 && rt <= 8 && (long)N * batch <= 16384;
}
inline int oz_slices(int w) { return w == 7 ? 9 : 10; }
// Slices of a column-major FP64 operator (rows x K, lda, nb entries of
// stride sA) into S [nb][S][KP/8][rowsP][8] (bf16 bits, zero padded; row r,
// column k of a slice plane at ((k/8) rowsP + r) 8 + k%8) and row exponents
// ex [nb][rowsP].
cudaError_t launch_oz_slice_rows(const double* A, long lda, long sA, int rows, int K, int nb, uint16_t* S, int* ex,
                                 int rowsP, int KP, int w, cudaStream_t s);
// Slices of the columns of X (K x N, row stride ldx, batch stride sX) into
// Xs [batch][S][KP][Np] (zero for k >= K, n >= N) and column exponents
// cexp [batch][Np].  Np is a multiple of 32.
cudaError_t launch_oz_slice_cols(const double* X, long ldx, long sX, int K, int N, int batch, uint16_t* Xs,
                                 int* cexp, int KP, int Np, int w, cudaStream_t s);
// Y = alpha A X from the slices of A (oz_s, oz_ex) and of X (oz_xs, oz_cexp).
cudaError_t launch_oz_gemm(const GemmArgs& g, cudaStream_t s);
// Row padding of operator slices: rows_total rounded up to 16, plus 64
// (the row blocks of the tensor-core kernel cover up to 64 rows).
inline int oz_rows_padded(int rows) { return ((rows + 15) / 16) * 16 + 64; }

// Elementwise arguments shared by the right-hand-side kernels.
struct RhsArgs {
  int R, M, B;
  const double* inv_r;      // R
  const double* inv_r2;     // R
  const double* ra_pr;      // B: Ra/Pr per instance
  const double* inv_pr;     // B: 1/Pr per instance
  double dt;
  // IMEX multistep
  int scheme_cn;            // 1: Crank-Nicolson implicit part, 0: BDF
  int n_imp, n_exp;
  double w_imp[4], w_exp[4], wt_lhs;
  const double2* th[4];     // T history, th[0] = current state
  const double2* wh[4];     // omega history
  double2* nt_new;          // explicit term of T written for this step
  double2* nw_new;
  const double2* nth[4];    // explicit history, nth[0] aliases nt_new
  const double2* nwh[4];
  const double* ubh[4];     // uphi_bar history [r][b]
  double* urom_new;         // mean(ur*omg) written for this step
  const double* uromh[4];
  const double2 *ntp, *ntr, *dntr, *nwp, *nwr, *dnwr;
  const double2 *lt, *lw;   // L T and L omega (CN)
  const double2* lu0;       // L applied to uphi_bar, [r][b] complex (CN)
  double2 *rhs_t, *rhs_w;
  const double2* up;        // u_phi at the start of the step
  double* up0_prev;         // [r][b]: Re u_phi(m = 0) recorded there (optional)
};

// IMEXRK stage arguments (src/fourierloop_imexrk.F90).
struct StageArgs {
  int R, M, B, st;
  const double* inv_r;
  const double* inv_r2;
  const double* ra_pr;
  const double* inv_pr;     // B: 1/Pr per instance
  double dt;
  double aD[kMaxStages], aA[kMaxStages];   // row `st` of the Butcher tables
  double aD_ss;
  int buo_imp;
  const double2* t0; const double2* w0; const double* u0;
  const double2* fat[kMaxStages]; const double2* fdt[kMaxStages];
  const double2* faw[kMaxStages]; const double2* fdw[kMaxStages];
  const double2* buo[kMaxStages];
  double2 *rhs_t, *rhs_w;
  // stage derivatives (RHS_construct_stage)
  const double2 *ntp, *ntr, *dntr, *nwp, *nwr, *dnwr, *lt, *lw, *lu0, *t, *w, *up;
  double2 *fat_out, *fdt_out, *faw_out, *fdw_out, *buo_out;
};

// Diagnostics of every instance of a group (writeKE_spectral).
struct DiagArgs {
  int R, M, B, mbc_sf;
  const double2 *t, *w, *up, *ur, *tprev;
  const double *wq, *d1_0, *d1_R, *ra_pr;
  double nu_top_den, nu_bot_den, pi;
  double* out;   // 8 per instance
  double* part;  // 8 R B partial sums (radial row, instance)
};

// Non-stiffly-accurate IMEXRK assembly (elementwise part).
struct AsmArgs {
  int R, M, B, ns;
  double dt;
  double bA[kMaxStages], bD[kMaxStages];
  const double2* fat[kMaxStages]; const double2* fdt[kMaxStages];
  const double2* faw[kMaxStages]; const double2* fdw[kMaxStages];
  const double2* buo[kMaxStages];
  double2 *t0, *w0, *rhs_w;
  double* u0;
};

// ---- launchers (falcon_kernels.cu; the nonlinear pass dispatches to falcon_fft*.cu) ----
cudaError_t launch_nonlin(const NonlinArgs& a, cudaStream_t s);
cudaError_t launch_gemm(const GemmArgs& g, cudaStream_t s);
cudaError_t launch_imex_rhs(const RhsArgs& a, cudaStream_t s);
// rhs_w(m>=1) += coef_b * (i m / r) * t_new, coef_b = scale * ra_pr[b]
cudaError_t launch_add_buoyancy(int R, int M, int B, const double* inv_r, const double* ra_pr,
                                double scale, const double2* t_new, double2* rhs_w,
                                double2* buo_out, cudaStream_t s);
// u_r = i m psi / r for m >= 1; m = 0 from the uphi_bar solve output
// ub (rows 0..R-1: uphi_bar, rows R..2R-1: d uphi_bar/dr, columns 2*b+{0,1}).
cudaError_t launch_post_w(int R, int M, int B, const double* inv_r, const double2* psi,
                          double2* ur, double2* up, double2* w, const double* ub,
                          double* ubar_new, cudaStream_t s);
cudaError_t launch_stage_rhs(const StageArgs& a, cudaStream_t s);
cudaError_t launch_stage_deriv(const StageArgs& a, cudaStream_t s);
// Fortran (M,R) complex of instance b <-> device [r][m][b]
cudaError_t launch_scatter_instance(int R, int M, int B, int b, const double2* src, double2* dst,
                                    cudaStream_t s);
cudaError_t launch_scatter_columns(int R, int M, int B, const double2* src, double2* dst, cudaStream_t s);
cudaError_t launch_gather_instance(int R, int M, int B, int b, const double2* src, double2* dst,
                                   cudaStream_t s);
// dst[r][b] = src[r][0][b].x  (mode-0 real part)
cudaError_t launch_extract_mode0(int R, int M, int B, const double2* src, double* dst, cudaStream_t s);
cudaError_t launch_getrs_batched(int n, int nsys, int nrhs, const double* lu, const int* ipiv,
                                 double* b, cudaStream_t s);
// out[c] = A in[c] for ncol complex columns of length n (A real row-major).
cudaError_t launch_apply_cols(int n, int ncol, const double* A, const double2* in, double2* out, cudaStream_t s);
// Instance-column remap of a [rows][B] array (ew doubles per element).
cudaError_t launch_remap_cols(const double* src, double* dst, size_t rows, int bs, int bd, int ew, const int* map,
                              cudaStream_t s);
// Column b of a [rows][B] array: dst = src (or zero when src is null).
cudaError_t launch_col_op(const double* src, double* dst, size_t rows, int B, int b, int ew, cudaStream_t s);
cudaError_t launch_diagnostics(const DiagArgs& a, cudaStream_t s);
// calculate_spectra of every instance: ke, ts [b][m] (x four_pi)
cudaError_t launch_spectra(int R, int M, int B, const double2* t, const double2* ur, const double2* up,
                           const double* wq, double four_pi, double* ke, double* ts, cudaStream_t s);
// u_phi balance of every instance: out [b][r][3] = d(up_0)/dt, advection, diffusion
cudaError_t launch_upbalance(int R, int M, int B, const double2* ur, const double2* up, const double2* d1up,
                             const double* up0_prev, const double* Lp, const double* inv_r, const double* inv_r2,
                             double dt, double* out, cudaStream_t s);
cudaError_t launch_assembly(const AsmArgs& a, cudaStream_t s);
cudaError_t launch_assembly_post(int R, int M, int B, const double* inv_r, const double2* psi, const double* u0,
                                 const double* du0, double2* ur, double2* up, double2* w0, cudaStream_t s);
// ---- explicit RK (falcon_rk.cu) ----
// y_out = y0 + dt sum_i c_i F_i for T (with its boundary values), the
// vorticity of modes m >= 1 (all rows) and uphi_bar (held in the m = 0
// column of the vorticity stage arrays); rhs_w = -omega with zero boundary
// rows (m >= 1), 0 for m = 0.  Outputs may alias the y0 inputs.
struct RkCombineArgs {
  int R, M, B, nf;
  double dt;
  double c[kMaxStages];
  const double2* ft[kMaxStages]; const double2* fw[kMaxStages];
  const double2 *t0, *w0; const double* u0;
  double2 *t_out, *w_out, *rhs_w; double* u_out;
};
// Explicit right-hand sides of one stage (rhs_create_rk): temperature for
// every mode, vorticity for m >= 1, and uphi_bar into fw[(r, 0, b)].
struct RkRhsArgs {
  int R, M, B;
  const double* inv_pr;     // B: 1/Pr per instance
  const double *inv_r, *inv_r2, *ra_pr;
  const double2 *t, *w, *lt, *lw, *ntp, *ntr, *dntr, *nwp, *nwr, *dnwr;
  const double2 *up, *ur, *dup, *lub;  // lub: radial Laplacian of the m = 0 column, R x B
  double2 *ft, *fw;
};
cudaError_t launch_rk_combine(const RkCombineArgs& a, cudaStream_t s);
cudaError_t launch_rk_rhs(const RkRhsArgs& a, cudaStream_t s);
cudaError_t launch_rk_ubar(const RkRhsArgs& a, cudaStream_t s);
// ---- operator construction (falcon_ops.cu) ----
// kind 0: AT, kind 4: LAPpsi (R x R column-major per mode, modes m0..)
cudaError_t launch_assemble(int kind, int R, int m0, int nmodes, const double* t, const double* D, const double* D2,
                            const double* inv_r, const double* inv_r2, double wdt, double inv_pr, double C,
                            double* out, cudaStream_t s);
// AF (2R x 2R column-major per mode), irk selects the IMEXRK boundary-row order
cudaError_t launch_assemble_af(int R, int m0, int nmodes, int mbc, int irk, const double* t, const double* D,
                               const double* D2, const double* inv_r, const double* inv_r2, double wdt, double C,
                               double* out, cudaStream_t s);
// dgetrf + dgetrs per matrix; rhs row-major (n x nrhs); mats may be overwritten
cudaError_t launch_lu_solve(int n, int nb, double* mats, size_t mstride, double* rhs, size_t rstride, int nrhs,
                            int* info, cudaStream_t s);
cudaError_t launch_unit_rhs(int n, int nrhs, int off, int nb, double* out, cudaStream_t s);
// dgetrs only, with given factors (column-major n x n, stride mstride) and
// 1-based pivots (stride pstride); rhs row-major (n x nrhs), stride rstride
cudaError_t launch_getrs_rows(int n, int nb, const double* lu, size_t mstride, const int* ipiv, size_t pstride,
                              double* rhs, size_t rstride, int nrhs, cudaStream_t s);
// Self-timed FP64 FMA throughput kernel (returns GFLOP/s, or < 0 on error).
double measure_fp64_peak();
// Same for the FP64 tensor-core MMA (mma.sync m8n8k4 f64).
double measure_fp64_mma_peak();
// Set the odd-prime DFT coefficient tables (constant memory); idempotent.
cudaError_t init_dft_tables();

}  // namespace falcon
