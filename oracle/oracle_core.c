/*
 * CPU oracle for the FAlCon-DNS per-time-step hot path (TEST INFRASTRUCTURE).
 *
 * A plain-C FP64 restatement of the reference Fortran, used only by tests/,
 * __graft_entry__.smoke() and the cpu_baseline leg of bench.py as the
 * checker and the timed CPU baseline.  Every routine cites the reference
 * file:line it follows (paths relative to the FAlCon-DNS project root).
 * OpenMP parallelism is placed exactly where the reference has it: the loop
 * over Fourier modes (src/fourierloop.F90:211-215,
 * src/fourierloop_imexrk.F90:162-168,519-525); the radial loop of the
 * nonlinear pass stays serial as in src/nonlin.F90:52-54.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle.h"
#include "imexrk_tables.h"

#define PI_ (4.0 * atan(1.0))

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* Azimuthal transforms: src/fourier_fftw.F90:39-57 (forfft), :76-97 (invfft) */
/* ------------------------------------------------------------------------ */

/* forfft: r2c of the real line, divided by Np, truncated to modes 0..Nm. */
void orc_forfft(int nm, int np, const double* ff, double* f) {
  double* z = (double*)malloc(sizeof(double) * 4 * (size_t)np);
  double* zo = z + 2 * np;
  for (int j = 0; j < np; ++j) { z[2 * j] = ff[j]; z[2 * j + 1] = 0.0; }
  orc_fft(np, z, zo, -1);
  for (int m = 0; m <= nm; ++m) {
    f[2 * m] = zo[2 * m] / (double)np;
    f[2 * m + 1] = zo[2 * m + 1] / (double)np;
  }
  free(z);
}

/* invfft: modes 0..Nm zero-padded to Np/2+1, unnormalised c2r.  A c2r
 * transform reads only the Hermitian half; the imaginary part of the mean
 * mode does not contribute. */
void orc_invfft(int nm, int np, const double* f, double* ff) {
  double* z = (double*)calloc(4 * (size_t)np, sizeof(double));
  double* zo = z + 2 * np;
  z[0] = f[0]; z[1] = 0.0;
  for (int m = 1; m <= nm; ++m) {
    z[2 * m] = f[2 * m]; z[2 * m + 1] = f[2 * m + 1];
    z[2 * (np - m)] = f[2 * m]; z[2 * (np - m) + 1] = -f[2 * m + 1];
  }
  orc_fft(np, z, zo, +1);
  for (int j = 0; j < np; ++j) ff[j] = zo[2 * j];
  free(z);
}

/* ------------------------------------------------------------------------ */
/* Chebyshev collocation: src/chebyshev_fftw.F90                             */
/* ------------------------------------------------------------------------ */

/* dcheb, src/chebyshev_fftw.F90:88-121.  Outputs t(i,j)=T_{j-1}(x_i),
 * D = 2 dT/dx, D2 = 4 d2T/dx2, column-major (R,R). */
void orc_dcheb(int nr, double* xp, double* t, double* d, double* d2) {
  double* tt = (double*)malloc(sizeof(double) * nr * nr);
  double* dt = (double*)malloc(sizeof(double) * nr * nr);
  double* d2t = (double*)malloc(sizeof(double) * nr * nr);
  const double pi = PI_;
  for (int i = 0; i < nr; ++i) xp[i] = cos(((double)(nr - 1 - i) * pi) / (double)(nr - 1));
  /* tt(j,i): polynomial j at point i (before the transposes of the reference) */
#define A_(a, j, i) a[(j) + nr * (i)]
  for (int i = 0; i < nr; ++i) {
    A_(tt, 0, i) = 1.0; A_(tt, 1, i) = xp[i];
    A_(dt, 0, i) = 0.0; A_(dt, 1, i) = 1.0;
    A_(d2t, 0, i) = 0.0; A_(d2t, 1, i) = 0.0;
    for (int j = 2; j < nr; ++j) {
      A_(tt, j, i) = 2.0 * xp[i] * A_(tt, j - 1, i) - A_(tt, j - 2, i);
      A_(dt, j, i) = 2.0 * A_(tt, j - 1, i) + 2.0 * xp[i] * A_(dt, j - 1, i) - A_(dt, j - 2, i);
      A_(d2t, j, i) = 4.0 * A_(dt, j - 1, i) + 2.0 * xp[i] * A_(d2t, j - 1, i) - A_(d2t, j - 2, i);
    }
  }
  for (int i = 0; i < nr; ++i)
    for (int j = 0; j < nr; ++j) {
      t[i + nr * j] = A_(tt, j, i);
      d[i + nr * j] = 2.0 * A_(dt, j, i);
      d2[i + nr * j] = 4.0 * A_(d2t, j, i);
    }
#undef A_
  free(tt); free(dt); free(d2t);
}

/* chebtransform, src/chebyshev_fftw.F90:124-155: values (x ascending) to the
 * scaled Chebyshev coefficients via the length-(2R-2) even extension. */
void orc_chebtransform(int nr, const double* f, double* ft) {
  int L = 2 * nr - 2;
  double* f00 = (double*)malloc(sizeof(double) * 4 * (size_t)L);
  double* ff = f00 + 2 * L;
  for (int i = 0; i < nr; ++i) {  /* f0 = f reversed */
    f00[2 * i] = f[2 * (nr - 1 - i)]; f00[2 * i + 1] = f[2 * (nr - 1 - i) + 1];
  }
  for (int i = 1; i < nr - 1; ++i) {  /* f00(Nr+1:2Nr-2) = f(2:Nr-1) */
    f00[2 * (nr - 1 + i)] = f[2 * i]; f00[2 * (nr - 1 + i) + 1] = f[2 * i + 1];
  }
  orc_fft(L, f00, ff, +1); /* FFTW_BACKWARD plan */
  double fac = sqrt(2.0 / (double)(nr - 1));
  for (int k = 0; k < nr; ++k) {
    double re = ff[2 * k] / (double)L, im = ff[2 * k + 1] / (double)L;
    if (k != 0 && k != nr - 1) { re = 2.0 * re; im = 2.0 * im; }
    re = re / fac; im = im / fac;
    if (k == 0 || k == nr - 1) { re = 2.0 * re; im = 2.0 * im; }
    ft[2 * k] = re; ft[2 * k + 1] = im;
  }
  free(f00);
}

/* REDFT00 of length n applied to re and im parts: Y_k = X_0 + (-1)^k X_{n-1}
 * + 2 sum_{j=1}^{n-2} X_j cos(pi j k/(n-1)), computed through the complex
 * FFT of the even extension. */
static void redft00_cplx(int n, const double* x, double* y) {
  int L = 2 * n - 2;
  double* e = (double*)calloc(4 * (size_t)L, sizeof(double));
  double* eo = e + 2 * L;
  for (int j = 0; j < n; ++j) { e[2 * j] = x[2 * j]; e[2 * j + 1] = x[2 * j + 1]; }
  for (int j = 1; j < n - 1; ++j) {
    e[2 * (L - j)] = x[2 * j]; e[2 * (L - j) + 1] = x[2 * j + 1];
  }
  orc_fft(L, e, eo, -1);
  for (int k = 0; k < n; ++k) { y[2 * k] = eo[2 * k]; y[2 * k + 1] = eo[2 * k + 1]; }
  free(e);
}

/* chebinvtran, src/chebyshev_fftw.F90:157-194. */
void orc_chebinvtran(int nr, const double* ft, double* ff) {
  double* y = (double*)malloc(sizeof(double) * 2 * (size_t)nr);
  redft00_cplx(nr, ft, y);
  double fact = sqrt(2.0 / (double)(nr - 1));
  for (int i = 0; i < nr; ++i) {
    int k = nr - 1 - i;
    ff[2 * i] = y[2 * k] * 0.5 * fact;
    ff[2 * i + 1] = y[2 * k + 1] * 0.5 * fact;
  }
  free(y);
}

/* Derivative-coefficient recurrence, src/chebyshev_fftw.F90:263-271. */
static void deriv_coeffs(int nr, const double* f, double* beta) {
  beta[2 * (nr - 1)] = 0.0; beta[2 * (nr - 1) + 1] = 0.0;
  beta[2 * (nr - 2)] = 2.0 * (double)(nr - 1) * f[2 * (nr - 1)];
  beta[2 * (nr - 2) + 1] = 2.0 * (double)(nr - 1) * f[2 * (nr - 1) + 1];
  for (int i = nr - 1; i >= 2; --i) { /* Fortran i; beta(i-1) = beta(i+1) + 4(i-1) f(i) */
    beta[2 * (i - 2)] = beta[2 * i] + 4.0 * (double)(i - 1) * f[2 * (i - 1)];
    beta[2 * (i - 2) + 1] = beta[2 * i + 1] + 4.0 * (double)(i - 1) * f[2 * (i - 1) + 1];
  }
}

/* Inverse of a derivative series, src/chebyshev_fftw.F90:269-288. */
static void deriv_inverse(int nr, double* beta, double* df) {
  int L = 2 * nr - 2;
  double fact = sqrt(2.0 / (double)(nr - 1));
  for (int i = 0; i < 2 * nr; ++i) beta[i] = beta[i] * fact;
  beta[0] /= 2.0; beta[1] /= 2.0;
  beta[2 * (nr - 1)] /= 2.0; beta[2 * (nr - 1) + 1] /= 2.0;
  double* f2c = (double*)malloc(sizeof(double) * 4 * (size_t)L);
  double* f2r = f2c + 2 * L;
  f2c[0] = beta[0]; f2c[1] = beta[1];
  for (int i = 1; i < nr; ++i) { f2c[2 * i] = beta[2 * i] / 2.0; f2c[2 * i + 1] = beta[2 * i + 1] / 2.0; }
  for (int i = 0; i < nr - 2; ++i) { /* f2c(Nr+1:2Nr-2) = beta1(Nr-1:2:-1)/2 */
    int src = nr - 2 - i;
    f2c[2 * (nr + i)] = beta[2 * src] / 2.0;
    f2c[2 * (nr + i) + 1] = beta[2 * src + 1] / 2.0;
  }
  orc_fft(L, f2c, f2r, -1); /* FFTW_FORWARD plan */
  for (int i = 0; i < nr; ++i) {
    df[2 * i] = f2r[2 * (nr - 1 - i)];
    df[2 * i + 1] = f2r[2 * (nr - 1 - i) + 1];
  }
  free(f2c);
}

/* chebinvtranD1, src/chebyshev_fftw.F90:247-291. */
void orc_chebinvtranD1(int nr, const double* ft, double* df) {
  double* b1 = (double*)malloc(sizeof(double) * 2 * (size_t)nr);
  deriv_coeffs(nr, ft, b1);
  deriv_inverse(nr, b1, df);
  free(b1);
}

/* chebinvtranD2, src/chebyshev_fftw.F90:293-352. */
void orc_chebinvtranD2(int nr, const double* ft, double* d2f) {
  double* b1 = (double*)malloc(sizeof(double) * 4 * (size_t)nr);
  double* b2 = b1 + 2 * nr;
  deriv_coeffs(nr, ft, b1);
  deriv_coeffs(nr, b1, b2);
  deriv_inverse(nr, b2, d2f);
  free(b1);
}

/* chebinvtranD1D2, src/chebyshev_fftw.F90:354-427. */
void orc_chebinvtranD1D2(int nr, const double* ft, double* df, double* d2f) {
  double* b1 = (double*)malloc(sizeof(double) * 4 * (size_t)nr);
  double* b2 = b1 + 2 * nr;
  deriv_coeffs(nr, ft, b1);
  deriv_coeffs(nr, b1, b2);
  deriv_inverse(nr, b1, df);
  deriv_inverse(nr, b2, d2f);
  free(b1);
}

/* Lagrange derivative weights, src/chebyshev_fftw.F90:449-478 (dlagrange)
 * and :480-517 (d2lagrange). */
static void dlagrange(int n, const double* xp, double x, double* dw) {
  double* w = (double*)malloc(sizeof(double) * n);
  double* ww = (double*)malloc(sizeof(double) * n);
  for (int i = 0; i < n; ++i) { dw[i] = 0.0; w[i] = 1.0; ww[i] = 0.0; }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      w[i] = 1.0;
      if (i != j) {
        for (int m = 0; m < n; ++m)
          if (m != i && m != j) w[i] = w[i] * (x - xp[m]) / (xp[j] - xp[m]);
        ww[i] = w[i] / (xp[j] - xp[i]);
        dw[j] = dw[j] + ww[i];
      }
    }
  free(w); free(ww);
}

static void d2lagrange(int n, const double* xp, double x, double* d2w) {
  double* w = (double*)malloc(sizeof(double) * n);
  double* ww = (double*)malloc(sizeof(double) * n);
  double* mw = (double*)malloc(sizeof(double) * n);
  for (int i = 0; i < n; ++i) { d2w[i] = 0.0; w[i] = 1.0; ww[i] = 0.0; mw[i] = 0.0; }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i)
      if (i != j) {
        mw[i] = 0.0;
        for (int m = 0; m < n; ++m)
          if (m != i && m != j) {
            w[i] = 1.0;
            for (int l = 0; l < n; ++l)
              if (l != j && l != i && l != m) w[i] = w[i] * (x - xp[l]) / (xp[j] - xp[l]);
            ww[i] = w[i] / (xp[j] - xp[m]);
            mw[i] = mw[i] + ww[i];
          }
        d2w[j] = d2w[j] + mw[i] / (xp[j] - xp[i]);
      }
  free(w); free(ww); free(mw);
}

/* ------------------------------------------------------------------------ */
/* Dense LU: src/algebra_lapack.F90:14-53 (dgetrf / dgetrs 'N')              */
/* Restates LAPACK's right-looking partial-pivoting LU (first index of the   */
/* maximum modulus as pivot) and the column-oriented triangular solves.      */
/* ------------------------------------------------------------------------ */
int orc_dgetrf(int n, double* a, int* ipiv) {
  int info = 0;
  for (int j = 0; j < n; ++j) {
    int p = j;
    double amax = fabs(a[j + n * j]);
    for (int i = j + 1; i < n; ++i) {
      double v = fabs(a[i + n * j]);
      if (v > amax) { amax = v; p = i; }
    }
    ipiv[j] = p + 1;
    if (a[p + n * j] != 0.0) {
      if (p != j)
        for (int k = 0; k < n; ++k) {
          double tmp = a[j + n * k]; a[j + n * k] = a[p + n * k]; a[p + n * k] = tmp;
        }
      double piv = a[j + n * j];
      if (fabs(piv) >= 2.2250738585072014e-308) {
        double rp = 1.0 / piv;
        for (int i = j + 1; i < n; ++i) a[i + n * j] *= rp;
      } else {
        for (int i = j + 1; i < n; ++i) a[i + n * j] /= piv;
      }
    } else if (info == 0) {
      info = j + 1;
    }
    for (int k = j + 1; k < n; ++k) {
      double akj = a[j + n * k];
      if (akj != 0.0)
        for (int i = j + 1; i < n; ++i) a[i + n * k] -= a[i + n * j] * akj;
    }
  }
  return info;
}

void orc_dgetrs(int n, const double* a, const int* ipiv, double* b) {
  for (int i = 0; i < n; ++i) {
    int p = ipiv[i] - 1;
    if (p != i) { double t = b[i]; b[i] = b[p]; b[p] = t; }
  }
  for (int j = 0; j < n; ++j) { /* L, unit diagonal */
    double bj = b[j];
    if (bj != 0.0)
      for (int i = j + 1; i < n; ++i) b[i] -= bj * a[i + n * j];
  }
  for (int j = n - 1; j >= 0; --j) { /* U */
    if (b[j] != 0.0) {
      b[j] = b[j] / a[j + n * j];
      double bj = b[j];
      for (int i = 0; i < j; ++i) b[i] -= bj * a[i + n * j];
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Nonlinear pass: src/nonlin.F90:35-91                                      */
/* ------------------------------------------------------------------------ */
static void nonlin_line(int nm, int np, const double* t_m, const double* o_m,
                        const double* up_m, const double* ur_m, double* tt, double* og,
                        double* upg, double* urg, double* f1, double* f2, double* f3,
                        double* f4, double* work) {
  orc_invfft(nm, np, t_m, tt);
  orc_invfft(nm, np, o_m, og);
  orc_invfft(nm, np, up_m, upg);
  orc_invfft(nm, np, ur_m, urg);
  double* a = work;
  double* b = work + np;
  for (int i = 0; i < np; ++i) { a[i] = upg[i] * tt[i]; b[i] = urg[i] * tt[i]; }
  orc_forfft(nm, np, a, f1);
  orc_forfft(nm, np, b, f2);
  for (int i = 0; i < np; ++i) { a[i] = upg[i] * og[i]; b[i] = urg[i] * og[i]; }
  orc_forfft(nm, np, a, f3);
  orc_forfft(nm, np, b, f4);
}

void orc_nonlin(int nm, int nr, const double* tFR, const double* omgFR,
                const double* upFR, const double* urFR, double* uphi_temp,
                double* ur_temp, double* uphi_omg, double* ur_omg) {
  int M = nm + 1, np = 3 * nm;
  double* g = (double*)malloc(sizeof(double) * 6 * (size_t)np);
  double* in = (double*)malloc(sizeof(double) * 8 * (size_t)M);
  double* out = (double*)malloc(sizeof(double) * 8 * (size_t)M);
  for (int r = 0; r < nr; ++r) {
    nonlin_line(nm, np, tFR + 2 * (size_t)M * r, omgFR + 2 * (size_t)M * r,
                upFR + 2 * (size_t)M * r, urFR + 2 * (size_t)M * r, g, g + np, g + 2 * np,
                g + 3 * np, uphi_temp + 2 * (size_t)M * r, ur_temp + 2 * (size_t)M * r,
                uphi_omg + 2 * (size_t)M * r, ur_omg + 2 * (size_t)M * r, g + 4 * np);
  }
  free(g); free(in); free(out);
}

/* ------------------------------------------------------------------------ */
/* Time-scheme tables: src/timeschemes.F90                                   */
/* ------------------------------------------------------------------------ */
typedef struct {
  int n_imp, n_exp;          /* n_order_tscheme_imp / _exp (stages for RK) */
  double wt_lhs;
  double w_imp[4], w_exp[4];
  double aD[8][8], bD[8], aA[8][8], bA[8];
  int check_A, check_D, diag_index; /* diag_index 0-based */
  int diag_diff;             /* implicit diagonal varies by stage */
} scheme_t;

/* Variable-dt multistep weights with dt_array(1..4); constant dt reduces them
 * to the textbook coefficients.  CN :1004-1006, BDF2 :1008-1015,
 * BDF3 :1017-1027, BDF4 :1029-1052; AB2 :1628-1630, AB3 :1632-1638
 * (CN/AB3), BDF2/AB2 :1643-1651, BDF3/AB3 :1655-1668, BDF4/AB4 :1672-1701. */
static void multistep_weights(const orc_params* p, const double* dta, scheme_t* s) {
  switch (p->scheme_imp) {
    case ORC_IMP_CN:
      s->w_imp[0] = 0.5; s->wt_lhs = 0.5; break;
    case ORC_IMP_BDF2: {
      double r1 = dta[1] / dta[0];
      double a0 = (2.0 + r1) / (1.0 + r1), a1 = 1.0 + 1.0 / r1;
      double a2 = -1.0 * (1.0 / r1 / (1.0 + r1));
      s->wt_lhs = 1.0 / a0; s->w_imp[0] = a1 / a0; s->w_imp[1] = a2 / a0;
    } break;
    case ORC_IMP_BDF3: {
      double r1 = dta[1] / dta[0], r2 = dta[2] / dta[0];
      double a0 = (1.0 + 1.0 / (1.0 + r1) + 1.0 / (1.0 + r1 + r2));
      double a1 = (((1.0 + r1) * (1.0 + r1 + r2)) / (r1 * (r1 + r2)));
      double a2 = (-1.0 * (1.0 + r1 + r2) / (r1 * r2 * (1.0 + r1)));
      double a3 = ((1.0 + r1) / (r2 * (r1 + r2) * (1.0 + r1 + r2)));
      s->wt_lhs = 1.0 / a0; s->w_imp[0] = a1 / a0; s->w_imp[1] = a2 / a0; s->w_imp[2] = a3 / a0;
    } break;
    case ORC_IMP_BDF4: {
      double r1 = dta[0] / dta[1], r2 = dta[1] / dta[2], r3 = dta[2] / dta[3];
      double c1 = 1.0 + r3 * (1.0 + r2), c2 = 1.0 + r2 * (1.0 + r1), c3 = 1.0 + r3 * c2;
      double a0 = 1.0 + r1 / (1.0 + r1) + r2 * r1 / c2 + r3 * r2 * r1 / c3;
      double a1 = -1.0 - r1 * (1.0 + r2 * (1.0 + r1) * (1.0 + r3 * c2 / c1) / (1.0 + r2));
      double a2 = r1 * (r1 / (1.0 + r1) + r2 * r1 * (c3 + r3) / (1.0 + r3));
      double a3 = -pow(r2, 3) * pow(r1, 2) * (1.0 + r1) / (1.0 + r2) * c3 / c2;
      double a4 = (1.0 + r1) / (1.0 + r3) * c2 / c1 / c3 * (pow(r3, 4) * pow(r2, 3) * pow(r1, 2));
      s->wt_lhs = 1.0 / a0;
      s->w_imp[0] = -a1 / a0; s->w_imp[1] = -a2 / a0; s->w_imp[2] = -a3 / a0; s->w_imp[3] = -a4 / a0;
    } break;
  }
  switch (p->scheme_imp) {
    case ORC_IMP_CN:
      if (p->scheme_exp == ORC_EXP_AB2) {
        s->w_exp[0] = 1.0 + 0.5 * dta[0] / dta[1];
        s->w_exp[1] = -0.5 * dta[0] / dta[1];
      } else { /* AB3 */
        s->w_exp[1] = (dta[0] * dta[2] * 0.5 + (1.0 / 6.0) * dta[0] * dta[0]) /
                      (dta[1] * dta[1] * 0.5 - dta[1] * dta[2]);
        s->w_exp[2] = (-dta[0] * 0.5 - dta[1] * s->w_exp[1]) * 0.5 / (dta[2]);
        s->w_exp[0] = 1.0 - s->w_exp[1] - s->w_exp[2];
      }
      break;
    case ORC_IMP_BDF2: {
      double r1 = dta[1] / dta[0];
      double a0 = (2.0 + r1) / (1.0 + r1), b0 = 1.0 + 1.0 / r1, b1 = -1.0 / r1;
      s->w_exp[0] = b0 / a0; s->w_exp[1] = b1 / a0;
    } break;
    case ORC_IMP_BDF3: {
      double r1 = dta[1] / dta[0], r2 = dta[2] / dta[0];
      double a0 = (1.0 + 1.0 / (1.0 + r1) + 1.0 / (1.0 + r1 + r2));
      double b0 = 1.0 * ((1.0 + r1) * (1.0 + r1 + r2)) / (r1 * (r1 + r2));
      double b1 = 1.0 * (-(1.0 + r1 + r2) / (r1 * r2));
      double b2 = 1.0 * (1.0 + r1) / (r2 * (r1 + r2));
      s->w_exp[0] = b0 / a0; s->w_exp[1] = b1 / a0; s->w_exp[2] = b2 / a0;
    } break;
    case ORC_IMP_BDF4: {
      double r1 = dta[0] / dta[1], r2 = dta[1] / dta[2], r3 = dta[2] / dta[3];
      double c1 = 1.0 + r3 * (1.0 + r2), c2 = 1.0 + r2 * (1.0 + r1), c3 = 1.0 + r3 * c2;
      double a0 = 1.0 + r1 / (1.0 + r1) + r2 * r1 / c2 + r3 * r2 * r1 / c3;
      double b3 = -pow(r3, 3) * pow(r2, 2) * r1 * (1.0 + r1) / (1.0 + r3) * c2 / c1;
      double b2 = pow(r2, 2) * r1 * (1.0 + r1) / (1.0 + r2) * c3;
      double b1 = -c2 * c3 * r1 / (1.0 + r3);
      double b0 = r2 * (1.0 + r1) / (1.0 + r2) * ((1.0 + r1) * (c3 + r3) + (1.0 + r3) / r2) / c1;
      s->w_exp[0] = b0 / a0; s->w_exp[1] = b1 / a0; s->w_exp[2] = b2 / a0; s->w_exp[3] = b3 / a0;
    } break;
  }
}

/* Butcher pairs: init_time_schemes src/timeschemes.F90:37-973 (stage counts),
 * rhs_update_wts_imp :1053-1612 and rhs_update_wts_exp :1733-2388. */
/* IMEXRK Butcher tables (src/timeschemes.F90) from the shared table of
 * published coefficients (up to 8 stages). */
static int butcher_tables(const orc_params* p, scheme_t* s) {
  imexrk_table t;
  memset(s->aD, 0, sizeof(s->aD)); memset(s->aA, 0, sizeof(s->aA));
  memset(s->bD, 0, sizeof(s->bD)); memset(s->bA, 0, sizeof(s->bA));
  if (imexrk_table_get(p->scheme_imp, p->scheme_exp, &t) != 0 || t.n > 8) return -1;
  for (int i = 0; i < t.n; ++i) {
    for (int j = 0; j < t.n; ++j) { s->aD[i][j] = t.aD[i][j]; s->aA[i][j] = t.aA[i][j]; }
    s->bD[i] = t.bD[i]; s->bA[i] = t.bA[i];
  }
  s->check_A = t.check_A; s->check_D = t.check_D; s->diag_index = t.diag_index - 1;
  s->diag_diff = t.diag_diff;
  s->n_imp = t.n; s->n_exp = t.n;
  return 0;
}

/* Exported for the table tests: n, then aD (n x n), bD, aA, bA, then
 * check_D, check_A, diag_index (1-based); returns -1 if not built. */
int orc_imexrk_table(int scheme, double* out) {
  imexrk_table t;
  if (imexrk_table_get(scheme, scheme, &t) != 0) return -1;
  int n = t.n, k = 0;
  out[k++] = n;
  for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) out[k++] = t.aD[i][j];
  for (int i = 0; i < n; ++i) out[k++] = t.bD[i];
  for (int i = 0; i < n; ++i) for (int j = 0; j < n; ++j) out[k++] = t.aA[i][j];
  for (int i = 0; i < n; ++i) out[k++] = t.bA[i];
  out[k++] = t.check_D; out[k++] = t.check_A; out[k++] = t.diag_index; out[k++] = t.diag_diff;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Simulation state (module globals of src/init.F90:19-56,                   */
/* src/timeschemes.F90:12-25, src/mat_assembly.F90:16-27 gathered per handle) */
/* ------------------------------------------------------------------------ */
struct orc_sim {
  orc_params p;
  int R, M, Nm, P;
  double rmin, rmax;
  double *xp, *t, *D, *D2;
  double *radius, *r_radius, *r_radius2, *dr;
  /* complex (M,R) fields, element (m,r) at 2*(m + M*r) */
  double *tFR, *omgFR, *upFR, *urFR, *psii, *temp_spec, *omg_spec, *upFC;
  double *upFR_prev, *urFR_prev;
  double *uphi_bar_spec; /* complex (R) */
  double *TFC;           /* complex (R) */
  /* physical grids (Np,R), element (j,r) at j + P*r */
  double *tt, *up, *ur, *omg;
  /* products of the nonlinear pass */
  double *uphi_temp_FR, *ur_temp_FR, *uphi_omg_FR, *ur_omg_FR;
  /* IMEX history (order, M, R) and their copies */
  double *rhs_imp_temp, *rhs_exp_temp, *rhs_imp_vort, *rhs_exp_vort, *rhs_buo_term;
  double *tmp_imp_temp, *tmp_exp_temp, *tmp_imp_vort, *tmp_exp_vort, *tmp_buo_term;
  double *rhs_imp_uphi, *rhs_exp_uphi, *tmp_imp_uphi, *tmp_exp_uphi; /* complex (order,R) */
  /* IMEXRK stage derivatives (stage, M, R) */
  double *dtemp_a, *dtemp_d, *domg_a, *domg_d, *rhs_buo;
  /* operators */
  double *AT_all, *AF_all, *A_uphi; int *ipiv1, *ipiv2, *ipiv_uphi;
  /* diag_diff: the operators of stages whose diagonal differs from that of
   * stage diag_index (AT_all_IRK(:,:,:,rk_stage), ...), else NULL */
  double *AT_st[8], *AF_st[8], *Au_st[8]; int *p1_st[8], *p2_st[8], *pu_st[8];
  double *LAPpsi_all; int *ipiv_lap;
  double *dw_rmin, *d2w_rmin, *dw_rmax, *d2w_rmax;
  double *dtval_r, *dtval_p, *dtval_rkr, *dtval_rkp;  /* get_dtvals of the last nonlinear pass */
  scheme_t sch;
  double dt_array[4];
  double dt_new, tot_time;
  int n_step;      /* steps completed (since the start or the restart) */
  int mats_built;
  int restarted;   /* l_restart: the run continues from checkpoint files */
};

#define CX(a, m, r) ((a) + 2 * ((size_t)(m) + (size_t)M * (r)))
#define HX(a, i, m, r) ((a) + 2 * ((size_t)(i) + (size_t)nord * ((size_t)(m) + (size_t)M * (r))))

static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* init_grid, src/init.F90:120-162 */
static void init_grid(orc_sim* s) {
  int R = s->R;
  const double pi = PI_;
  for (int i = 0; i < R; ++i) {
    s->radius[i] = (s->rmin + (0.5 * (1.0 + cos((double)(R - 1 - i) * pi / (double)(R - 1)))));
    s->r_radius[i] = 1.0 / s->radius[i];
  }
  for (int i = 0; i < R - 1; ++i) s->dr[i + 1] = s->radius[i + 1] - s->radius[i];
  s->dr[0] = s->dr[1];
  for (int i = 0; i < R; ++i) s->r_radius2[i] = s->r_radius[i] * s->r_radius[i];
}

orc_sim* orc_sim_create(const orc_params* p) {
  if (p->nr_max < 4 || p->nm_max < 1) return NULL;
  orc_sim* s = (orc_sim*)calloc(1, sizeof(orc_sim));
  s->p = *p;
  s->R = p->nr_max; s->Nm = p->nm_max; s->M = p->nm_max + 1; s->P = 3 * p->nm_max;
  s->rmin = p->eta / (1.0 - p->eta);   /* src/namelists.F90:106-107 */
  s->rmax = 1.0 / (1.0 - p->eta);
  int R = s->R, M = s->M, P = s->P;
  size_t cf = 2 * (size_t)M * R;
  s->xp = zalloc(R); s->t = zalloc((size_t)R * R); s->D = zalloc((size_t)R * R); s->D2 = zalloc((size_t)R * R);
  orc_dcheb(R, s->xp, s->t, s->D, s->D2);
  s->radius = zalloc(R); s->r_radius = zalloc(R); s->r_radius2 = zalloc(R); s->dr = zalloc(R);
  init_grid(s);
  s->tFR = zalloc(cf); s->omgFR = zalloc(cf); s->upFR = zalloc(cf); s->urFR = zalloc(cf);
  s->psii = zalloc(cf); s->temp_spec = zalloc(cf); s->omg_spec = zalloc(cf); s->upFC = zalloc(cf);
  s->upFR_prev = zalloc(cf); s->urFR_prev = zalloc(cf);
  s->uphi_bar_spec = zalloc(2 * (size_t)R); s->TFC = zalloc(2 * (size_t)R);
  s->tt = zalloc((size_t)P * R); s->up = zalloc((size_t)P * R); s->ur = zalloc((size_t)P * R);
  s->omg = zalloc((size_t)P * R);
  s->uphi_temp_FR = zalloc(cf); s->ur_temp_FR = zalloc(cf); s->uphi_omg_FR = zalloc(cf);
  s->ur_omg_FR = zalloc(cf);
  for (int i = 0; i < 4; ++i) s->dt_array[i] = p->dt;
  if (p->scheme_type == ORC_TYPE_IMEX) {
    int ni = 0, ne = 0;
    switch (p->scheme_imp) {
      case ORC_IMP_CN: ni = 2; ne = (p->scheme_exp == ORC_EXP_AB3) ? 3 : 2; break;
      case ORC_IMP_BDF2: ni = 2; ne = 2; break;
      case ORC_IMP_BDF3: ni = 3; ne = 3; break;
      case ORC_IMP_BDF4: ni = 4; ne = 4; break;
      default: orc_sim_destroy(s); return NULL;
    }
    s->sch.n_imp = ni; s->sch.n_exp = ne;
    s->rhs_imp_temp = zalloc(cf * ni); s->tmp_imp_temp = zalloc(cf * ni);
    s->rhs_imp_vort = zalloc(cf * ni); s->tmp_imp_vort = zalloc(cf * ni);
    s->rhs_buo_term = zalloc(cf * ni); s->tmp_buo_term = zalloc(cf * ni);
    s->rhs_exp_temp = zalloc(cf * ne); s->tmp_exp_temp = zalloc(cf * ne);
    s->rhs_exp_vort = zalloc(cf * ne); s->tmp_exp_vort = zalloc(cf * ne);
    s->rhs_imp_uphi = zalloc(2 * (size_t)R * ni); s->tmp_imp_uphi = zalloc(2 * (size_t)R * ni);
    s->rhs_exp_uphi = zalloc(2 * (size_t)R * ne); s->tmp_exp_uphi = zalloc(2 * (size_t)R * ne);
    s->AT_all = zalloc((size_t)R * R * M); s->AF_all = zalloc((size_t)4 * R * R * M);
    s->A_uphi = zalloc((size_t)R * R);
    s->ipiv1 = (int*)calloc((size_t)R * M, sizeof(int));
    s->ipiv2 = (int*)calloc((size_t)2 * R * M, sizeof(int));
    s->ipiv_uphi = (int*)calloc((size_t)R, sizeof(int));
  } else if (p->scheme_type == ORC_TYPE_IMEXRK) {
    if (butcher_tables(p, &s->sch) != 0) { orc_sim_destroy(s); return NULL; }
    int ns = s->sch.n_exp;
    s->dtemp_a = zalloc(cf * ns); s->dtemp_d = zalloc(cf * ns);
    s->domg_a = zalloc(cf * ns); s->domg_d = zalloc(cf * ns); s->rhs_buo = zalloc(cf * ns);
    s->AT_all = zalloc((size_t)R * R * M); s->AF_all = zalloc((size_t)4 * R * R * M);
    s->A_uphi = zalloc((size_t)R * R);
    s->ipiv1 = (int*)calloc((size_t)R * M, sizeof(int));
    s->ipiv2 = (int*)calloc((size_t)2 * R * M, sizeof(int));
    s->ipiv_uphi = (int*)calloc((size_t)R, sizeof(int));
    const int di = s->sch.diag_index;
    for (int st = 1; st < ns && s->sch.diag_diff; ++st) {
      if (s->sch.aD[st][st] == s->sch.aD[di][di]) continue;
      s->AT_st[st] = zalloc((size_t)R * R * M); s->AF_st[st] = zalloc((size_t)4 * R * R * M);
      s->Au_st[st] = zalloc((size_t)R * R);
      s->p1_st[st] = (int*)calloc((size_t)R * M, sizeof(int));
      s->p2_st[st] = (int*)calloc((size_t)2 * R * M, sizeof(int));
      s->pu_st[st] = (int*)calloc((size_t)R, sizeof(int));
    }
  } else if (p->scheme_type == ORC_TYPE_RK) {
    /* butcher_a / butcher_b of RK2 (midpoint) and RK4 (classical),
     * src/timeschemes.F90:1701-1720 */
    memset(&s->sch, 0, sizeof(s->sch));
    if (p->scheme_exp == ORC_EXP_RK2) {
      s->sch.n_exp = 2;
      s->sch.aA[1][0] = 0.5;
      s->sch.bA[0] = 0.0; s->sch.bA[1] = 1.0;
    } else if (p->scheme_exp == ORC_EXP_RK4) {
      s->sch.n_exp = 4;
      s->sch.aA[1][0] = 0.5; s->sch.aA[1][2] = 0.5; /* a(2,3) is never read: stage 2 sums i < 2 */
      s->sch.aA[2][1] = 0.5;
      s->sch.aA[3][2] = 1.0;
      s->sch.bA[0] = 1.0 / 6.0; s->sch.bA[1] = 1.0 / 3.0; s->sch.bA[2] = 1.0 / 3.0; s->sch.bA[3] = 1.0 / 6.0;
    } else {
      orc_sim_destroy(s);
      return NULL;
    }
    s->sch.n_imp = s->sch.n_exp;
    int ns = s->sch.n_exp;
    s->dtemp_a = zalloc(cf * ns); s->dtemp_d = zalloc(cf * ns);
    s->domg_a = zalloc(cf * ns); s->domg_d = zalloc(cf * ns); s->rhs_buo = zalloc(cf * ns);
  } else {
    orc_sim_destroy(s);
    return NULL;
  }
  s->LAPpsi_all = zalloc((size_t)R * R * M);
  s->ipiv_lap = (int*)calloc((size_t)R * M, sizeof(int));
  /* Lagrange weights for the Johnston vorticity boundary values,
   * src/init.F90:267-272. */
  int lm = p->lagpts;
  if (lm > R - 2) lm = R - 2;
  s->p.lagpts = lm;
  s->dw_rmin = zalloc(lm); s->d2w_rmin = zalloc(lm); s->dw_rmax = zalloc(lm); s->d2w_rmax = zalloc(lm);
  s->dtval_r = zalloc(R); s->dtval_p = zalloc(R); s->dtval_rkr = zalloc(R); s->dtval_rkp = zalloc(R);
  {
    double* pts = zalloc(lm);
    for (int i = 0; i < lm; ++i) pts[i] = s->radius[1 + i];
    dlagrange(lm, pts, s->rmin, s->dw_rmin);
    d2lagrange(lm, pts, s->rmin, s->d2w_rmin);
    for (int i = 0; i < lm; ++i) pts[i] = s->radius[R - 2 - i];
    dlagrange(lm, pts, s->rmax, s->dw_rmax);
    d2lagrange(lm, pts, s->rmax, s->d2w_rmax);
    free(pts);
  }
  return s;
}

void orc_sim_destroy(orc_sim* s) {
  if (!s) return;
  void* ptrs[] = {s->xp, s->t, s->D, s->D2, s->radius, s->r_radius, s->r_radius2, s->dr,
                  s->tFR, s->omgFR, s->upFR, s->urFR, s->psii, s->temp_spec, s->omg_spec,
                  s->upFC, s->upFR_prev, s->urFR_prev, s->uphi_bar_spec, s->TFC, s->tt, s->up,
                  s->ur, s->omg, s->uphi_temp_FR, s->ur_temp_FR, s->uphi_omg_FR, s->ur_omg_FR,
                  s->rhs_imp_temp, s->rhs_exp_temp, s->rhs_imp_vort, s->rhs_exp_vort,
                  s->rhs_buo_term, s->tmp_imp_temp, s->tmp_exp_temp, s->tmp_imp_vort,
                  s->tmp_exp_vort, s->tmp_buo_term, s->rhs_imp_uphi, s->rhs_exp_uphi,
                  s->tmp_imp_uphi, s->tmp_exp_uphi, s->dtemp_a, s->dtemp_d, s->domg_a,
                  s->domg_d, s->rhs_buo, s->AT_all, s->AF_all, s->A_uphi, s->ipiv1, s->ipiv2,
                  s->ipiv_uphi, s->LAPpsi_all, s->ipiv_lap, s->dw_rmin, s->d2w_rmin,
                  s->dw_rmax, s->d2w_rmax, s->dtval_r, s->dtval_p, s->dtval_rkr, s->dtval_rkp};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
  for (int st = 0; st < 8; ++st) {
    free(s->AT_st[st]); free(s->AF_st[st]); free(s->Au_st[st]);
    free(s->p1_st[st]); free(s->p2_st[st]); free(s->pu_st[st]);
  }
  free(s);
}

int orc_sim_nstep(const orc_sim* s) { return s->n_step; }
double orc_sim_dt(const orc_sim* s) { return s->dt_new; }

/* splitmix64 stream keyed by (seed, m, i) -> two standard normals (Box-Muller). */
static uint64_t splitmix64(uint64_t* x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
void orc_noise_pair(uint64_t seed, int m, int i, double* a, double* b) {
  uint64_t st = seed * 0xD1B54A32D192ED03ull ^ ((uint64_t)(unsigned)m << 32) ^ (uint64_t)(unsigned)i;
  splitmix64(&st);
  double u1 = ((double)(splitmix64(&st) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
  double u2 = (double)(splitmix64(&st) >> 11) * (1.0 / 9007199254740992.0);
  double rad = sqrt(-2.0 * log(u1));
  double ang = 2.0 * PI_ * u2;
  *a = rad * cos(ang);
  *b = rad * sin(ang);
}

/* Gaspari-Cohn compact profile pieces, src/init.F90:937-985 */
static double gasp_middle(double r, double c, double L) {
  const double pi = PI_;
  return pi / 3.0 * L * r * (r + 3.0 * L) * exp(-r / L) +
         (2.0 * pi * L * L * (c + L) * (c + L)) / r * exp(-2.0 * c / L) *
             (1.0 - (1.0 - r / (c + L)) * exp(r / L)) +
         pi * L * L * L * (exp(-r / L) - exp((r - 2.0 * c) / L));
}
static double gasp_edge(double r, double c, double L) {
  const double pi = PI_;
  return 2.0 * pi * L / r * exp(-r / L) *
         (0.5 * (r * (r + L) * (2.0 * c - r)) + 1.0 / 3.0 * ((r - c) * (r - c) * (r - c) - c * c * c) -
          L * (c + L) * (r - c + L) + L * (c + L) * (c + L) * exp((r - 2.0 * c) / L));
}
static double gasp_center(double c, double L) {
  const double pi = PI_;
  return pi * L * L * L * (1.0 - exp(-2.0 * c / L)) - 2.0 * pi * c * L * (c + L) * exp(-2.0 * c / L);
}

static void reset_after_state(orc_sim* s) {
  int M = s->M, R = s->R;
  size_t cf = 2 * (size_t)M * R;
  s->n_step = 0; s->tot_time = 0.0; s->mats_built = 0; s->restarted = 0;
  for (int i = 0; i < 4; ++i) s->dt_array[i] = s->p.dt;
  /* temp_spec = tFR, omg_spec = omgFR, upFC = upFR (src/init.F90:393-395) */
  memcpy(s->temp_spec, s->tFR, cf * sizeof(double));
  memcpy(s->omg_spec, s->omgFR, cf * sizeof(double));
  memcpy(s->upFC, s->upFR, cf * sizeof(double));
  memcpy(s->upFR_prev, s->upFR, cf * sizeof(double));
  memcpy(s->urFR_prev, s->upFR, cf * sizeof(double));
  for (int r = 0; r < R; ++r) {
    s->uphi_bar_spec[2 * r] = s->upFR[2 * (size_t)M * r];
    s->uphi_bar_spec[2 * r + 1] = s->upFR[2 * (size_t)M * r + 1];
  }
  memset(s->uphi_temp_FR, 0, cf * sizeof(double));
  memset(s->ur_temp_FR, 0, cf * sizeof(double));
  memset(s->uphi_omg_FR, 0, cf * sizeof(double));
  memset(s->ur_omg_FR, 0, cf * sizeof(double));
  /* physical grids as left by the initialisation */
  for (int r = 0; r < R; ++r) {
    orc_invfft(s->Nm, s->P, CX(s->tFR, 0, r), s->tt + (size_t)s->P * r);
    orc_invfft(s->Nm, s->P, CX(s->omgFR, 0, r), s->omg + (size_t)s->P * r);
    orc_invfft(s->Nm, s->P, CX(s->upFR, 0, r), s->up + (size_t)s->P * r);
    orc_invfft(s->Nm, s->P, CX(s->urFR, 0, r), s->ur + (size_t)s->P * r);
  }
  if (s->rhs_imp_temp) {
    int ni = s->sch.n_imp, ne = s->sch.n_exp;
    memset(s->rhs_imp_temp, 0, cf * ni * sizeof(double)); memset(s->tmp_imp_temp, 0, cf * ni * sizeof(double));
    memset(s->rhs_imp_vort, 0, cf * ni * sizeof(double)); memset(s->tmp_imp_vort, 0, cf * ni * sizeof(double));
    memset(s->rhs_buo_term, 0, cf * ni * sizeof(double)); memset(s->tmp_buo_term, 0, cf * ni * sizeof(double));
    memset(s->rhs_exp_temp, 0, cf * ne * sizeof(double)); memset(s->tmp_exp_temp, 0, cf * ne * sizeof(double));
    memset(s->rhs_exp_vort, 0, cf * ne * sizeof(double)); memset(s->tmp_exp_vort, 0, cf * ne * sizeof(double));
    memset(s->rhs_imp_uphi, 0, 2 * (size_t)R * ni * sizeof(double));
    memset(s->rhs_exp_uphi, 0, 2 * (size_t)R * ne * sizeof(double));
  }
  if (s->dtemp_a) {
    int ns = s->sch.n_exp;
    memset(s->dtemp_a, 0, cf * ns * sizeof(double)); memset(s->dtemp_d, 0, cf * ns * sizeof(double));
    memset(s->domg_a, 0, cf * ns * sizeof(double)); memset(s->domg_d, 0, cf * ns * sizeof(double));
    memset(s->rhs_buo, 0, cf * ns * sizeof(double));
  }
}

/* init_fields + init_perturbation (src/init.F90:164-399) for kind 0; the
 * seeded-noise initial state for kind 1. */
int orc_sim_init(orc_sim* s, int kind, int n_init, double amp, uint64_t seed) {
  int R = s->R, M = s->M, P = s->P, Nm = s->Nm;
  size_t cf = 2 * (size_t)M * R;
  memset(s->tFR, 0, cf * sizeof(double)); memset(s->omgFR, 0, cf * sizeof(double));
  memset(s->upFR, 0, cf * sizeof(double)); memset(s->urFR, 0, cf * sizeof(double));
  memset(s->psii, 0, cf * sizeof(double));
  double lrr = log(s->rmin / s->rmax), lrmax = log(s->rmax);
  if (kind == 1) {
    for (int r = 0; r < R; ++r) {
      CX(s->tFR, 0, r)[0] = log(s->radius[r]) / lrr - lrmax / lrr; /* tcon, src/init.F90:209 */
      if (r == 0 || r == R - 1) continue;
      for (int m = 1; m <= Nm; ++m) {
        double a, b;
        orc_noise_pair(seed, m, r, &a, &b);
        CX(s->tFR, m, r)[0] = amp * a;
        CX(s->tFR, m, r)[1] = amp * b;
      }
    }
  } else {
    double* tt = zalloc((size_t)P);
    const double pi = PI_;
    double* gasp = zalloc(R);
    if (n_init == 0) {
      double sigma_r = 0.1 / sqrt(2.0), sigma_p = 0.2;
      double rc = 0.5 * (s->rmax + s->rmin);
      int ir = 0; double best = fabs(s->radius[0] - rc);
      for (int i = 1; i < R; ++i) if (fabs(s->radius[i] - rc) < best) { best = fabs(s->radius[i] - rc); ir = i; }
      rc = s->radius[ir];
      double c1 = 0.5 * (s->radius[R - 1] - rc), c2 = 0.5 * (rc - s->radius[0]), L = 0.5 * sigma_r;
      for (int i = 0; i < R; ++i) {
        double rr = s->radius[i];
        if (i == ir) gasp[i] = 1.0;
        else if (rr < rc - c2) gasp[i] = gasp_edge(rc - rr, c2, L);
        else if (rr >= rc - c2 && rr < rc) gasp[i] = gasp_middle(rc - rr, c2, L);
        else if (rr > rc && rr <= rc + c1) gasp[i] = gasp_middle(rr - rc, c1, L);
        else if (rr > rc + c1) gasp[i] = gasp_edge(rr - rc, c1, L);
      }
      for (int i = 0; i < R; ++i) {
        if (i < ir) gasp[i] = gasp[i] / gasp_center(c1, L);
        else if (i > ir) gasp[i] = gasp[i] / gasp_center(c2, L);
      }
      for (int r = 0; r < R; ++r) {
        double c_r = amp * gasp[r];
        double tcon = log(s->radius[r]) / lrr - lrmax / lrr;
        for (int j = 0; j < P; ++j) {
          double ph = (double)j * 2.0 * pi / (double)P;
          tt[j] = c_r * exp(-(ph - pi) * (ph - pi) / (sigma_p * sigma_p)) + tcon;
        }
        orc_forfft(Nm, P, tt, CX(s->tFR, 0, r));
      }
    } else {
      double* phi = zalloc(P);
      for (int j = 1; j < P; ++j) phi[j] = phi[j - 1] + 2.0 * pi / (double)P;
      for (int r = 0; r < R; ++r) {
        double tcon = log(s->radius[r]) / lrr - lrmax / lrr;
        double rad = s->radius[r];
        for (int j = 0; j < P; ++j) {
          if (n_init < 0) {
            double sp = 0.25, sr = 0.25, rmid = s->rmax - (s->rmax - s->rmin) / 2.0;
            if (phi[j] > 1.0 && phi[j] < 3.0)
              tt[j] = -1.0 * (s->rmax - rad) * (s->rmin - rad) * amp * (1.0 / (2.0 * pi * sp * sr)) *
                          exp(-1.0 * ((rad - rmid) * (rad - rmid) / (sr * sr) +
                                      (phi[j] - 2.0) * (phi[j] - 2.0) / (sp * sp))) + tcon;
            else
              tt[j] = tcon;
          } else {
            tt[j] = amp * (s->rmax - rad) * (s->rmin - rad) * cos((double)n_init * phi[j]) + tcon;
          }
        }
        orc_forfft(Nm, P, tt, CX(s->tFR, 0, r));
      }
      free(phi);
    }
    free(tt); free(gasp);
  }
  reset_after_state(s);
  return 0;
}

int orc_sim_set_state(orc_sim* s, const double* tFR, const double* omgFR, const double* upFR,
                      const double* urFR) {
  size_t cf = 2 * (size_t)s->M * s->R;
  memcpy(s->tFR, tFR, cf * sizeof(double)); memcpy(s->omgFR, omgFR, cf * sizeof(double));
  memcpy(s->upFR, upFR, cf * sizeof(double)); memcpy(s->urFR, urFR, cf * sizeof(double));
  memset(s->psii, 0, cf * sizeof(double));
  reset_after_state(s);
  return 0;
}

int orc_sim_get_state(const orc_sim* s, double* tFR, double* omgFR, double* upFR, double* urFR,
                      double* psi) {
  size_t cf = 2 * (size_t)s->M * s->R;
  if (tFR) memcpy(tFR, s->tFR, cf * sizeof(double));
  if (omgFR) memcpy(omgFR, s->omgFR, cf * sizeof(double));
  if (upFR) memcpy(upFR, s->upFR, cf * sizeof(double));
  if (urFR) memcpy(urFR, s->urFR, cf * sizeof(double));
  if (psi) memcpy(psi, s->psii, cf * sizeof(double));
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Operator assembly and LU: src/mat_assembly.F90                            */
/* ------------------------------------------------------------------------ */

/* mat_build (:242-359) when irk == 0; mat_build_IRK (:68-187) when irk == 1.
 * The two differ only in which boundary rows of AF carry psi=0 and the
 * second psi condition (:143-150 vs :316-323). */
static void assemble_at_af(orc_sim* s, double dt, int n, double wt, int irk, double* AT, double* AF) {
  int R = s->R, R2 = 2 * R;
  const double *t = s->t, *D = s->D, *D2 = s->D2, *rr = s->r_radius, *rr2 = s->r_radius2;
  double C = pow(2.0 / (double)(R - 1), 0.5);
  double nn = (double)n * (double)n;
  double* bcp2 = zalloc(2 * (size_t)R);
#define M2(a, i, j) a[(i) + R * (j)]
#define F2(a, i, j) a[(i) + R2 * (j)]
  for (int j = 0; j < R; ++j) {
    if (s->p.mbc == 0) {
      bcp2[2 * j] = M2(D, 0, j);
      bcp2[2 * j + 1] = M2(D, R - 1, j);
    } else {
      bcp2[2 * j] = M2(D2, 0, j) - rr[0] * M2(D, 0, j);
      bcp2[2 * j + 1] = M2(D2, R - 1, j) - rr[R - 1] * M2(D, R - 1, j);
    }
  }
  memset(AT, 0, sizeof(double) * R * R);
  memset(AF, 0, sizeof(double) * R2 * R2);
  for (int j = 0; j < R; ++j) {
    for (int i = 0; i < R; ++i)
      M2(AT, i, j) = M2(t, i, j) - wt * dt * (1.0 / s->p.pr) *
                                       (rr[i] * M2(D, i, j) + M2(D2, i, j) - nn * rr2[i] * M2(t, i, j));
    M2(AT, 0, j) = M2(t, 0, j);
    M2(AT, R - 1, j) = M2(t, R - 1, j);
  }
  for (int i = 0; i < R; ++i) { M2(AT, i, 0) *= 0.5; M2(AT, i, R - 1) *= 0.5; }
  for (int k = 0; k < R * R; ++k) AT[k] = C * AT[k];
  for (int j = 0; j < R; ++j) {
    for (int i = 0; i < R; ++i) {
      F2(AF, i, j) = rr[i] * M2(D, i, j) + M2(D2, i, j) - nn * rr2[i] * M2(t, i, j);
      F2(AF, i, R + j) = M2(t, i, j);
      F2(AF, R + i, j) = 0.0;
      F2(AF, R + i, R + j) = M2(t, i, j) - wt * dt * (rr[i] * M2(D, i, j) + M2(D2, i, j) - nn * rr2[i] * M2(t, i, j));
    }
    if (irk) {
      F2(AF, 0, j) = bcp2[2 * j]; F2(AF, R - 1, j) = bcp2[2 * j + 1];
    } else {
      F2(AF, 0, j) = M2(t, 0, j); F2(AF, R - 1, j) = M2(t, R - 1, j);
    }
    F2(AF, 0, R + j) = 0.0; F2(AF, R - 1, R + j) = 0.0;
    if (irk) {
      F2(AF, R, j) = M2(t, 0, j); F2(AF, R2 - 1, j) = M2(t, R - 1, j);
    } else {
      F2(AF, R, j) = bcp2[2 * j]; F2(AF, R2 - 1, j) = bcp2[2 * j + 1];
    }
    F2(AF, R, R + j) = 0.0; F2(AF, R2 - 1, R + j) = 0.0;
  }
  for (int i = 0; i < R; ++i) {
    F2(AF, i, 0) *= 0.5; F2(AF, i, R - 1) *= 0.5;
    F2(AF, i, R) *= 0.5; F2(AF, i, R2 - 1) *= 0.5;
    F2(AF, R + i, 0) *= 0.5; F2(AF, R + i, R - 1) *= 0.5;
    F2(AF, R + i, R) *= 0.5; F2(AF, R + i, R2 - 1) *= 0.5;
  }
  for (int k = 0; k < R2 * R2; ++k) AF[k] = C * AF[k];
#undef F2
  free(bcp2);
}

static void mat_build(orc_sim* s, double dt, int n, double wt, int irk, double* AT, int* piv1,
                      double* AF, int* piv2) {
  assemble_at_af(s, dt, n, wt, irk, AT, AF);
  orc_dgetrf(s->R, AT, piv1);
  orc_dgetrf(2 * s->R, AF, piv2);
}

/* mat_build_uphibar (:361-413) / mat_build_uphibar_IRK (:189-240). */
static void assemble_uphibar(orc_sim* s, double dt, double wt, double* A) {
  int R = s->R;
  const double *t = s->t, *D = s->D, *D2 = s->D2, *rr = s->r_radius, *rr2 = s->r_radius2;
  double C = pow(2.0 / (double)(R - 1), 0.5);
  for (int j = 0; j < R; ++j) {
    for (int i = 0; i < R; ++i)
      M2(A, i, j) = M2(t, i, j) - wt * dt * (rr[i] * M2(D, i, j) + M2(D2, i, j) - rr2[i] * M2(t, i, j));
    if (s->p.mbc == 0) {
      M2(A, 0, j) = M2(t, 0, j); M2(A, R - 1, j) = M2(t, R - 1, j);
    } else {
      M2(A, 0, j) = M2(D, 0, j) - rr[0] * M2(t, 0, j);
      M2(A, R - 1, j) = M2(D, R - 1, j) - rr[R - 1] * M2(t, R - 1, j);
    }
  }
  for (int i = 0; i < R; ++i) { M2(A, i, 0) *= 0.5; M2(A, i, R - 1) *= 0.5; }
  for (int k = 0; k < R * R; ++k) A[k] = C * A[k];
}

static void mat_build_uphibar(orc_sim* s, double dt, double wt, double* A, int* piv) {
  assemble_uphibar(s, dt, wt, A);
  orc_dgetrf(s->R, A, piv);
}

/* mat_build_rk (:415-462): the psi Poisson operator with psi=0 rows. */
static void assemble_rk(orc_sim* s, int n, double* L) {
  int R = s->R;
  const double *t = s->t, *D = s->D, *D2 = s->D2, *rr = s->r_radius, *rr2 = s->r_radius2;
  double C = pow(2.0 / (double)(R - 1), 0.5);
  double nn = (double)n * (double)n;
  for (int j = 0; j < R; ++j) {
    for (int i = 0; i < R; ++i)
      M2(L, i, j) = rr[i] * M2(D, i, j) + M2(D2, i, j) - nn * rr2[i] * M2(t, i, j);
    M2(L, 0, j) = 1.0 * M2(t, 0, j);
    M2(L, R - 1, j) = 1.0 * M2(t, R - 1, j);
  }
  for (int i = 0; i < R; ++i) { M2(L, i, 0) *= 0.5; M2(L, i, R - 1) *= 0.5; }
  for (int k = 0; k < R * R; ++k) L[k] = 1.0 * C * L[k];
}

static void mat_build_rk(orc_sim* s, int n, double* L, int* piv) {
  assemble_rk(s, n, L);
  orc_dgetrf(s->R, L, piv);
}
#undef M2

int orc_mat_assemble(const orc_params* p, int kind, int n, double dt, double wt, int irk, double* out) {
  orc_sim* s = orc_sim_create(p);
  if (!s) return -1;
  switch (kind) {
    case 0:
    case 1: {
      const int R = s->R;
      double* AT = zalloc((size_t)R * R);
      double* AF = zalloc((size_t)4 * R * R);
      assemble_at_af(s, dt, n, wt, irk, AT, AF);
      memcpy(out, kind == 0 ? AT : AF, sizeof(double) * (kind == 0 ? (size_t)R * R : (size_t)4 * R * R));
      free(AT);
      free(AF);
      break;
    }
    case 2: assemble_uphibar(s, dt, wt, out); break;
    case 3: assemble_rk(s, n, out); break;
    default: orc_sim_destroy(s); return -1;
  }
  orc_sim_destroy(s);
  return 0;
}

/* matsolve (src/algebra_lapack.F90:26-38): two dgetrs on the re/im parts. */
static void matsolve_cplx(int n, const double* A, const int* piv, double* x /*complex n*/,
                          double* work) {
  double* re = work;
  double* im = work + n;
  for (int i = 0; i < n; ++i) { re[i] = x[2 * i]; im[i] = x[2 * i + 1]; }
  orc_dgetrs(n, A, piv, re);
  orc_dgetrs(n, A, piv, im);
  for (int i = 0; i < n; ++i) { x[2 * i] = re[i]; x[2 * i + 1] = im[i]; }
}

/* ------------------------------------------------------------------------ */
/* Nonlinear pass on the handle: src/nonlin.F90:35-91 (grids kept, as the   */
/* module arrays tt, omg, up, ur of the reference)                           */
/* ------------------------------------------------------------------------ */
static void nr_maxloop(orc_sim* s) {
  int M = s->M, R = s->R, P = s->P, Nm = s->Nm;
  double* work = zalloc(2 * (size_t)P);
  for (int r = 0; r < R; ++r)
    nonlin_line(Nm, P, CX(s->tFR, 0, r), CX(s->omgFR, 0, r), CX(s->upFR, 0, r), CX(s->urFR, 0, r),
                s->tt + (size_t)P * r, s->omg + (size_t)P * r, s->up + (size_t)P * r,
                s->ur + (size_t)P * r, CX(s->uphi_temp_FR, 0, r), CX(s->ur_temp_FR, 0, r),
                CX(s->uphi_omg_FR, 0, r), CX(s->ur_omg_FR, 0, r), work);
  free(work);
  /* get_dtvals (src/nonlin.F90:93-106): advective time scales per radius */
  for (int r = 0; r < R; ++r) {
    double mr = 0.0, mp = 0.0;
    for (int j = 0; j < P; ++j) {
      mr = fmax(mr, fabs(s->ur[j + (size_t)P * r]));
      mp = fmax(mp, fabs(s->up[j + (size_t)P * r]));
    }
    s->dtval_r[r] = s->dr[r] / mr;
    s->dtval_p[r] = (2.0 / 3.0) * (s->radius[r] * PI_) / ((double)Nm * mp);
    s->dtval_rkr[r] = s->dr[r] * s->dr[r];
    s->dtval_rkp[r] = (2.0 / 3.0) * (s->radius[r] * PI_) / (double)Nm * (2.0 / 3.0) * (s->radius[r] * PI_) / (double)Nm;
  }
}

/* gather / scatter one mode's radial vector */
static void get_mode(const orc_sim* s, const double* a, int m, double* v) {
  int M = s->M;
  for (int r = 0; r < s->R; ++r) { v[2 * r] = CX(a, m, r)[0]; v[2 * r + 1] = CX(a, m, r)[1]; }
}
static void put_mode(const orc_sim* s, double* a, int m, const double* v) {
  int M = s->M;
  for (int r = 0; r < s->R; ++r) { CX(a, m, r)[0] = v[2 * r]; CX(a, m, r)[1] = v[2 * r + 1]; }
}

/* complex helpers */
static inline void cmul(double ar, double ai, double br, double bi, double* cr, double* ci) {
  *cr = ar * br - ai * bi; *ci = ar * bi + ai * br;
}

/* Physical-space mean of ur*omg over the azimuthal grid (src/rhs_create.F90:329-335). */
static void mean_ur_omg(const orc_sim* s, double* out) {
  int P = s->P;
  for (int r = 0; r < s->R; ++r) {
    double acc = 0.0;
    for (int j = 0; j < P; ++j) acc = acc + s->ur[j + (size_t)P * r] * s->omg[j + (size_t)P * r];
    out[r] = acc * (1.0 / (double)P);
  }
}

/* ------------------------------------------------------------------------ */
/* IMEX multistep step: src/steptime.F90:196-251 with Nm_maxLOOP             */
/* (src/fourierloop.F90:156-346) and rhs_construct_* (src/rhs_create.F90)   */
/* ------------------------------------------------------------------------ */
static double* hist(double* a, int nord, int i, int M, int m, int r) {
  return a + 2 * ((size_t)i + (size_t)nord * ((size_t)m + (size_t)M * r));
}

/* history shift of src/rhs_create.F90:54-70 (one mode, one field) */
static void shift_hist(orc_sim* s, double* rhs, const double* tmp, int nord, int m) {
  int M = s->M;
  for (int io = 0; io < nord - 1; ++io)
    for (int r = 0; r < s->R; ++r) {
      double* d = hist(rhs, nord, io + 1, M, m, r);
      const double* q = hist((double*)tmp, nord, io, M, m, r);
      d[0] = q[0]; d[1] = q[1];
    }
}

/* n_step-n_restart>1 .or. l_restart .and. (.not. l_imexrk_started) */
static int shift_condition(const orc_sim* s, int n_step) {
  return (n_step > 1) || (s->restarted && !s->p.l_imexrk_started);
}

/* rhs_construct_temp, src/rhs_create.F90:24-140 */
static void rhs_construct_temp(orc_sim* s, int n_step, int m, double dt, double* rhs, double* wk) {
  int R = s->R, M = s->M, ni = s->sch.n_imp, ne = s->sch.n_exp;
  const double* rr = s->r_radius; const double* rr2 = s->r_radius2;
  if (n_step > 1 && s->p.l_imexrk_started) {
    shift_hist(s, s->rhs_exp_temp, s->tmp_exp_temp, ne, m);
    shift_hist(s, s->rhs_imp_temp, s->tmp_imp_temp, ni, m);
  }
  if (shift_condition(s, n_step)) {
    shift_hist(s, s->rhs_exp_temp, s->tmp_exp_temp, ne, m);
    shift_hist(s, s->rhs_imp_temp, s->tmp_imp_temp, ni, m);
  }
  double* uphi_t = wk; double* ur_t = wk + 2 * R; double* ur_t_spec = wk + 4 * R;
  double* Tr = wk + 6 * R; double* dT = wk + 8 * R; double* d2T = wk + 10 * R;
  double* dur = wk + 12 * R; double* tspec = wk + 14 * R;
  get_mode(s, s->uphi_temp_FR, m, uphi_t);
  get_mode(s, s->ur_temp_FR, m, ur_t);
  get_mode(s, s->temp_spec, m, tspec);
  for (int i = 0; i < 2 * R; ++i) rhs[i] = 0.0;
  orc_chebtransform(R, ur_t, ur_t_spec);
  orc_chebinvtran(R, tspec, Tr);
  orc_chebinvtranD1D2(R, tspec, dT, d2T);
  orc_chebinvtranD1(R, ur_t_spec, dur);
  double dm = (double)m, mm = (double)m * (double)m;
  for (int i = 0; i < R; ++i) {
    double* imp1 = hist(s->rhs_imp_temp, ni, 0, M, m, i);
    double* exp1 = hist(s->rhs_exp_temp, ne, 0, M, m, i);
    imp1[0] = Tr[2 * i]; imp1[1] = Tr[2 * i + 1];
    if (s->p.scheme_imp == ORC_IMP_CN) {
      double c = (1.0 - s->sch.w_imp[0]) * dt * (1.0 / s->p.pr);
      rhs[2 * i] = imp1[0] + c * (rr[i] * dT[2 * i] + d2T[2 * i] - mm * rr2[i] * Tr[2 * i]);
      rhs[2 * i + 1] = imp1[1] + c * (rr[i] * dT[2 * i + 1] + d2T[2 * i + 1] - mm * rr2[i] * Tr[2 * i + 1]);
    } else {
      for (int io = 0; io < ni; ++io) {
        double* h = hist(s->rhs_imp_temp, ni, io, M, m, i);
        rhs[2 * i] = rhs[2 * i] + s->sch.w_imp[io] * h[0];
        rhs[2 * i + 1] = rhs[2 * i + 1] + s->sch.w_imp[io] * h[1];
      }
    }
    /* i*m*r^-1*uphi_T + d(ur_T)/dr + r^-1*ur_T */
    double ar, ai;
    cmul(0.0, dm * rr[i], uphi_t[2 * i], uphi_t[2 * i + 1], &ar, &ai);
    exp1[0] = ar + dur[2 * i] + rr[i] * ur_t[2 * i];
    exp1[1] = ai + dur[2 * i + 1] + rr[i] * ur_t[2 * i + 1];
    for (int io = 0; io < ne; ++io) {
      double* h = hist(s->rhs_exp_temp, ne, io, M, m, i);
      rhs[2 * i] = rhs[2 * i] - dt * (s->sch.w_exp[io] * h[0]);
      rhs[2 * i + 1] = rhs[2 * i + 1] - dt * (s->sch.w_exp[io] * h[1]);
    }
  }
  rhs[0] = (m == 0) ? 1.0 : 0.0; rhs[1] = 0.0;
  rhs[2 * (R - 1)] = 0.0; rhs[2 * (R - 1) + 1] = 0.0;
}

/* rhs_construct_vort, src/rhs_create.F90:142-271; rhsf has 2R complex. */
static void rhs_construct_vort(orc_sim* s, int n_step, int m, double dt, const double* tFRp,
                               double* rhsf, double* wk) {
  int R = s->R, M = s->M, ni = s->sch.n_imp, ne = s->sch.n_exp;
  const double* rr = s->r_radius; const double* rr2 = s->r_radius2;
  if (n_step > 1 && s->p.l_imexrk_started) {
    shift_hist(s, s->rhs_exp_vort, s->tmp_exp_vort, ne, m);
    shift_hist(s, s->rhs_imp_vort, s->tmp_imp_vort, ni, m);
  }
  if (shift_condition(s, n_step)) {
    shift_hist(s, s->rhs_exp_vort, s->tmp_exp_vort, ne, m);
    shift_hist(s, s->rhs_imp_vort, s->tmp_imp_vort, ni, m);
  }
  double* uphi_o = wk; double* ur_o = wk + 2 * R; double* ur_o_spec = wk + 4 * R;
  double* Or = wk + 6 * R; double* dO = wk + 8 * R; double* d2O = wk + 10 * R;
  double* dur = wk + 12 * R; double* ospec = wk + 14 * R; double* rhs2 = wk + 16 * R;
  get_mode(s, s->uphi_omg_FR, m, uphi_o);
  get_mode(s, s->ur_omg_FR, m, ur_o);
  get_mode(s, s->omg_spec, m, ospec);
  for (int i = 0; i < 2 * R; ++i) rhs2[i] = 0.0;
  orc_chebtransform(R, ur_o, ur_o_spec);
  orc_chebinvtran(R, ospec, Or);
  orc_chebinvtranD1D2(R, ospec, dO, d2O);
  orc_chebinvtranD1(R, ur_o_spec, dur);
  double dm = (double)m, mm = (double)m * (double)m, rp = s->p.ra / s->p.pr;
  for (int i = 0; i < R; ++i) {
    double* imp1 = hist(s->rhs_imp_vort, ni, 0, M, m, i);
    double* exp1 = hist(s->rhs_exp_vort, ne, 0, M, m, i);
    double ar, ai;
    if (s->p.scheme_imp == ORC_IMP_CN) {
      imp1[0] = Or[2 * i]; imp1[1] = Or[2 * i + 1];
      double c = (1.0 - s->sch.w_imp[0]) * dt;
      double* told = hist(s->rhs_imp_temp, ni, 0, M, m, i);
      double b1r, b1i, b2r, b2i;
      cmul(0.0, dm * rr[i], tFRp[2 * i], tFRp[2 * i + 1], &b1r, &b1i);
      cmul(0.0, dm * rr[i], told[0], told[1], &b2r, &b2i);
      rhs2[2 * i] = imp1[0] + c * (rr[i] * dO[2 * i] + d2O[2 * i] - mm * rr2[i] * Or[2 * i]) -
                    rp * dt * 0.5 * (b1r + b2r);
      rhs2[2 * i + 1] = imp1[1] + c * (rr[i] * dO[2 * i + 1] + d2O[2 * i + 1] - mm * rr2[i] * Or[2 * i + 1]) -
                        rp * dt * 0.5 * (b1i + b2i);
      cmul(0.0, dm * rr[i], uphi_o[2 * i], uphi_o[2 * i + 1], &ar, &ai);
      exp1[0] = ar + dur[2 * i] + rr[i] * ur_o[2 * i];
      exp1[1] = ai + dur[2 * i + 1] + rr[i] * ur_o[2 * i + 1];
      for (int io = 0; io < ne; ++io) {
        double* h = hist(s->rhs_exp_vort, ne, io, M, m, i);
        rhs2[2 * i] = rhs2[2 * i] - dt * (s->sch.w_exp[io] * h[0]);
        rhs2[2 * i + 1] = rhs2[2 * i + 1] - dt * (s->sch.w_exp[io] * h[1]);
      }
    } else {
      imp1[0] = Or[2 * i]; imp1[1] = Or[2 * i + 1];
      for (int io = 0; io < ni; ++io) {
        double* h = hist(s->rhs_imp_vort, ni, io, M, m, i);
        rhs2[2 * i] = rhs2[2 * i] + s->sch.w_imp[io] * h[0];
        rhs2[2 * i + 1] = rhs2[2 * i + 1] + s->sch.w_imp[io] * h[1];
      }
      double* buo = hist(s->rhs_buo_term, ni, 0, M, m, i);
      double br, bi;
      cmul(0.0, dm * rr[i], tFRp[2 * i], tFRp[2 * i + 1], &br, &bi);
      buo[0] = -rp * br; buo[1] = -rp * bi;
      cmul(0.0, dm * rr[i], uphi_o[2 * i], uphi_o[2 * i + 1], &ar, &ai);
      exp1[0] = ar + dur[2 * i] + rr[i] * ur_o[2 * i];
      exp1[1] = ai + dur[2 * i + 1] + rr[i] * ur_o[2 * i + 1];
      for (int io = 0; io < ne; ++io) {
        double* h = hist(s->rhs_exp_vort, ne, io, M, m, i);
        rhs2[2 * i] = rhs2[2 * i] - dt * (s->sch.w_exp[io] * h[0]);
        rhs2[2 * i + 1] = rhs2[2 * i + 1] - dt * (s->sch.w_exp[io] * h[1]);
      }
      rhs2[2 * i] = rhs2[2 * i] + dt * s->sch.wt_lhs * buo[0];
      rhs2[2 * i + 1] = rhs2[2 * i + 1] + dt * s->sch.wt_lhs * buo[1];
    }
  }
  rhs2[0] = 0.0; rhs2[1] = 0.0; rhs2[2 * (R - 1)] = 0.0; rhs2[2 * (R - 1) + 1] = 0.0;
  for (int i = 0; i < R; ++i) {
    rhsf[2 * i] = 0.0; rhsf[2 * i + 1] = 0.0;
    rhsf[2 * (i + R)] = rhs2[2 * i]; rhsf[2 * (i + R) + 1] = rhs2[2 * i + 1];
  }
}

/* rhs_construct_uphi_bar, src/rhs_create.F90:273-385 (only the m=0 row of the
 * derivatives is used by the reference; the others are not computed here). */
static void rhs_construct_uphi_bar(orc_sim* s, int n_step, double dt, double* rhs_uphi, double* wk) {
  int R = s->R, M = s->M, ni = s->sch.n_imp, ne = s->sch.n_exp;
  const double* rr = s->r_radius; const double* rr2 = s->r_radius2;
  if (n_step > 1 && s->p.l_imexrk_started) {
    for (int io = 0; io < ne - 1; ++io)
      memcpy(s->rhs_exp_uphi + 2 * (size_t)R * (io + 1), s->tmp_exp_uphi + 2 * (size_t)R * io, 2 * R * sizeof(double));
    for (int io = 0; io < ni - 1; ++io)
      memcpy(s->rhs_imp_uphi + 2 * (size_t)R * (io + 1), s->tmp_imp_uphi + 2 * (size_t)R * io, 2 * R * sizeof(double));
  }
  if (shift_condition(s, n_step)) {
    for (int io = 0; io < ne - 1; ++io)
      memcpy(s->rhs_exp_uphi + 2 * (size_t)R * (io + 1), s->tmp_exp_uphi + 2 * (size_t)R * io, 2 * R * sizeof(double));
    for (int io = 0; io < ni - 1; ++io)
      memcpy(s->rhs_imp_uphi + 2 * (size_t)R * (io + 1), s->tmp_imp_uphi + 2 * (size_t)R * io, 2 * R * sizeof(double));
  }
  double* upc = wk; double* d1 = wk + 2 * R; double* d2 = wk + 4 * R; double* urom = wk + 6 * R;
  get_mode(s, s->upFC, 0, upc);
  orc_chebinvtranD1(R, upc, d1);
  orc_chebinvtranD2(R, upc, d2);
  mean_ur_omg(s, urom);
  for (int i = 0; i < R; ++i) rhs_uphi[i] = 0.0;
  for (int i = 0; i < R; ++i) {
    const double* up0 = CX(s->upFR, 0, i);
    double udiff = d2[2 * i] - rr2[i] * up0[0] + rr[i] * d1[2 * i];
    double* imp1 = s->rhs_imp_uphi + 2 * (size_t)i;           /* order index 0 */
    (void)imp1;
    s->rhs_imp_uphi[2 * i] = up0[0]; s->rhs_imp_uphi[2 * i + 1] = up0[1];
    if (s->p.scheme_imp == ORC_IMP_CN) {
      rhs_uphi[i] = s->rhs_imp_uphi[2 * i] + (1.0 - s->sch.w_imp[0]) * dt * udiff;
    } else {
      for (int io = 0; io < ni; ++io)
        rhs_uphi[i] = rhs_uphi[i] + s->sch.w_imp[io] * s->rhs_imp_uphi[2 * ((size_t)R * io + i)];
    }
    s->rhs_exp_uphi[2 * i] = urom[i]; s->rhs_exp_uphi[2 * i + 1] = 0.0;
    for (int io = 0; io < ne; ++io)
      rhs_uphi[i] = rhs_uphi[i] - dt * (s->sch.w_exp[io] * s->rhs_exp_uphi[2 * ((size_t)R * io + i)]);
  }
  rhs_uphi[0] = 0.0; rhs_uphi[R - 1] = 0.0;
}

/* compute_new_dt of the multistep loop (src/steptime.F90:313-370), called
 * from the second step on: the CFL time step from the last nonlinear pass,
 * optionally changed only when needed (l_optimizedt), and the dt_array
 * history shifted (n_order_tscheme_max = max(n_imp, n_exp)). */
static double minval(const double* v, int n) {
  double m = v[0];
  for (int i = 1; i < n; ++i) m = fmin(m, v[i]);
  return m;
}

/* compute_new_dt of the IMEXRK loop (src/steptime_imexrk.F90:248-308) and of
 * the RK loop (src/steptime_rk.F90:180-238): as the multistep one, but only
 * dt_array(2) is shifted; RK adds the diffusive scales to dt_cal and always
 * takes the "optimize" branch, after dt_array(:) was reset to dt. */
static void compute_new_dt_rk(orc_sim* s, int rk, int n_step) {
  const orc_params* p = &s->p;
  int R = s->R;
  double dt_cal = fmin(minval(s->dtval_r, R), minval(s->dtval_p, R));
  if (rk) dt_cal = fmin(dt_cal, fmin(minval(s->dtval_rkr, R), minval(s->dtval_rkp, R)));
  double dt_n;
  if (p->pr == 1.0 || p->pr > 1.0) dt_n = fmax(1.0 / p->pr, 1.0) * p->cfl * dt_cal;
  else dt_n = fmin(1.0 / p->pr, 1.0) * p->cfl * dt_cal;
  double dt2 = fmin(0.5 * (1.0 / p->dt_coef + 1.0) * dt_n, p->dt_max);
  if (rk || p->l_optimizedt) {
    if (n_step > 1) {
      if (s->dt_array[1] > p->dt_max) s->dt_new = p->dt_max;
      else if (s->dt_array[1] >= dt_cal) s->dt_new = dt2;
      else if (p->dt_coef * s->dt_array[1] < dt_cal && s->dt_array[1] < p->dt_max)
        s->dt_new = (s->dt_array[0] < dt2) ? dt2 : s->dt_array[0];
    }
  } else {
    s->dt_new = dt2;
  }
  if (n_step == 1) {  /* first step after a restart */
    s->dt_array[0] = s->dt_new;
    return;
  }
  s->dt_array[1] = s->dt_array[0];
  s->dt_array[0] = s->dt_new;
}

static void compute_new_dt_imex(orc_sim* s, int n_step) {
  const orc_params* p = &s->p;
  int R = s->R;
  double mr = s->dtval_r[0], mp = s->dtval_p[0];
  for (int r = 1; r < R; ++r) { mr = fmin(mr, s->dtval_r[r]); mp = fmin(mp, s->dtval_p[r]); }
  double dt_cal = fmin(mr, mp);
  double dt_n;
  if (p->pr == 1.0 || p->pr > 1.0) dt_n = fmax(1.0 / p->pr, 1.0) * p->cfl * dt_cal;
  else dt_n = fmin(1.0 / p->pr, 1.0) * p->cfl * dt_cal;
  double dt2 = fmin(0.5 * (1.0 / p->dt_coef + 1.0) * dt_n, p->dt_max);
  if (p->l_optimizedt) {
    /* dt_new keeps its previous value when no branch applies (all of them
     * need n_step > 1 + n_restart) */
    if (n_step > 1) {
      if (s->dt_array[1] > p->dt_max) s->dt_new = p->dt_max;
      else if (s->dt_array[1] >= dt_cal) s->dt_new = dt2;
      else if (p->dt_coef * s->dt_array[1] < dt_cal && s->dt_array[1] < p->dt_max)
        s->dt_new = (s->dt_array[0] < dt2) ? dt2 : s->dt_array[0];
    }
  } else {
    s->dt_new = dt2;
  }
  if (n_step == 1) {  /* first step after a restart: the restored history stays */
    s->dt_array[0] = s->dt_new;
    return;
  }
  int nmax = s->sch.n_imp > s->sch.n_exp ? s->sch.n_imp : s->sch.n_exp;
  for (int i = nmax - 1; i >= 1; --i) s->dt_array[i] = s->dt_array[i - 1];
  s->dt_array[0] = s->dt_new;
}

static void imex_step(orc_sim* s) {
  int R = s->R, M = s->M;
  int n_step = s->n_step + 1;
  size_t cf = 2 * (size_t)M * R;
  if (n_step == 1) s->dt_new = s->p.dt;
  if (n_step > 1 || s->restarted) {
    nr_maxloop(s);
    memcpy(s->upFR_prev, s->upFR, cf * sizeof(double));
    memcpy(s->urFR_prev, s->urFR, cf * sizeof(double));
  }
  if (s->p.l_vartimestep && (n_step > 1 || s->restarted)) {
    compute_new_dt_imex(s, n_step);
  } else {
    s->dt_new = s->p.dt;
    for (int i = 0; i < 4; ++i) s->dt_array[i] = s->p.dt;
  }
  if (n_step > 1) {
    int ni = s->sch.n_imp, ne = s->sch.n_exp;
    memcpy(s->tmp_imp_temp, s->rhs_imp_temp, cf * ni * sizeof(double));
    memcpy(s->tmp_exp_temp, s->rhs_exp_temp, cf * ne * sizeof(double));
    memcpy(s->tmp_imp_vort, s->rhs_imp_vort, cf * ni * sizeof(double));
    memcpy(s->tmp_exp_vort, s->rhs_exp_vort, cf * ne * sizeof(double));
    memcpy(s->tmp_buo_term, s->rhs_buo_term, cf * ni * sizeof(double));
    memcpy(s->tmp_imp_uphi, s->rhs_imp_uphi, 2 * (size_t)R * ni * sizeof(double));
    memcpy(s->tmp_exp_uphi, s->rhs_exp_uphi, 2 * (size_t)R * ne * sizeof(double));
  }
  /* Nm_maxLOOP */
  multistep_weights(&s->p, s->dt_array, &s->sch);
  if (n_step == 1) {
    double* v = zalloc(4 * (size_t)R);
    for (int m = 0; m < M; ++m) {
      get_mode(s, s->tFR, m, v); orc_chebtransform(R, v, v + 2 * R); put_mode(s, s->temp_spec, m, v + 2 * R);
      get_mode(s, s->omgFR, m, v); orc_chebtransform(R, v, v + 2 * R); put_mode(s, s->omg_spec, m, v + 2 * R);
      get_mode(s, s->upFR, m, v); orc_chebtransform(R, v, v + 2 * R); put_mode(s, s->upFC, m, v + 2 * R);
    }
    free(v);
  }
  if (n_step == 1 || s->dt_array[0] != s->dt_array[1] || !s->mats_built) {
    for (int m = 0; m < M; ++m) {
      mat_build(s, s->dt_array[0], m, s->sch.wt_lhs, 0, s->AT_all + (size_t)R * R * m, s->ipiv1 + (size_t)R * m,
                s->AF_all + (size_t)4 * R * R * m, s->ipiv2 + (size_t)2 * R * m);
      mat_build_uphibar(s, s->dt_array[0], s->sch.wt_lhs, s->A_uphi, s->ipiv_uphi);
    }
    s->mats_built = 1;
  }
  double dt = s->dt_new;
  const double* rr = s->r_radius;
#pragma omp parallel
  {
    double* wk = zalloc(40 * (size_t)R);
    double* rhs = zalloc(4 * (size_t)R);
    double* tmp = zalloc(4 * (size_t)R);
    double* solw = zalloc(4 * (size_t)R);
#pragma omp for schedule(static)
    for (int m = 0; m < M; ++m) {
      rhs_construct_temp(s, n_step, m, dt, rhs, wk);
      matsolve_cplx(R, s->AT_all + (size_t)R * R * m, s->ipiv1 + (size_t)R * m, rhs, solw);
      if (m == 0) memcpy(s->TFC, rhs, 2 * R * sizeof(double));
      orc_chebinvtran(R, rhs, tmp);
      put_mode(s, s->temp_spec, m, rhs);
      put_mode(s, s->tFR, m, tmp);
      if (m == 0) {
        double* ru = zalloc(R);
        rhs_construct_uphi_bar(s, n_step, dt, ru, wk);
        orc_dgetrs(R, s->A_uphi, s->ipiv_uphi, ru);
        double* c = zalloc(6 * (size_t)R);
        for (int i = 0; i < R; ++i) { c[2 * i] = ru[i]; c[2 * i + 1] = 0.0; }
        put_mode(s, s->upFC, 0, c);
        orc_chebinvtran(R, c, c + 2 * R);
        put_mode(s, s->upFR, 0, c + 2 * R);
        orc_chebinvtranD1(R, c, c + 4 * R);
        for (int i = 0; i < R; ++i) {
          CX(s->urFR, 0, i)[0] = 0.0; CX(s->urFR, 0, i)[1] = 0.0;
          const double* u = CX(s->upFR, 0, i);
          CX(s->omgFR, 0, i)[0] = u[0] * rr[i] + c[4 * R + 2 * i];
          CX(s->omgFR, 0, i)[1] = u[1] * rr[i] + c[4 * R + 2 * i + 1];
        }
        free(c); free(ru);
      } else {
        double* rhsf = zalloc(4 * (size_t)R);
        double* sw = zalloc(8 * (size_t)R);
        rhs_construct_vort(s, n_step, m, dt, tmp, rhsf, wk);
        matsolve_cplx(2 * R, s->AF_all + (size_t)4 * R * R * m, s->ipiv2 + (size_t)2 * R * m, rhsf, sw);
        double* om = rhsf + 2 * R; double* ps = rhsf;
        put_mode(s, s->omg_spec, m, om);
        double* omr = sw; double* psr = sw + 2 * R; double* dps = sw + 4 * R;
        orc_chebinvtran(R, om, omr);
        put_mode(s, s->omgFR, m, omr);
        orc_chebinvtran(R, ps, psr);
        orc_chebinvtranD1(R, ps, dps);
        for (int i = 0; i < R; ++i) {
          CX(s->psii, m, i)[0] = psr[2 * i]; CX(s->psii, m, i)[1] = psr[2 * i + 1];
          CX(s->upFR, m, i)[0] = -1.0 * dps[2 * i]; CX(s->upFR, m, i)[1] = -1.0 * dps[2 * i + 1];
          double ar, ai;
          cmul(0.0, (double)m * rr[i], psr[2 * i], psr[2 * i + 1], &ar, &ai);
          CX(s->urFR, m, i)[0] = ar; CX(s->urFR, m, i)[1] = ai;
        }
        double* v = wk; double* vt = wk + 2 * R;
        get_mode(s, s->upFR, m, v);
        orc_chebtransform(R, v, vt);
        put_mode(s, s->upFC, m, vt);
        free(rhsf); free(sw);
      }
    }
    free(wk); free(rhs); free(tmp); free(solw);
  }
  s->tot_time = s->tot_time + s->dt_new;
  s->n_step = n_step;
}

/* ------------------------------------------------------------------------ */
/* IMEXRK: src/steptime_imexrk.F90:96-190, src/fourierloop_imexrk.F90,       */
/* src/rhs_create_imexrk.F90                                                 */
/* ------------------------------------------------------------------------ */
static double* stg(double* a, int ns, int st, int M, int m, int r) { return hist(a, ns, st, M, m, r); }

/* L_m applied in physical space through the Chebyshev coefficients, the way
 * rhs_construct_temp_d / _vort_d do it (src/rhs_create_imexrk.F90:70-102,
 * :268-300): r^-1 f' + f'' - m^2 r^-2 f. */
static void lap_phys(const orc_sim* s, int m, const double* f, double* out, double* wk) {
  int R = s->R;
  double* c = wk; double* d1 = wk + 2 * R; double* d2 = wk + 4 * R;
  orc_chebtransform(R, f, c);
  orc_chebinvtranD1D2(R, c, d1, d2);
  double mm = (double)m * (double)m;
  for (int i = 0; i < R; ++i)
    for (int q = 0; q < 2; ++q)
      out[2 * i + q] = s->r_radius[i] * d1[2 * i + q] + d2[2 * i + q] - mm * s->r_radius2[i] * f[2 * i + q];
}

/* -(i m r^-1 a + d(b)/dr + r^-1 b) (src/rhs_create_imexrk.F90:20-52, :209-245) */
static void advect_term(const orc_sim* s, int m, const double* a, const double* b, double* out,
                        double* wk) {
  int R = s->R;
  double* bs = wk; double* db = wk + 2 * R;
  orc_chebtransform(R, b, bs);
  orc_chebinvtranD1(R, bs, db);
  for (int i = 0; i < R; ++i) {
    double ar, ai;
    cmul(0.0, (double)m * s->r_radius[i], a[2 * i], a[2 * i + 1], &ar, &ai);
    out[2 * i] = -(ar + db[2 * i] + s->r_radius[i] * b[2 * i]);
    out[2 * i + 1] = -(ai + db[2 * i + 1] + s->r_radius[i] * b[2 * i + 1]);
  }
}

/* RHS_construct_stage, src/fourierloop_imexrk.F90:403-497 */
static void rhs_construct_stage(orc_sim* s, int st) {
  int R = s->R, M = s->M, ns = s->sch.n_exp;
  double* wk = zalloc(24 * (size_t)R);
  double* a = wk + 12 * R; double* b = wk + 14 * R; double* o = wk + 16 * R;
  double* urom = wk + 18 * R;
  double rp = s->p.ra / s->p.pr;
  for (int m = 0; m < M; ++m) {
    get_mode(s, s->uphi_temp_FR, m, a);
    get_mode(s, s->ur_temp_FR, m, b);
    advect_term(s, m, a, b, o, wk);
    for (int r = 0; r < R; ++r) { double* d = stg(s->dtemp_a, ns, st, M, m, r); d[0] = o[2 * r]; d[1] = o[2 * r + 1]; }
    get_mode(s, s->tFR, m, a);
    lap_phys(s, m, a, o, wk);
    for (int r = 0; r < R; ++r) {
      double* d = stg(s->dtemp_d, ns, st, M, m, r);
      d[0] = (1.0 / s->p.pr) * o[2 * r]; d[1] = (1.0 / s->p.pr) * o[2 * r + 1];
    }
    if (m == 0) {
      /* uphibar advective part: minus the physical mean of ur*omg (:158-170) */
      mean_ur_omg(s, urom);
      for (int r = 0; r < R; ++r) { double* d = stg(s->domg_a, ns, st, M, 0, r); d[0] = -urom[r]; d[1] = 0.0; }
      /* uphibar diffusive part (:174-203): real(u'' - u/r^2 + u'/r) */
      get_mode(s, s->upFR, 0, a);
      double* c = wk; double* d1 = wk + 2 * R; double* d2 = wk + 4 * R;
      orc_chebtransform(R, a, c);
      orc_chebinvtranD1D2(R, c, d1, d2);
      for (int r = 0; r < R; ++r) {
        double* d = stg(s->domg_d, ns, st, M, 0, r);
        d[0] = d2[2 * r] - s->r_radius2[r] * a[2 * r] + s->r_radius[r] * d1[2 * r];
        d[1] = 0.0;
      }
    } else {
      get_mode(s, s->uphi_omg_FR, m, a);
      get_mode(s, s->ur_omg_FR, m, b);
      advect_term(s, m, a, b, o, wk);
      for (int r = 0; r < R; ++r) { double* d = stg(s->domg_a, ns, st, M, m, r); d[0] = o[2 * r]; d[1] = o[2 * r + 1]; }
      get_mode(s, s->omgFR, m, a);
      lap_phys(s, m, a, o, wk);
      for (int r = 0; r < R; ++r) { double* d = stg(s->domg_d, ns, st, M, m, r); d[0] = o[2 * r]; d[1] = o[2 * r + 1]; }
      if (st == 0) {
        get_mode(s, s->tFR, m, a);
        for (int r = 0; r < R; ++r) {
          double br, bi;
          cmul(0.0, (double)m * s->r_radius[r], a[2 * r], a[2 * r + 1], &br, &bi);
          double* d = stg(s->rhs_buo, ns, 0, M, m, r);
          d[0] = -rp * br; d[1] = -rp * bi;
        }
      }
    }
  }
  free(wk);
}

/* Get_stage_var, src/fourierloop_imexrk.F90:75-401 */
static void get_stage_var(orc_sim* s, int st, int n_step) {
  int R = s->R, M = s->M, ns = s->sch.n_exp;
  /* matrices at stage 2 of the first step, and again whenever dt changed
   * (src/fourierloop_imexrk.F90:108-125).  With diag_diff (:134-160) the
   * reference rebuilds under the same conditions at every stage, each stage
   * whose diagonal differs from that of stage diag_index into a set of its
   * own; the values do not change within a step, so they are built here
   * together at stage 2. */
  if ((n_step == 1 && st == 1 && !s->mats_built) || (n_step > 1 && st == 1 && s->dt_array[0] != s->dt_array[1])) {
    double w = s->sch.aD[s->sch.diag_index][s->sch.diag_index];
    for (int m = 0; m < M; ++m) {
      mat_build(s, s->dt_array[0], m, w, 1, s->AT_all + (size_t)R * R * m, s->ipiv1 + (size_t)R * m,
                s->AF_all + (size_t)4 * R * R * m, s->ipiv2 + (size_t)2 * R * m);
      mat_build_uphibar(s, s->dt_array[0], w, s->A_uphi, s->ipiv_uphi);
    }
    for (int k = 1; k < ns; ++k) {
      if (!s->AT_st[k]) continue;
      double wk = s->sch.aD[k][k];
      for (int m = 0; m < M; ++m)
        mat_build(s, s->dt_array[0], m, wk, 1, s->AT_st[k] + (size_t)R * R * m, s->p1_st[k] + (size_t)R * m,
                  s->AF_st[k] + (size_t)4 * R * R * m, s->p2_st[k] + (size_t)2 * R * m);
      mat_build_uphibar(s, s->dt_array[0], wk, s->Au_st[k], s->pu_st[k]);
    }
    s->mats_built = 1;
  }
  const double* AT = s->AT_st[st] ? s->AT_st[st] : s->AT_all;
  const double* AF = s->AT_st[st] ? s->AF_st[st] : s->AF_all;
  const double* Au = s->AT_st[st] ? s->Au_st[st] : s->A_uphi;
  const int* p1 = s->AT_st[st] ? s->p1_st[st] : s->ipiv1;
  const int* p2 = s->AT_st[st] ? s->p2_st[st] : s->ipiv2;
  const int* pu = s->AT_st[st] ? s->pu_st[st] : s->ipiv_uphi;
  double dt = s->dt_array[0];
  double rp = s->p.ra / s->p.pr;
  const double* rr = s->r_radius;
#pragma omp parallel
  {
    double* v = zalloc(30 * (size_t)R);
    double* solw = zalloc(4 * (size_t)R);
#pragma omp for schedule(static)
    for (int m = 0; m < M; ++m) {
      double* Fd = v; double* Fa = v + 2 * R; double* rhs = v + 4 * R; double* tr = v + 6 * R;
      for (int i = 0; i < 4 * R; ++i) v[i] = 0.0;
      for (int r = 0; r < R; ++r)
        for (int i = 0; i < st; ++i) {
          double cd = s->sch.aD[st][i];
          const double* q = stg(s->dtemp_d, ns, i, M, m, r);
          Fd[2 * r] = Fd[2 * r] + cd * q[0]; Fd[2 * r + 1] = Fd[2 * r + 1] + cd * q[1];
        }
      for (int r = 0; r < R; ++r)
        for (int i = 0; i < st; ++i) {
          double ca = s->sch.aA[st][i];
          const double* q = stg(s->dtemp_a, ns, i, M, m, r);
          Fa[2 * r] = Fa[2 * r] + ca * q[0]; Fa[2 * r + 1] = Fa[2 * r + 1] + ca * q[1];
        }
      for (int r = 0; r < R; ++r) {
        const double* y0 = CX(s->temp_spec, m, r);
        rhs[2 * r] = y0[0] + dt * (Fd[2 * r] + Fa[2 * r]);
        rhs[2 * r + 1] = y0[1] + dt * (Fd[2 * r + 1] + Fa[2 * r + 1]);
      }
      rhs[0] = (m == 0) ? 1.0 : 0.0; rhs[1] = 0.0;
      rhs[2 * (R - 1)] = 0.0; rhs[2 * (R - 1) + 1] = 0.0;
      matsolve_cplx(R, AT + (size_t)R * R * m, p1 + (size_t)R * m, rhs, solw);
      orc_chebinvtran(R, rhs, tr);
      put_mode(s, s->tFR, m, tr);
      if (m == 0) {
        double* Fud = v + 8 * R; double* Fua = v + 10 * R; double* ru = v + 12 * R;
        for (int i = 0; i < 4 * R; ++i) Fud[i] = 0.0;
        for (int r = 0; r < R; ++r)
          for (int i = 0; i < st; ++i) {
            const double* q = stg(s->domg_d, ns, i, M, 0, r);
            Fud[2 * r] = Fud[2 * r] + s->sch.aD[st][i] * q[0];
            Fud[2 * r + 1] = Fud[2 * r + 1] + s->sch.aD[st][i] * q[1];
          }
        for (int r = 0; r < R; ++r)
          for (int i = 0; i < st; ++i) {
            const double* q = stg(s->domg_a, ns, i, M, 0, r);
            Fua[2 * r] = Fua[2 * r] + s->sch.aA[st][i] * q[0];
            Fua[2 * r + 1] = Fua[2 * r + 1] + s->sch.aA[st][i] * q[1];
          }
        for (int r = 0; r < R; ++r) ru[r] = s->uphi_bar_spec[2 * r] + dt * (Fud[2 * r] + Fua[2 * r]);
        ru[0] = 0.0; ru[R - 1] = 0.0;
        orc_dgetrs(R, Au, pu, ru);
        double* c = v + 14 * R; double* u = v + 16 * R; double* du = v + 18 * R;
        for (int r = 0; r < R; ++r) { c[2 * r] = ru[r]; c[2 * r + 1] = 0.0; }
        put_mode(s, s->upFC, 0, c);
        orc_chebinvtran(R, c, u);
        put_mode(s, s->upFR, 0, u);
        orc_chebinvtranD1(R, c, du);
        for (int r = 0; r < R; ++r) {
          CX(s->urFR, 0, r)[0] = 0.0; CX(s->urFR, 0, r)[1] = 0.0;
          CX(s->omgFR, 0, r)[0] = u[2 * r] * rr[r] + du[2 * r];
          CX(s->omgFR, 0, r)[1] = u[2 * r + 1] * rr[r] + du[2 * r + 1];
        }
      } else {
        for (int r = 0; r < R; ++r) {
          double br, bi;
          cmul(0.0, (double)m * rr[r], tr[2 * r], tr[2 * r + 1], &br, &bi);
          double* d = stg(s->rhs_buo, ns, st, M, m, r);
          d[0] = -rp * br; d[1] = -rp * bi;
        }
        double* Fod = v + 8 * R; double* Foa = v + 10 * R; double* Fb = v + 12 * R;
        for (int i = 0; i < 6 * R; ++i) Fod[i] = 0.0;
        for (int r = 0; r < R; ++r) {
          for (int i = 0; i < st; ++i) {
            const double* q = stg(s->domg_d, ns, i, M, m, r);
            Fod[2 * r] = Fod[2 * r] + s->sch.aD[st][i] * q[0];
            Fod[2 * r + 1] = Fod[2 * r + 1] + s->sch.aD[st][i] * q[1];
          }
          for (int i = 0; i < st; ++i) {
            const double* q = stg(s->domg_a, ns, i, M, m, r);
            Foa[2 * r] = Foa[2 * r] + s->sch.aA[st][i] * q[0];
            Foa[2 * r + 1] = Foa[2 * r + 1] + s->sch.aA[st][i] * q[1];
          }
          if (s->p.buo_imp) {
            for (int i = 0; i <= st; ++i) {
              const double* q = stg(s->rhs_buo, ns, i, M, m, r);
              Fb[2 * r] = Fb[2 * r] + s->sch.aD[st][i] * q[0];
              Fb[2 * r + 1] = Fb[2 * r + 1] + s->sch.aD[st][i] * q[1];
            }
          } else {
            for (int i = 0; i < st; ++i) {
              const double* q = stg(s->rhs_buo, ns, i, M, m, r);
              Fb[2 * r] = Fb[2 * r] + s->sch.aA[st][i] * q[0];
              Fb[2 * r + 1] = Fb[2 * r + 1] + s->sch.aA[st][i] * q[1];
            }
          }
        }
        double* rf = v + 14 * R; /* 2R complex */
        for (int r = 0; r < R; ++r) {
          const double* y0 = CX(s->omg_spec, m, r);
          rf[2 * r] = 0.0; rf[2 * r + 1] = 0.0;
          rf[2 * (R + r)] = y0[0] + dt * (Fod[2 * r] + Foa[2 * r] + Fb[2 * r]);
          rf[2 * (R + r) + 1] = y0[1] + dt * (Fod[2 * r + 1] + Foa[2 * r + 1] + Fb[2 * r + 1]);
        }
        rf[2 * R] = 0.0; rf[2 * R + 1] = 0.0; rf[2 * (2 * R - 1)] = 0.0; rf[2 * (2 * R - 1) + 1] = 0.0;
        double* sw = zalloc(4 * (size_t)R);
        matsolve_cplx(2 * R, AF + (size_t)4 * R * R * m, p2 + (size_t)2 * R * m, rf, sw);
        free(sw);
        double* omr = v + 18 * R; double* psr = v + 20 * R; double* dps = v + 22 * R; double* ut = v + 24 * R;
        orc_chebinvtran(R, rf + 2 * R, omr);
        put_mode(s, s->omgFR, m, omr);
        orc_chebinvtran(R, rf, psr);
        orc_chebinvtranD1(R, rf, dps);
        for (int r = 0; r < R; ++r) {
          CX(s->psii, m, r)[0] = psr[2 * r]; CX(s->psii, m, r)[1] = psr[2 * r + 1];
          CX(s->upFR, m, r)[0] = -1.0 * dps[2 * r]; CX(s->upFR, m, r)[1] = -1.0 * dps[2 * r + 1];
          double ar, ai;
          cmul(0.0, (double)m * rr[r], psr[2 * r], psr[2 * r + 1], &ar, &ai);
          CX(s->urFR, m, r)[0] = ar; CX(s->urFR, m, r)[1] = ai;
        }
        get_mode(s, s->upFR, m, ut);
        orc_chebtransform(R, ut, ut + 2 * R);
        put_mode(s, s->upFC, m, ut + 2 * R);
      }
    }
    free(v); free(solw);
  }
}

/* Assembly_stage (non stiffly accurate), src/fourierloop_imexrk.F90:499-651 */
static void assembly_stage(orc_sim* s) {
  int R = s->R, M = s->M, ns = s->sch.n_exp, lm = s->p.lagpts;
  double dt = s->dt_new;
  const double* rr = s->r_radius;
#pragma omp parallel
  {
    double* v = zalloc(24 * (size_t)R);
    double* solw = zalloc(4 * (size_t)R);
#pragma omp for schedule(static)
    for (int m = 0; m < M; ++m) {
      double* F = v;
      for (int i = 0; i < 2 * R; ++i) F[i] = 0.0;
      for (int r = 0; r < R; ++r)
        for (int i = 0; i < ns; ++i) {
          const double* qa = stg(s->dtemp_a, ns, i, M, m, r);
          const double* qd = stg(s->dtemp_d, ns, i, M, m, r);
          F[2 * r] = F[2 * r] + s->sch.bA[i] * qa[0] + s->sch.bD[i] * qd[0];
          F[2 * r + 1] = F[2 * r + 1] + s->sch.bA[i] * qa[1] + s->sch.bD[i] * qd[1];
        }
      for (int r = 0; r < R; ++r) {
        double* y = CX(s->temp_spec, m, r);
        y[0] = y[0] + dt * F[2 * r]; y[1] = y[1] + dt * F[2 * r + 1];
      }
      CX(s->temp_spec, m, 0)[0] = (m == 0) ? 1.0 : 0.0; CX(s->temp_spec, m, 0)[1] = 0.0;
      CX(s->temp_spec, m, R - 1)[0] = 0.0; CX(s->temp_spec, m, R - 1)[1] = 0.0;
      if (m == 0) {
        for (int i = 0; i < 2 * R; ++i) F[i] = 0.0;
        for (int r = 0; r < R; ++r)
          for (int i = 0; i < ns; ++i) {
            const double* qa = stg(s->domg_a, ns, i, M, 0, r);
            const double* qd = stg(s->domg_d, ns, i, M, 0, r);
            F[2 * r] = F[2 * r] + s->sch.bA[i] * qa[0] + s->sch.bD[i] * qd[0];
            F[2 * r + 1] = F[2 * r + 1] + s->sch.bA[i] * qa[1] + s->sch.bD[i] * qd[1];
          }
        for (int r = 0; r < R; ++r) {
          s->uphi_bar_spec[2 * r] = s->uphi_bar_spec[2 * r] + dt * F[2 * r];
          s->uphi_bar_spec[2 * r + 1] = s->uphi_bar_spec[2 * r + 1] + dt * F[2 * r + 1];
        }
        s->uphi_bar_spec[0] = 0.0; s->uphi_bar_spec[1] = 0.0;
        s->uphi_bar_spec[2 * (R - 1)] = 0.0; s->uphi_bar_spec[2 * (R - 1) + 1] = 0.0;
        put_mode(s, s->upFR, 0, s->uphi_bar_spec);
        double* c = v + 2 * R; double* du = v + 4 * R;
        orc_chebtransform(R, s->uphi_bar_spec, c);
        put_mode(s, s->upFC, 0, c);
        orc_chebinvtranD1(R, c, du);
        for (int r = 0; r < R; ++r) {
          CX(s->urFR, 0, r)[0] = 0.0; CX(s->urFR, 0, r)[1] = 0.0;
          CX(s->omg_spec, 0, r)[0] = s->uphi_bar_spec[2 * r] * rr[r] + du[2 * r];
          CX(s->omg_spec, 0, r)[1] = s->uphi_bar_spec[2 * r + 1] * rr[r] + du[2 * r + 1];
        }
      } else {
        for (int i = 0; i < 2 * R; ++i) F[i] = 0.0;
        for (int i = 0; i < ns; ++i)
          for (int r = 1; r < R - 1; ++r) {
            const double* qa = stg(s->domg_a, ns, i, M, m, r);
            const double* qd = stg(s->domg_d, ns, i, M, m, r);
            const double* qb = stg(s->rhs_buo, ns, i, M, m, r);
            F[2 * r] = F[2 * r] + s->sch.bA[i] * qa[0] + s->sch.bD[i] * qd[0] + s->sch.bD[i] * qb[0];
            F[2 * r + 1] = F[2 * r + 1] + s->sch.bA[i] * qa[1] + s->sch.bD[i] * qd[1] + s->sch.bD[i] * qb[1];
          }
        for (int r = 1; r < R - 1; ++r) {
          double* y = CX(s->omg_spec, m, r);
          y[0] = y[0] + dt * F[2 * r]; y[1] = y[1] + dt * F[2 * r + 1];
        }
        double* rhs = v + 2 * R;
        for (int r = 0; r < R; ++r) {
          rhs[2 * r] = -1.0 * CX(s->omg_spec, m, r)[0];
          rhs[2 * r + 1] = -1.0 * CX(s->omg_spec, m, r)[1];
        }
        rhs[0] = 0.0; rhs[1] = 0.0; rhs[2 * (R - 1)] = 0.0; rhs[2 * (R - 1) + 1] = 0.0;
        matsolve_cplx(R, s->LAPpsi_all + (size_t)R * R * m, s->ipiv_lap + (size_t)R * m, rhs, solw);
        double* psr = v + 4 * R; double* dps = v + 6 * R; double* d2ps = v + 8 * R; double* ut = v + 10 * R;
        orc_chebinvtran(R, rhs, psr);
        orc_chebinvtranD1(R, rhs, dps);
        orc_chebinvtranD2(R, rhs, d2ps);
        double d2min[2] = {0, 0}, dmin[2] = {0, 0}, d2max[2] = {0, 0}, dmax[2] = {0, 0};
        for (int i = 0; i < lm; ++i)
          for (int q = 0; q < 2; ++q) {
            d2min[q] = d2min[q] + s->d2w_rmin[i] * psr[2 * (i + 1) + q];
            dmin[q] = dmin[q] + s->dw_rmin[i] * psr[2 * (i + 1) + q];
          }
        for (int i = 0; i < lm; ++i)
          for (int q = 0; q < 2; ++q) {
            d2max[q] = d2max[q] + s->d2w_rmax[i] * psr[2 * (R - 2 - i) + q];
            dmax[q] = dmax[q] + s->dw_rmax[i] * psr[2 * (R - 2 - i) + q];
          }
        for (int r = 0; r < R; ++r) {
          CX(s->upFR, m, r)[0] = -1.0 * dps[2 * r]; CX(s->upFR, m, r)[1] = -1.0 * dps[2 * r + 1];
          double ar, ai;
          cmul(0.0, 1.0 * (double)m * rr[r], psr[2 * r], psr[2 * r + 1], &ar, &ai);
          CX(s->urFR, m, r)[0] = ar; CX(s->urFR, m, r)[1] = ai;
        }
        for (int q = 0; q < 2; ++q) {
          if (s->p.mbc == 0) {
            CX(s->omg_spec, m, 0)[q] = -1.0 * (d2min[q] - 2.0 * s->dw_rmin[0] * dmin[q]);
            CX(s->omg_spec, m, R - 1)[q] = -1.0 * (d2max[q] - 2.0 * s->dw_rmax[0] * dmax[q]);
          } else {
            CX(s->omg_spec, m, 0)[q] = -2.0 / s->radius[0] * dmin[q];
            CX(s->omg_spec, m, R - 1)[q] = -2.0 / s->radius[R - 1] * dmax[q];
          }
        }
        get_mode(s, s->upFR, m, ut);
        orc_chebtransform(R, ut, ut + 2 * R);
        put_mode(s, s->upFC, m, ut + 2 * R);
      }
    }
    free(v); free(solw);
  }
  size_t cf = 2 * (size_t)M * R;
  memcpy(s->tFR, s->temp_spec, cf * sizeof(double));
  memcpy(s->omgFR, s->omg_spec, cf * sizeof(double));
}

/* Assembly_stage_SA, src/fourierloop_imexrk.F90:653-665 */
static void assembly_stage_sa(orc_sim* s) {
  int M = s->M, R = s->R;
  size_t cf = 2 * (size_t)M * R;
  memcpy(s->temp_spec, s->tFR, cf * sizeof(double));
  memcpy(s->omg_spec, s->omgFR, cf * sizeof(double));
  for (int r = 0; r < R; ++r) {
    s->uphi_bar_spec[2 * r] = CX(s->upFR, 0, r)[0];
    s->uphi_bar_spec[2 * r + 1] = CX(s->upFR, 0, r)[1];
  }
}

static void imexrk_step(orc_sim* s) {
  int R = s->R, M = s->M, ns = s->sch.n_exp;
  int n_step = s->n_step + 1;
  if (n_step == 1 && !s->mats_built) {
    /* mat_build_rk for every mode before the loop (src/steptime_imexrk.F90:93-95) */
    for (int m = 0; m < M; ++m) mat_build_rk(s, m, s->LAPpsi_all + (size_t)R * R * m, s->ipiv_lap + (size_t)R * m);
  }
  /* src/steptime_imexrk.F90:102-137: with a variable dt, the CFL step comes
   * from a nonlinear pass on the assembled state (non stiffly accurate
   * schemes) or from the last stage pass (stiffly accurate ones) */
  if (n_step == 1) {
    s->dt_new = s->p.dt;
    for (int i = 0; i < 4; ++i) s->dt_array[i] = s->p.dt;
  }
  if (s->p.l_vartimestep) {
    if (n_step == 1 && s->restarted) {
      nr_maxloop(s);
      compute_new_dt_rk(s, 0, n_step);
    }
    if (n_step > 1) {
      if (!s->sch.check_A || !s->sch.check_D) nr_maxloop(s);
      compute_new_dt_rk(s, 0, n_step);
    }
  } else {
    s->dt_new = s->p.dt;
    for (int i = 0; i < 4; ++i) s->dt_array[i] = s->p.dt;
  }
  for (int st = 0; st < ns; ++st) {
    if (st > 0) get_stage_var(s, st, n_step);
    double colsum = 0.0;
    for (int i = 0; i < ns; ++i) colsum += s->sch.aA[i][st];
    if ((n_step > 1 || st > 0 || s->restarted) && (colsum + s->sch.bA[st] != 0.0)) nr_maxloop(s);
    rhs_construct_stage(s, st);
  }
  if (!s->sch.check_A || !s->sch.check_D) assembly_stage(s);
  else assembly_stage_sa(s);
  s->tot_time = s->tot_time + s->dt_new;
  double* v = zalloc(2 * (size_t)R);
  get_mode(s, s->tFR, 0, v);
  orc_chebtransform(R, v, s->TFC);
  free(v);
  s->n_step = n_step;
}

/* ------------------------------------------------------------------------ */
/* Explicit RK (RK2, RK4): src/steptime_rk.F90:52-180,                       */
/* src/fourierloop_rk.F90, src/rhs_create_rk.F90                             */
/* ------------------------------------------------------------------------ */

/* psi from the vorticity of mode m >= 1 through LAPpsi (rhs = -omega with
 * zero boundary rows), then psii, u_phi = -dpsi/dr, u_r = i m psi / r, the
 * Johnston wall vorticity written into w[0], w[R-1], and upFC(m)
 * (src/fourierloop_rk.F90:168-212, :373-413). */
static void rk_psi_update(orc_sim* s, int m, double* w, double* v) {
  int R = s->R, M = s->M, lm = s->p.lagpts;
  const double* rr = s->r_radius;
  double* rhs = v; double* psr = v + 2 * R; double* dps = v + 4 * R; double* ut = v + 6 * R;
  double* solw = v + 8 * R;
  for (int r = 0; r < R; ++r) { rhs[2 * r] = -1.0 * w[2 * r]; rhs[2 * r + 1] = -1.0 * w[2 * r + 1]; }
  rhs[0] = 0.0; rhs[1] = 0.0; rhs[2 * (R - 1)] = 0.0; rhs[2 * (R - 1) + 1] = 0.0;
  matsolve_cplx(R, s->LAPpsi_all + (size_t)R * R * m, s->ipiv_lap + (size_t)R * m, rhs, solw);
  orc_chebinvtran(R, rhs, psr);
  orc_chebinvtranD1(R, rhs, dps);
  double d2min[2] = {0, 0}, dmin[2] = {0, 0}, d2max[2] = {0, 0}, dmax[2] = {0, 0};
  for (int i = 0; i < lm; ++i)
    for (int q = 0; q < 2; ++q) {
      d2min[q] = d2min[q] + s->d2w_rmin[i] * psr[2 * (i + 1) + q];
      dmin[q] = dmin[q] + s->dw_rmin[i] * psr[2 * (i + 1) + q];
    }
  for (int i = 0; i < lm; ++i)
    for (int q = 0; q < 2; ++q) {
      d2max[q] = d2max[q] + s->d2w_rmax[i] * psr[2 * (R - 2 - i) + q];
      dmax[q] = dmax[q] + s->dw_rmax[i] * psr[2 * (R - 2 - i) + q];
    }
  for (int r = 0; r < R; ++r) {
    CX(s->psii, m, r)[0] = psr[2 * r]; CX(s->psii, m, r)[1] = psr[2 * r + 1];
    CX(s->upFR, m, r)[0] = -1.0 * dps[2 * r]; CX(s->upFR, m, r)[1] = -1.0 * dps[2 * r + 1];
    double ar, ai;
    cmul(0.0, (double)m * rr[r], psr[2 * r], psr[2 * r + 1], &ar, &ai);
    CX(s->urFR, m, r)[0] = ar; CX(s->urFR, m, r)[1] = ai;
  }
  for (int q = 0; q < 2; ++q) {
    if (s->p.mbc == 0) {
      w[q] = -1.0 * (d2min[q] - 2.0 * s->dw_rmin[0] * dmin[q]);
      w[2 * (R - 1) + q] = -1.0 * (d2max[q] - 2.0 * s->dw_rmax[0] * dmax[q]);
    } else {
      w[q] = -2.0 * rr[0] * dmin[q];
      w[2 * (R - 1) + q] = -2.0 * rr[R - 1] * dmax[q];
    }
  }
  get_mode(s, s->upFR, m, ut);
  orc_chebtransform(R, ut, ut + 2 * R);
  put_mode(s, s->upFC, m, ut + 2 * R);
}

/* Mode 0 from uphi_bar: upFC(0), omega_0 = ubar/r + d ubar/dr, u_r = 0. */
static void rk_mode0_update(orc_sim* s, const double* u, double* w0, double* v) {
  int R = s->R, M = s->M;
  double* c = v; double* du = v + 2 * R;
  orc_chebtransform(R, u, c);
  put_mode(s, s->upFC, 0, c);
  orc_chebinvtranD1(R, c, du);
  for (int r = 0; r < R; ++r) {
    CX(s->urFR, 0, r)[0] = 0.0; CX(s->urFR, 0, r)[1] = 0.0;
    w0[2 * r] = u[2 * r] * s->r_radius[r] + du[2 * r];
    w0[2 * r + 1] = u[2 * r + 1] * s->r_radius[r] + du[2 * r + 1];
  }
}

/* Get_stage_var, src/fourierloop_rk.F90:75-222: Y_s = Y_0 + dt sum_i a(s,i) F_i */
static void rk_get_stage_var(orc_sim* s, int st) {
  int R = s->R, M = s->M, ns = s->sch.n_exp;
  double dt = s->dt_array[0];
#pragma omp parallel
  {
    double* v = zalloc(24 * (size_t)R);
#pragma omp for schedule(static)
    for (int m = 0; m < M; ++m) {
      double* F = v; double* y = v + 2 * R; double* wk = v + 4 * R;
      for (int i = 0; i < 2 * R; ++i) F[i] = 0.0;
      for (int i = 0; i < st; ++i)
        for (int r = 0; r < R; ++r) {
          const double* q = stg(s->dtemp_a, ns, i, M, m, r);
          F[2 * r] = F[2 * r] + s->sch.aA[st][i] * q[0];
          F[2 * r + 1] = F[2 * r + 1] + s->sch.aA[st][i] * q[1];
        }
      for (int r = 0; r < R; ++r) {
        const double* y0 = CX(s->temp_spec, m, r);
        CX(s->tFR, m, r)[0] = y0[0] + dt * F[2 * r];
        CX(s->tFR, m, r)[1] = y0[1] + dt * F[2 * r + 1];
      }
      CX(s->tFR, m, 0)[0] = (m == 0) ? 1.0 : 0.0; CX(s->tFR, m, 0)[1] = 0.0;
      CX(s->tFR, m, R - 1)[0] = 0.0; CX(s->tFR, m, R - 1)[1] = 0.0;
      for (int i = 0; i < 2 * R; ++i) F[i] = 0.0;
      for (int i = 0; i < st; ++i)
        for (int r = 0; r < R; ++r) {
          const double* q = stg(s->domg_a, ns, i, M, m, r);
          F[2 * r] = F[2 * r] + s->sch.aA[st][i] * q[0];
          F[2 * r + 1] = F[2 * r + 1] + s->sch.aA[st][i] * q[1];
        }
      if (m == 0) {
        for (int r = 0; r < R; ++r) {
          y[2 * r] = s->uphi_bar_spec[2 * r] + dt * F[2 * r];
          y[2 * r + 1] = s->uphi_bar_spec[2 * r + 1] + dt * F[2 * r + 1];
        }
        y[0] = 0.0; y[1] = 0.0; y[2 * (R - 1)] = 0.0; y[2 * (R - 1) + 1] = 0.0;
        put_mode(s, s->upFR, 0, y);
        rk_mode0_update(s, y, F, wk);
        put_mode(s, s->omgFR, 0, F);
      } else {
        for (int r = 0; r < R; ++r) {
          const double* y0 = CX(s->omg_spec, m, r);
          y[2 * r] = y0[0] + dt * F[2 * r];
          y[2 * r + 1] = y0[1] + dt * F[2 * r + 1];
        }
        rk_psi_update(s, m, y, wk);
        put_mode(s, s->omgFR, m, y);
      }
    }
    free(v);
  }
}

/* RHS_construct_stage with rhs_create_rk (src/fourierloop_rk.F90:224-279,
 * src/rhs_create_rk.F90:19-224): the full explicit right-hand sides. */
static void rk_rhs_construct_stage(orc_sim* s, int st) {
  int R = s->R, M = s->M, ns = s->sch.n_exp;
  const double* rr = s->r_radius;
  const double* rr2 = s->r_radius2;
  double rp = s->p.ra / s->p.pr;
#pragma omp parallel
  {
    double* wk = zalloc(24 * (size_t)R);
    double* a = wk + 12 * R; double* b = wk + 14 * R; double* o = wk + 16 * R; double* l = wk + 18 * R;
#pragma omp for schedule(static)
    for (int m = 0; m < M; ++m) {
      get_mode(s, s->uphi_temp_FR, m, a);
      get_mode(s, s->ur_temp_FR, m, b);
      advect_term(s, m, a, b, o, wk);
      get_mode(s, s->tFR, m, a);
      lap_phys(s, m, a, l, wk);
      for (int r = 0; r < R; ++r) {
        double* d = stg(s->dtemp_a, ns, st, M, m, r);
        d[0] = (1.0 / s->p.pr) * l[2 * r] + o[2 * r];
        d[1] = (1.0 / s->p.pr) * l[2 * r + 1] + o[2 * r + 1];
      }
      if (m == 0) continue;
      get_mode(s, s->uphi_omg_FR, m, a);
      get_mode(s, s->ur_omg_FR, m, b);
      advect_term(s, m, a, b, o, wk);
      get_mode(s, s->omgFR, m, a);
      lap_phys(s, m, a, l, wk);
      get_mode(s, s->tFR, m, a);
      for (int r = 0; r < R; ++r) {
        double br, bi;
        cmul(0.0, (double)m * rr[r], a[2 * r], a[2 * r + 1], &br, &bi);
        double* d = stg(s->domg_a, ns, st, M, m, r);
        d[0] = (l[2 * r] + o[2 * r]) - rp * br;
        d[1] = (l[2 * r + 1] + o[2 * r + 1]) - rp * bi;
      }
    }
    free(wk);
  }
  /* rhs_construct_uphi_bar (src/rhs_create_rk.F90:135-224): diffusion of
   * ubar minus the Fourier-space means of ur d(u_phi)/dr + ur u_phi / r,
   * with d(u_phi)/dr from upFC of every mode. */
  double* d1 = zalloc(2 * (size_t)M * R);
  double* d2u = zalloc(2 * (size_t)R);
  double* c = zalloc(2 * (size_t)R); double* tmp = zalloc(2 * (size_t)R);
  for (int m = 0; m < M; ++m) {
    get_mode(s, s->upFC, m, c);
    orc_chebinvtranD1(R, c, tmp);
    for (int r = 0; r < R; ++r) { d1[2 * ((size_t)M * r + m)] = tmp[2 * r]; d1[2 * ((size_t)M * r + m) + 1] = tmp[2 * r + 1]; }
    if (m == 0) orc_chebinvtranD2(R, c, d2u);
  }
  for (int r = 0; r < R; ++r) {
    double uu = 0.0, ud = 0.0;
    for (int m = 0; m < M; ++m) {
      const double* ur = CX(s->urFR, m, r);
      const double* up = CX(s->upFR, m, r);
      const double* du = d1 + 2 * ((size_t)M * r + m);
      if (m == 0) {
        uu = uu + (ur[0] * up[0] - ur[1] * up[1]);
        ud = ud + (ur[0] * du[0] - ur[1] * du[1]);
      } else {
        /* real(ur conj(up) + conj(ur) up) */
        uu = uu + ((ur[0] * up[0] - ur[1] * (-up[1])) + (ur[0] * up[0] - (-ur[1]) * up[1]));
        ud = ud + ((ur[0] * du[0] - ur[1] * (-du[1])) + (ur[0] * du[0] - (-ur[1]) * du[1]));
      }
    }
    const double* u0 = CX(s->upFR, 0, r);
    const double diff = (d2u[2 * r] - rr2[r] * u0[0]) + rr[r] * d1[2 * ((size_t)M * r)];
    double* d = stg(s->domg_a, ns, st, M, 0, r);
    d[0] = diff - (ud + rr[r] * uu);
    d[1] = 0.0;
  }
  free(d1); free(d2u); free(c); free(tmp);
}

/* Assembly_stage, src/fourierloop_rk.F90:281-424: Y_n = Y_0 + dt sum b_i F_i */
static void rk_assembly_stage(orc_sim* s) {
  int R = s->R, M = s->M, ns = s->sch.n_exp;
  double dt = s->dt_new;
#pragma omp parallel
  {
    double* v = zalloc(24 * (size_t)R);
#pragma omp for schedule(static)
    for (int m = 0; m < M; ++m) {
      double* F = v; double* y = v + 2 * R; double* wk = v + 4 * R;
      for (int i = 0; i < 2 * R; ++i) F[i] = 0.0;
      for (int i = 0; i < ns; ++i)
        for (int r = 0; r < R; ++r) {
          const double* q = stg(s->dtemp_a, ns, i, M, m, r);
          F[2 * r] = F[2 * r] + s->sch.bA[i] * q[0];
          F[2 * r + 1] = F[2 * r + 1] + s->sch.bA[i] * q[1];
        }
      for (int r = 0; r < R; ++r) {
        double* t = CX(s->temp_spec, m, r);
        t[0] = t[0] + dt * F[2 * r]; t[1] = t[1] + dt * F[2 * r + 1];
      }
      CX(s->temp_spec, m, 0)[0] = (m == 0) ? 1.0 : 0.0; CX(s->temp_spec, m, 0)[1] = 0.0;
      CX(s->temp_spec, m, R - 1)[0] = 0.0; CX(s->temp_spec, m, R - 1)[1] = 0.0;
      for (int i = 0; i < 2 * R; ++i) F[i] = 0.0;
      for (int i = 0; i < ns; ++i)
        for (int r = 0; r < R; ++r) {
          const double* q = stg(s->domg_a, ns, i, M, m, r);
          F[2 * r] = F[2 * r] + s->sch.bA[i] * q[0];
          F[2 * r + 1] = F[2 * r + 1] + s->sch.bA[i] * q[1];
        }
      if (m == 0) {
        for (int r = 0; r < R; ++r) {
          s->uphi_bar_spec[2 * r] = s->uphi_bar_spec[2 * r] + dt * F[2 * r];
          s->uphi_bar_spec[2 * r + 1] = s->uphi_bar_spec[2 * r + 1] + dt * F[2 * r + 1];
        }
        s->uphi_bar_spec[0] = 0.0; s->uphi_bar_spec[1] = 0.0;
        s->uphi_bar_spec[2 * (R - 1)] = 0.0; s->uphi_bar_spec[2 * (R - 1) + 1] = 0.0;
        rk_mode0_update(s, s->uphi_bar_spec, y, wk);
        put_mode(s, s->omg_spec, 0, y);
      } else {
        for (int r = 0; r < R; ++r) {
          const double* y0 = CX(s->omg_spec, m, r);
          y[2 * r] = y0[0] + dt * F[2 * r];
          y[2 * r + 1] = y0[1] + dt * F[2 * r + 1];
        }
        rk_psi_update(s, m, y, wk);
        put_mode(s, s->omg_spec, m, y);
      }
    }
    free(v);
  }
  size_t cf = 2 * (size_t)M * R;
  memcpy(s->tFR, s->temp_spec, cf * sizeof(double));
  memcpy(s->omgFR, s->omg_spec, cf * sizeof(double));
  put_mode(s, s->upFR, 0, s->uphi_bar_spec);
}

static void rk_step(orc_sim* s) {
  int R = s->R, M = s->M, ns = s->sch.n_exp;
  int n_step = s->n_step + 1;
  if (n_step == 1 && !s->mats_built) {
    /* mat_build_rk for every mode before the loop (src/steptime_rk.F90:92-94) */
    for (int m = 0; m < M; ++m) mat_build_rk(s, m, s->LAPpsi_all + (size_t)R * R * m, s->ipiv_lap + (size_t)R * m);
    s->mats_built = 1;
  }
  /* src/steptime_rk.F90:103-115: dt and dt_array reset every step, then
   * compute_new_dt from the last nonlinear pass */
  s->dt_new = s->p.dt;
  for (int i = 0; i < 4; ++i) s->dt_array[i] = s->p.dt;
  if (s->p.l_vartimestep && n_step > 1) compute_new_dt_rk(s, 1, n_step);
  for (int st = 0; st < ns; ++st) {
    if (st > 0) rk_get_stage_var(s, st);
    if (n_step > 1 || st > 0 || s->restarted) nr_maxloop(s);
    rk_rhs_construct_stage(s, st);
  }
  rk_assembly_stage(s);
  s->tot_time = s->tot_time + s->dt_new;
  double* v = zalloc(2 * (size_t)R);
  get_mode(s, s->tFR, 0, v);
  orc_chebtransform(R, v, s->TFC);
  free(v);
  s->n_step = n_step;
}

int orc_sim_step(orc_sim* s, int nsteps) {
  for (int k = 0; k < nsteps; ++k) {
    if (s->p.scheme_type == ORC_TYPE_IMEX) imex_step(s);
    else if (s->p.scheme_type == ORC_TYPE_IMEXRK) imexrk_step(s);
    else if (s->p.scheme_type == ORC_TYPE_RK) rk_step(s);
    else return -1;
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Diagnostics: writeKE_spectral src/output.F90:122-324, radInt              */
/* src/integ.F90:36-76                                                        */
/* ------------------------------------------------------------------------ */
static double radint(const orc_sim* s, const double* f) {
  int R = s->R;
  const double pi = PI_;
  double* ff = zalloc(4 * (size_t)R);
  double* ft = ff + 2 * R;
  for (int i = 0; i < R; ++i) {
    double rad = (s->rmin + (0.5 * (1.0 + cos((double)(R - 1 - i) * pi / (double)(R - 1)))));
    ff[2 * i] = f[i] * rad; ff[2 * i + 1] = 0.0;
  }
  orc_chebtransform(R, ff, ft);
  double ftot = 0.0;
  for (int i = 0; i < R; ++i) {
    double Qm = (i % 2 == 0) ? -1.0 / (double)(i * i - 1) : 0.0;
    double cc = (i == 0 || i == R - 1) ? 0.5 * ft[2 * i] * Qm : ft[2 * i] * Qm;
    ftot = ftot + cc;
  }
  free(ff);
  return pow(2.0 / (double)(R - 1), 0.5) * ftot;
}

int orc_sim_diagnostics(orc_sim* s, double* out) {
  int R = s->R, M = s->M, P = s->P, Nm = s->Nm;
  const double pi = PI_;
  double* ur2 = zalloc(R); double* up2 = zalloc(R); double* upb2 = zalloc(R);
  double* w2 = zalloc(R); double* urt = zalloc(R);
  double* upg = zalloc(P); double* urg = zalloc(P);
  for (int j = 0; j < R; ++j) {
    /* the reference overwrites the module grids up/ur here (output.F90:176-181) */
    orc_invfft(Nm, P, CX(s->upFR, 0, j), upg);
    orc_invfft(Nm, P, CX(s->urFR, 0, j), urg);
    memcpy(s->up + (size_t)P * j, upg, P * sizeof(double));
    memcpy(s->ur + (size_t)P * j, urg, P * sizeof(double));
    double upavg = 0.0, ur_t = 0.0;
    for (int q = 0; q < P; ++q) {
      upavg = upavg + upg[q];
      ur_t = ur_t + urg[q] * s->tt[q + (size_t)P * j];
    }
    upavg = upavg * (1.0 / (double)P);
    ur_t = ur_t * (1.0 / (double)P);
    urt[j] = ur_t;
    double a = 0.0, b = 0.0;
    for (int m = 0; m < M; ++m) {
      const double* u = CX(s->urFR, m, j); const double* v = CX(s->upFR, m, j);
      double pr, pi_;
      cmul(u[0], u[1], u[0], u[1], &pr, &pi_);
      a = a + hypot(pr, pi_);
      cmul(v[0], v[1], v[0], v[1], &pr, &pi_);
      b = b + hypot(pr, pi_);
    }
    ur2[j] = a; up2[j] = b;
    upb2[j] = upavg * upavg;
    double w = 0.0;
    for (int m = 0; m < M; ++m) {
      const double* o = CX(s->omgFR, m, j);
      if (m == 0) w = w + (o[0] * o[0] - o[1] * o[1]);
      else w = w + ((o[0] * o[0] + o[1] * o[1]) + (o[0] * o[0] + o[1] * o[1]));
    }
    w2[j] = w;
  }
  double urk = radint(s, ur2), upk = radint(s, up2), upbk = radint(s, upb2);
  double KE = 2.0 * pi * (urk + upk);
  double* dT = zalloc(2 * (size_t)R);
  orc_chebinvtranD1(R, s->TFC, dT);
  double eta = s->p.eta;
  double nus_b = dT[0] / ((1.0 - eta) / (eta * log(eta)));
  double nus_t = dT[2 * (R - 1)] / ((1.0 - eta) / (log(eta)));
  double vis1 = radint(s, w2);
  double vis;
  if (s->p.mbc == 1) {
    double sro = 4.0 * pi * 2.0 * up2[R - 1], sri = 4.0 * pi * 2.0 * up2[0];
    vis = 2.0 * pi * vis1 - (sro - sri);
  } else {
    vis = 2.0 * pi * vis1;
  }
  double buo = 2.0 * pi * s->p.ra / s->p.pr * radint(s, urt);
  out[0] = KE; out[1] = 2.0 * pi * urk; out[2] = 2.0 * pi * upk; out[3] = 2.0 * pi * upbk;
  out[4] = nus_t; out[5] = nus_b; out[6] = vis; out[7] = buo; out[8] = s->tot_time;
  free(ur2); free(up2); free(upb2); free(w2); free(urt); free(upg); free(urg); free(dT);
  return 0;
}

/* calculate_spectra (src/output.F90:327-355): per mode m, 4 pi radInt of
 * |ur_m ur_m + up_m up_m| (complex squares) and of |T_m|. */
int orc_sim_spectra(orc_sim* s, double* kespec, double* tspec) {
  int R = s->R, M = s->M;
  const double pi = PI_;
  double* ek = zalloc(R);
  double* ts = zalloc(R);
  for (int m = 0; m < M; ++m) {
    for (int r = 0; r < R; ++r) {
      const double* u = CX(s->urFR, m, r); const double* v = CX(s->upFR, m, r); const double* t = CX(s->tFR, m, r);
      double ar, ai, br, bi;
      cmul(u[0], u[1], u[0], u[1], &ar, &ai);
      cmul(v[0], v[1], v[0], v[1], &br, &bi);
      ek[r] = hypot(ar + br, ai + bi);
      ts[r] = hypot(t[0], t[1]);
    }
    kespec[m] = 4.0 * pi * radint(s, ek);
    tspec[m] = 4.0 * pi * radint(s, ts);
  }
  free(ek);
  free(ts);
  return 0;
}

/* The u_phi force balance of writeKE_spectral (src/output.F90:145-228):
 * per radius r (out[4 r + 0..3]): radius, real((upFR(0) - upFR_prev(0))/dt),
 * the advection real(-(ur d(up)/dr + ur up / r)) summed over modes as the
 * reference forms it (m = 0 product, conjugate pairs for m >= 1), and the
 * diffusion real(d2 up_0/dr2 - up_0/r^2 + d up_0/dr / r), the derivatives
 * from chebinvtranD1/D2 of upFC. */
int orc_sim_upbalance(orc_sim* s, double* out) {
  int R = s->R, M = s->M;
  double* d1 = zalloc(2 * (size_t)M * R);
  double* d2 = zalloc(2 * (size_t)M * R);
  double* c = zalloc(2 * (size_t)R);
  double* v = zalloc(2 * (size_t)R);
  for (int m = 0; m < M; ++m) {
    get_mode(s, s->upFC, m, c);
    orc_chebinvtranD1(R, c, v);
    put_mode(s, d1, m, v);
    orc_chebinvtranD2(R, c, v);
    put_mode(s, d2, m, v);
  }
  for (int r = 0; r < R; ++r) {
    double pr = 0.0, pi_ = 0.0, qr = 0.0, qi = 0.0;  /* ur_up_FR, ur_d1up_FR */
    for (int m = 0; m < M; ++m) {
      const double* u = CX(s->urFR, m, r); const double* w = CX(s->upFR, m, r);
      const double* dw = d1 + 2 * ((size_t)m + (size_t)M * r);
      double ar, ai, br, bi;
      if (m == 0) {
        cmul(u[0], u[1], w[0], w[1], &ar, &ai);
        pr = pr + ar; pi_ = pi_ + ai;
        cmul(u[0], u[1], dw[0], dw[1], &ar, &ai);
        qr = qr + ar; qi = qi + ai;
      } else {
        cmul(u[0], u[1], w[0], -w[1], &ar, &ai);
        cmul(u[0], -u[1], w[0], w[1], &br, &bi);
        pr = pr + (ar + br); pi_ = pi_ + (ai + bi);
        cmul(u[0], u[1], dw[0], -dw[1], &ar, &ai);
        cmul(u[0], -u[1], dw[0], dw[1], &br, &bi);
        qr = qr + (ar + br); qi = qi + (ai + bi);
      }
    }
    const double* u0 = CX(s->upFR, 0, r); const double* up0 = CX(s->upFR_prev, 0, r);
    const double* d10 = d1 + 2 * ((size_t)M * r); const double* d20 = d2 + 2 * ((size_t)M * r);
    out[4 * r + 0] = s->radius[r];
    out[4 * r + 1] = (u0[0] - up0[0]) / s->dt_new;
    out[4 * r + 2] = -(qr + s->r_radius[r] * pr);
    out[4 * r + 3] = d20[0] - s->r_radius2[r] * u0[0] + s->r_radius[r] * d10[0];
  }
  free(d1); free(d2); free(c); free(v);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Checkpoint and snapshot files: store_checkpoint / store_checkpoint_imexrk */
/* and store_snapshot (src/output.F90:359-516), Fortran unformatted          */
/* sequential records framed by their byte length (4-byte integers).          */
/* ------------------------------------------------------------------------ */
static int rec_write(FILE* f, const void* data, size_t bytes) {
  int32_t n = (int32_t)bytes;
  return fwrite(&n, 4, 1, f) == 1 && (bytes == 0 || fwrite(data, 1, bytes, f) == bytes) && fwrite(&n, 4, 1, f) == 1;
}

int orc_sim_store_checkpoint(const orc_sim* s, const char* path) {
  int R = s->R, M = s->M, type = s->p.scheme_type;
  int ni, ne, nmax, li, le; /* header orders, and levels of the rhs records */
  if (type == ORC_TYPE_IMEX) {
    ni = s->sch.n_imp; ne = s->sch.n_exp; nmax = ni > ne ? ni : ne; li = ni; le = ne;
  } else {
    ni = ne = nmax = s->sch.n_exp;
    li = le = (type == ORC_TYPE_IMEXRK) ? 1 : ni;
  }
  FILE* f = fopen(path, "wb");
  if (!f) return -1;
  unsigned char hdr[36];
  int32_t iv[5] = {s->Nm, R, ni, ne, nmax};
  memcpy(hdr, &s->dt_new, 8); memcpy(hdr + 8, &s->tot_time, 8); memcpy(hdr + 16, iv, 20);
  int ok = rec_write(f, hdr, 36);
  double dta[8];
  for (int i = 0; i < nmax; ++i) dta[i] = (i < 4) ? s->dt_array[i] : s->dt_array[3];
  ok = ok && rec_write(f, dta, sizeof(double) * nmax);
  size_t cf = 2 * (size_t)M * R;
  ok = ok && rec_write(f, s->tFR, cf * sizeof(double)) && rec_write(f, s->omgFR, cf * sizeof(double)) &&
       rec_write(f, s->urFR, cf * sizeof(double)) && rec_write(f, s->upFR, cf * sizeof(double));
  int ms = (type == ORC_TYPE_IMEX);
  /* (order, M, R) arrays are held in that layout; the uphi_bar ones are (R, order) and transposed */
  const double* h3[4] = {ms ? s->rhs_imp_temp : NULL, ms ? s->rhs_exp_temp : NULL,
                         ms ? s->rhs_imp_vort : NULL, ms ? s->rhs_exp_vort : NULL};
  const int lv3[4] = {li, le, li, le};
  for (int k = 0; k < 4 && ok; ++k) {
    size_t n = cf * lv3[k];
    double* z = zalloc(n);
    if (h3[k]) memcpy(z, h3[k], n * sizeof(double));
    ok = rec_write(f, z, n * sizeof(double));
    free(z);
  }
  const double* h2[2] = {ms ? s->rhs_imp_uphi : NULL, ms ? s->rhs_exp_uphi : NULL};
  const int lv2[2] = {li, le};
  for (int k = 0; k < 2 && ok; ++k) {
    int n = lv2[k];
    double* z = zalloc(2 * (size_t)n * R);
    if (h2[k])
      for (int r = 0; r < R; ++r)
        for (int io = 0; io < n; ++io) {
          z[2 * (io + (size_t)n * r)] = h2[k][2 * ((size_t)R * io + r)];
          z[2 * (io + (size_t)n * r) + 1] = h2[k][2 * ((size_t)R * io + r) + 1];
        }
    ok = rec_write(f, z, 2 * (size_t)n * R * sizeof(double));
    free(z);
  }
  return (fclose(f) == 0 && ok) ? 0 : -1;
}

int orc_sim_store_snapshot(const orc_sim* s, const char* path) {
  int R = s->R, M = s->M;
  FILE* f = fopen(path, "wb");
  if (!f) return -1;
  double a[3] = {s->p.ra, s->p.pr, s->p.eta}, b[2] = {s->dt_new, s->tot_time};
  int32_t nn[2] = {s->Nm, R};
  size_t cf = 2 * (size_t)M * R;
  int ok = rec_write(f, a, sizeof(a)) && rec_write(f, b, sizeof(b)) && rec_write(f, nn, sizeof(nn)) &&
           rec_write(f, s->radius, sizeof(double) * R) && rec_write(f, s->tFR, cf * sizeof(double)) &&
           rec_write(f, s->omgFR, cf * sizeof(double)) && rec_write(f, s->urFR, cf * sizeof(double)) &&
           rec_write(f, s->upFR, cf * sizeof(double));
  return (fclose(f) == 0 && ok) ? 0 : -1;
}

/* ------------------------------------------------------------------------ */
/* Restart (l_restart): read_checkpoint and get_checkpoint_data             */
/* (src/init.F90:447-935), the restart branch of init_fields (:183-204) and  */
/* the multistep bootstrap of timeloop_imex (src/steptime.F90:87-193) with   */
/* rhs_*_from_restart (src/rhs_create.F90:387-573).                          */
/* ------------------------------------------------------------------------ */
static int rec_read(FILE* f, double** buf, size_t* bytes) {
  int32_t n1, n2;
  *buf = NULL;
  if (fread(&n1, 4, 1, f) != 1 || n1 < 0) return -1;
  *buf = (double*)malloc(n1 ? (size_t)n1 : 8);
  if (n1 && fread(*buf, 1, (size_t)n1, f) != (size_t)n1) return -1;
  if (fread(&n2, 4, 1, f) != 1 || n2 != n1) return -1;
  *bytes = (size_t)n1;
  return 0;
}

typedef struct {
  double dt_new, tot_time;
  int nm, nr, ni, ne, nmax;
  double dta[8];
  double* fld[4];  /* tFR, omgFR, urFR, upFR: complex (nm+1, nr) */
  double* h3[4];   /* rhs_imp_temp, rhs_exp_temp, rhs_imp_vort, rhs_exp_vort (order, M, R) */
  double* h2[2];   /* rhs_imp_uphi_bar, rhs_exp_uphi_bar (order, R) */
} ckpt_t;

static void ckpt_free(ckpt_t* c) {
  for (int k = 0; k < 4; ++k) { free(c->fld[k]); free(c->h3[k]); }
  for (int k = 0; k < 2; ++k) free(c->h2[k]);
}

/* read_checkpoint (src/init.F90:865-935) reads the header, dt_array and the
 * four fields; the history records that follow are read here as well when
 * they hold ni / ne levels (files of the multistep loop), else left NULL. */
static int ckpt_read(const char* path, ckpt_t* c) {
  memset(c, 0, sizeof(*c));
  FILE* f = fopen(path, "rb");
  if (!f) return -1;
  double* b = NULL;
  size_t n = 0;
  int ok = rec_read(f, &b, &n) == 0 && n == 36;
  if (ok) {
    int32_t iv[5];
    memcpy(&c->dt_new, b, 8); memcpy(&c->tot_time, (char*)b + 8, 8); memcpy(iv, (char*)b + 16, 20);
    c->nm = iv[0]; c->nr = iv[1]; c->ni = iv[2]; c->ne = iv[3]; c->nmax = iv[4];
    ok = c->nm >= 1 && c->nr >= 4 && c->ni >= 1 && c->ne >= 1 && c->nmax >= 1 && c->nmax <= 8;
  }
  free(b);
  ok = ok && rec_read(f, &b, &n) == 0 && n == sizeof(double) * (size_t)c->nmax;
  if (ok) memcpy(c->dta, b, n);
  free(b);
  size_t cf = 2 * (size_t)(c->nm + 1) * c->nr;
  for (int k = 0; k < 4 && ok; ++k) {
    ok = rec_read(f, &c->fld[k], &n) == 0 && n == cf * sizeof(double);
  }
  const int lv[6] = {c->ni, c->ne, c->ni, c->ne, c->ni, c->ne};
  for (int k = 0; k < 6 && ok; ++k) {
    double* h = NULL;
    if (rec_read(f, &h, &n) != 0) { free(h); break; }
    size_t want = sizeof(double) * 2 * (size_t)lv[k] * (k < 4 ? (size_t)(c->nm + 1) * c->nr : (size_t)c->nr);
    if (n != want) { free(h); continue; }
    if (k < 4) c->h3[k] = h; else c->h2[k - 4] = h;
  }
  fclose(f);
  if (!ok) { ckpt_free(c); return -1; }
  return 0;
}

/* Grid change at restart (src/init.F90:726-861): per radial line, the
 * unnormalised DCT-I of the old values (chebtransform_redft), zero padding
 * to the new length, the DCT-I at the new length divided by 2(Nr-1)
 * (chebinvtran_redft), then the factor (Nr-1)/(Nr_old-1). */
static void cheb_resample(int ro, int rn, const double* x, double* y) {
  double* c = zalloc(2 * (size_t)rn);
  redft00_cplx(ro, x, c);
  for (int k = ro; k < rn; ++k) { c[2 * k] = 0.0; c[2 * k + 1] = 0.0; }
  redft00_cplx(rn, c, y);
  double fac = (2.0 * (double)(rn - 1)) / (2.0 * (double)(ro - 1));
  for (int i = 0; i < 2 * rn; ++i) y[i] = y[i] / (2.0 * (double)(rn - 1));
  for (int i = 0; i < 2 * rn; ++i) y[i] = y[i] * fac;
  free(c);
}

/* rhs_temp/vort/uphibar_from_restart for the state held in tFR..upFR after
 * a nonlinear pass on it: implicit slot si, explicit slot se (0-based). */
static void history_from_state(orc_sim* s, int si, int se) {
  int R = s->R, M = s->M, ni = s->sch.n_imp, ne = s->sch.n_exp;
  const double* rr = s->r_radius;
  double rp = s->p.ra / s->p.pr;
  double* wk = zalloc(8 * (size_t)R);
  double* a = wk; double* b = wk + 2 * R; double* bs = wk + 4 * R; double* db = wk + 6 * R;
  for (int m = 0; m < M; ++m) {
    double dm = (double)m;
    for (int f = 0; f < 2; ++f) {
      get_mode(s, f == 0 ? s->uphi_temp_FR : s->uphi_omg_FR, m, a);
      get_mode(s, f == 0 ? s->ur_temp_FR : s->ur_omg_FR, m, b);
      orc_chebtransform(R, b, bs);
      orc_chebinvtranD1(R, bs, db);
      double* imp = f == 0 ? s->rhs_imp_temp : s->rhs_imp_vort;
      double* ex = f == 0 ? s->rhs_exp_temp : s->rhs_exp_vort;
      const double* st = f == 0 ? s->tFR : s->omgFR;
      for (int i = 0; i < R; ++i) {
        double* hi = hist(imp, ni, si, M, m, i);
        double* he = hist(ex, ne, se, M, m, i);
        hi[0] = CX(st, m, i)[0]; hi[1] = CX(st, m, i)[1];
        double ar, ai;
        cmul(0.0, dm * rr[i], a[2 * i], a[2 * i + 1], &ar, &ai);
        he[0] = ar + db[2 * i] + rr[i] * b[2 * i];
        he[1] = ai + db[2 * i + 1] + rr[i] * b[2 * i + 1];
        if (f == 1) {
          double* bu = hist(s->rhs_buo_term, ni, si, M, m, i);
          double br, bi;
          cmul(0.0, dm * rr[i], CX(s->tFR, m, i)[0], CX(s->tFR, m, i)[1], &br, &bi);
          bu[0] = -rp * br; bu[1] = -rp * bi;
        }
      }
    }
  }
  mean_ur_omg(s, wk);
  for (int i = 0; i < R; ++i) {
    s->rhs_imp_uphi[2 * ((size_t)R * si + i)] = CX(s->upFR, 0, i)[0];
    s->rhs_imp_uphi[2 * ((size_t)R * si + i) + 1] = CX(s->upFR, 0, i)[1];
    s->rhs_exp_uphi[2 * ((size_t)R * se + i)] = wk[i];
    s->rhs_exp_uphi[2 * ((size_t)R * se + i) + 1] = 0.0;
  }
  free(wk);
}

int orc_sim_restart(orc_sim* s, const char* dir, int npoint, int add_pert, double ampT) {
  const int type = s->p.scheme_type, R = s->R, M = s->M, Nm = s->Nm;
  const int ni = s->sch.n_imp, ne = s->sch.n_exp;
  const int started = (type == ORC_TYPE_IMEX) && s->p.l_imexrk_started;
  const int nfiles = started ? ni : 1;  /* CN, BDF2: 2 files; BDF3: 3; BDF4: 4 */
  const size_t cf = 2 * (size_t)M * R;
  if (npoint - nfiles + 1 < 0) return -1;
  ckpt_t c[4];
  memset(c, 0, sizeof(c));
  int rc = 0;
  for (int j = 0; j < nfiles && rc == 0; ++j) {
    char path[4096];
    snprintf(path, sizeof(path), "%s/checkpoint_%05d", dir, npoint - (nfiles - 1) + j);
    if (ckpt_read(path, &c[j]) != 0) rc = -2;
  }
  const ckpt_t* nw = &c[nfiles - 1];
  if (rc == 0) {
    int same = nw->nm == Nm && nw->nr == R;
    int grow = nw->nm <= Nm && nw->nr <= R && !same;
    if (!same && !grow) rc = -3;                       /* a smaller grid is not restored */
    if (!same && type == ORC_TYPE_IMEX) rc = -4;       /* histories cannot change grid */
    for (int j = 0; j < nfiles && rc == 0 && started; ++j)
      if (c[j].nm != Nm || c[j].nr != R) rc = -4;
    if (rc == 0 && type == ORC_TYPE_IMEX && !started && !(nw->h3[0] && nw->h3[1] && nw->h2[0] && nw->h2[1]))
      rc = -5;                                         /* no multistep histories in the file */
    if (rc == 0 && type == ORC_TYPE_IMEX && !started && nw->ne > ni && ne > nw->ne) rc = -5;
  }
  if (rc != 0) {
    for (int j = 0; j < nfiles; ++j) ckpt_free(&c[j]);
    return rc;
  }
  /* dt_array */
  int nmax = ni > ne ? ni : ne;
  double dta[8];
  for (int i = 0; i < 8; ++i) dta[i] = s->p.dt;
  if (started) {
    for (int j = 0; j < nfiles; ++j) dta[nfiles - 1 - j] = c[j].dta[0];
  } else {
    int mo = nw->nmax;
    for (int i = 0; i < (nmax < mo ? nmax : mo); ++i) dta[i] = nw->dta[i];
    for (int i = mo; i < nmax; ++i) dta[i] = dta[mo - 1];
  }
  for (int i = 0; i < 4; ++i) s->dt_array[i] = dta[i];
  /* zero every history and stage store, as allocated */
  if (s->rhs_imp_temp) {
    memset(s->rhs_imp_temp, 0, cf * ni * sizeof(double)); memset(s->rhs_imp_vort, 0, cf * ni * sizeof(double));
    memset(s->rhs_buo_term, 0, cf * ni * sizeof(double)); memset(s->rhs_exp_temp, 0, cf * ne * sizeof(double));
    memset(s->rhs_exp_vort, 0, cf * ne * sizeof(double));
    memset(s->rhs_imp_uphi, 0, 2 * (size_t)R * ni * sizeof(double));
    memset(s->rhs_exp_uphi, 0, 2 * (size_t)R * ne * sizeof(double));
  }
  if (s->dtemp_a) {
    memset(s->dtemp_a, 0, cf * ne * sizeof(double)); memset(s->dtemp_d, 0, cf * ne * sizeof(double));
    memset(s->domg_a, 0, cf * ne * sizeof(double)); memset(s->domg_d, 0, cf * ne * sizeof(double));
    memset(s->rhs_buo, 0, cf * ne * sizeof(double));
  }
  double* dst[4] = {s->tFR, s->omgFR, s->urFR, s->upFR};
  if (started) {
    /* timeloop_imex restart branch: for each stored step, oldest first, a
     * nonlinear pass on it and its history entries; implicit slot
     * n_imp - j, explicit slot n_exp - j (0-based, j = 0 the oldest) */
    for (int j = 0; j < nfiles; ++j) {
      for (int k = 0; k < 4; ++k) memcpy(dst[k], c[j].fld[k], cf * sizeof(double));
      nr_maxloop(s);
      history_from_state(s, ni - 1 - j, ne - 1 - j);
    }
  } else if (nw->nm == Nm && nw->nr == R) {
    for (int k = 0; k < 4; ++k) memcpy(dst[k], nw->fld[k], cf * sizeof(double));
    if (type == ORC_TYPE_IMEX) {
      /* the file's histories with the order rules of src/init.F90:593-716
       * (the reference's own read of these records is commented out) */
      int io_ = nw->ni, eo = nw->ne;
      for (int i = 0; i < ni; ++i) {
        int src = i < io_ ? i : io_ - 1;
        for (size_t mr = 0; mr < (size_t)M * R; ++mr)
          for (int q = 0; q < 2; ++q) {
            s->rhs_imp_temp[2 * (i + (size_t)ni * mr) + q] = nw->h3[0][2 * (src + (size_t)io_ * mr) + q];
            s->rhs_imp_vort[2 * (i + (size_t)ni * mr) + q] = nw->h3[2][2 * (src + (size_t)io_ * mr) + q];
          }
        for (int r = 0; r < R; ++r)
          for (int q = 0; q < 2; ++q)
            s->rhs_imp_uphi[2 * ((size_t)R * i + r) + q] = nw->h2[0][2 * (src + (size_t)io_ * r) + q];
      }
      for (int i = 0; i < ne; ++i) {
        for (size_t mr = 0; mr < (size_t)M * R; ++mr)
          for (int q = 0; q < 2; ++q) {
            if (i < eo) {
              s->rhs_exp_temp[2 * (i + (size_t)ne * mr) + q] = nw->h3[1][2 * (i + (size_t)eo * mr) + q];
              s->rhs_exp_vort[2 * (i + (size_t)ne * mr) + q] = nw->h3[3][2 * (i + (size_t)eo * mr) + q];
            } else {  /* rhs_exp(j) = rhs_imp(n_exp_old), src/init.F90:673-679 */
              s->rhs_exp_temp[2 * (i + (size_t)ne * mr) + q] = s->rhs_imp_temp[2 * ((eo - 1) + (size_t)ni * mr) + q];
              s->rhs_exp_vort[2 * (i + (size_t)ne * mr) + q] = s->rhs_imp_vort[2 * ((eo - 1) + (size_t)ni * mr) + q];
            }
          }
        for (int r = 0; r < R; ++r)
          for (int q = 0; q < 2; ++q)
            s->rhs_exp_uphi[2 * ((size_t)R * i + r) + q] =
                i < eo ? nw->h2[1][2 * (i + (size_t)eo * r) + q] : s->rhs_imp_uphi[2 * ((size_t)R * (eo - 1) + r) + q];
      }
    }
  } else {
    /* larger grid (IMEXRK, RK): modes above the old Nm are zero */
    int mo = nw->nm + 1, ro = nw->nr;
    double* x = zalloc(2 * (size_t)ro);
    double* y = zalloc(2 * (size_t)R);
    for (int k = 0; k < 4; ++k) {
      memset(dst[k], 0, cf * sizeof(double));
      for (int m = 0; m < M; ++m) {
        for (int r = 0; r < ro; ++r) {
          x[2 * r] = m < mo ? nw->fld[k][2 * (m + (size_t)mo * r)] : 0.0;
          x[2 * r + 1] = m < mo ? nw->fld[k][2 * (m + (size_t)mo * r) + 1] : 0.0;
        }
        cheb_resample(ro, R, x, y);
        put_mode(s, dst[k], m, y);
      }
    }
    free(x); free(y);
  }
  if (s->rhs_imp_temp) {
    memcpy(s->tmp_imp_temp, s->rhs_imp_temp, cf * ni * sizeof(double));
    memcpy(s->tmp_exp_temp, s->rhs_exp_temp, cf * ne * sizeof(double));
    memcpy(s->tmp_imp_vort, s->rhs_imp_vort, cf * ni * sizeof(double));
    memcpy(s->tmp_exp_vort, s->rhs_exp_vort, cf * ne * sizeof(double));
    memcpy(s->tmp_buo_term, s->rhs_buo_term, cf * ni * sizeof(double));
    memcpy(s->tmp_imp_uphi, s->rhs_imp_uphi, 2 * (size_t)R * ni * sizeof(double));
    memcpy(s->tmp_exp_uphi, s->rhs_exp_uphi, 2 * (size_t)R * ne * sizeof(double));
  }
  /* init_fields, restart branch */
  if (add_pert)
    for (size_t e = 0; e < (size_t)M * R; ++e) s->tFR[2 * e] = ampT + s->tFR[2 * e];
  memcpy(s->temp_spec, s->tFR, cf * sizeof(double));
  memcpy(s->omg_spec, s->omgFR, cf * sizeof(double));
  for (int r = 0; r < R; ++r) {
    s->uphi_bar_spec[2 * r] = CX(s->upFR, 0, r)[0];
    s->uphi_bar_spec[2 * r + 1] = CX(s->upFR, 0, r)[1];
  }
  /* upFC is not assigned by the reference's restart; the Chebyshev transform
   * of u_phi is what a continuing run holds */
  {
    double* v = zalloc(4 * (size_t)R);
    for (int m = 0; m < M; ++m) {
      get_mode(s, s->upFR, m, v);
      orc_chebtransform(R, v, v + 2 * R);
      put_mode(s, s->upFC, m, v + 2 * R);
    }
    free(v);
  }
  memcpy(s->upFR_prev, s->upFR, cf * sizeof(double));
  memcpy(s->urFR_prev, s->urFR, cf * sizeof(double));
  memset(s->psii, 0, cf * sizeof(double));
  s->tot_time = nw->tot_time;
  s->dt_new = nw->dt_new;
  s->n_step = 0;
  s->mats_built = 0;
  s->restarted = 1;
  for (int j = 0; j < nfiles; ++j) ckpt_free(&c[j]);
  return 0;
}
