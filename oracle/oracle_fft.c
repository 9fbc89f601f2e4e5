/*
 * Mixed-radix complex FFT for the CPU oracle (test infrastructure only).
 *
 * The reference calls FFTW3 (src/fourier_fftw.F90:51,93 and
 * src/chebyshev_fftw.F90:140,178,183,282,342,404,417).  FFTW is not vendored
 * by the reference and is absent here, so this file restates the published
 * discrete Fourier transform with FFTW's sign convention:
 *   out[k] = sum_j in[j] * exp(sign * 2*pi*i*j*k/n),  unnormalised.
 * Algorithm: recursive decimation in time over the prime factorisation of n
 * (radix 4, 2, then odd primes; odd primes by the direct O(p^2) sum).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

typedef struct {
  int n;
  int nf;
  int fac[64];
  double* tw_fwd; /* exp(-2 pi i k / n), k in [0,n) */
  double* tw_bwd; /* exp(+2 pi i k / n) */
} fft_plan;

#define MAX_PLANS 64
static fft_plan g_plans[MAX_PLANS];
static int g_nplans = 0;

static void factorize_n(int n, int* fac, int* nf) {
  int k = 0;
  while (n % 4 == 0) { fac[k++] = 4; n /= 4; }
  while (n % 2 == 0) { fac[k++] = 2; n /= 2; }
  for (int p = 3; p * p <= n; p += 2)
    while (n % p == 0) { fac[k++] = p; n /= p; }
  if (n > 1) fac[k++] = n;
  *nf = k;
}

static const fft_plan* get_plan(int n) {
  const fft_plan* found = NULL;
#pragma omp critical(orc_fft_plan)
  {
    for (int i = 0; i < g_nplans; ++i)
      if (g_plans[i].n == n) { found = &g_plans[i]; break; }
    if (!found && g_nplans < MAX_PLANS) {
      fft_plan* p = &g_plans[g_nplans];
      p->n = n;
      factorize_n(n, p->fac, &p->nf);
      p->tw_fwd = (double*)malloc(sizeof(double) * 2 * (size_t)n);
      p->tw_bwd = (double*)malloc(sizeof(double) * 2 * (size_t)n);
      const double two_pi = 8.0 * atan(1.0);
      for (int k = 0; k < n; ++k) {
        double a = two_pi * (double)k / (double)n;
        double c = cos(a), s = sin(a);
        p->tw_fwd[2 * k] = c; p->tw_fwd[2 * k + 1] = -s;
        p->tw_bwd[2 * k] = c; p->tw_bwd[2 * k + 1] = s;
      }
      __sync_synchronize();
      g_nplans++;
      found = p;
    }
  }
  return found;
}

/* out: n outputs contiguous; in: read with stride `is` (complex elements). */
static void fft_rec(double* out, const double* in, int is, const int* fac, int nf,
                    int n, int fstride, const double* tw) {
  int p = fac[0];
  int m = n / p;
  if (nf == 1) {
    for (int j = 0; j < p; ++j) {
      out[2 * j] = in[2 * (size_t)j * is];
      out[2 * j + 1] = in[2 * (size_t)j * is + 1];
    }
  } else {
    for (int q = 0; q < p; ++q)
      fft_rec(out + 2 * (size_t)q * m, in + 2 * (size_t)q * is, is * p, fac + 1, nf - 1, m,
              fstride * p, tw);
  }
  /* butterflies: combine p sub-transforms of length m */
  const int ntot_ = n * fstride;
  if (p == 2) {
    for (int k = 0; k < m; ++k) {
      double* a = out + 2 * k;
      double* b = out + 2 * (k + m);
      long idx = (long)k * fstride;
      double wr = tw[2 * idx], wi = tw[2 * idx + 1];
      double br = b[0] * wr - b[1] * wi, bi = b[0] * wi + b[1] * wr;
      b[0] = a[0] - br; b[1] = a[1] - bi;
      a[0] = a[0] + br; a[1] = a[1] + bi;
    }
    return;
  }
  if (p == 4) {
    /* w_4 = exp(sign*i*pi/2): tw[ntot/4] gives (0, sign) */
    const double s = tw[2 * (ntot_ / 4) + 1];
    for (int k = 0; k < m; ++k) {
      double r[4], im[4];
      for (int q = 0; q < 4; ++q) {
        double ar = out[2 * (k + q * m)], ai = out[2 * (k + q * m) + 1];
        long idx = (long)q * k * fstride;
        double wr = tw[2 * idx], wi = tw[2 * idx + 1];
        r[q] = ar * wr - ai * wi;
        im[q] = ar * wi + ai * wr;
      }
      double t0r = r[0] + r[2], t0i = im[0] + im[2];
      double t1r = r[0] - r[2], t1i = im[0] - im[2];
      double t2r = r[1] + r[3], t2i = im[1] + im[3];
      double t3r = r[1] - r[3], t3i = im[1] - im[3];
      /* multiply t3 by w_4 = (0, s): (x + i y) * i s = -s y + i s x */
      double u3r = -s * t3i, u3i = s * t3r;
      out[2 * k] = t0r + t2r;            out[2 * k + 1] = t0i + t2i;
      out[2 * (k + m)] = t1r + u3r;      out[2 * (k + m) + 1] = t1i + u3i;
      out[2 * (k + 2 * m)] = t0r - t2r;  out[2 * (k + 2 * m) + 1] = t0i - t2i;
      out[2 * (k + 3 * m)] = t1r - u3r;  out[2 * (k + 3 * m) + 1] = t1i - u3i;
    }
    return;
  }
  double xr[64], xi[64];
  double* xr_big = NULL;
  double* xi_big = NULL;
  double* xr_use = xr;
  double* xi_use = xi;
  if (p > 64) {
    xr_big = (double*)malloc(sizeof(double) * p);
    xi_big = (double*)malloc(sizeof(double) * p);
    xr_use = xr_big; xi_use = xi_big;
  }
  const int ntot = n * fstride; /* full transform length of the twiddle table */
  for (int k = 0; k < m; ++k) {
    for (int q = 0; q < p; ++q) {
      double ar = out[2 * (k + q * m)], ai = out[2 * (k + q * m) + 1];
      long idx = ((long)q * k * fstride) % ntot;
      double wr = tw[2 * idx], wi = tw[2 * idx + 1];
      xr_use[q] = ar * wr - ai * wi;
      xi_use[q] = ar * wi + ai * wr;
    }
    for (int j = 0; j < p; ++j) {
      double sr = 0.0, si = 0.0;
      for (int q = 0; q < p; ++q) {
        long idx = ((long)j * q * m * fstride) % ntot;
        double wr = tw[2 * idx], wi = tw[2 * idx + 1];
        sr += xr_use[q] * wr - xi_use[q] * wi;
        si += xr_use[q] * wi + xi_use[q] * wr;
      }
      out[2 * (k + j * m)] = sr;
      out[2 * (k + j * m) + 1] = si;
    }
  }
  if (xr_big) { free(xr_big); free(xi_big); }
}

void orc_fft(int n, const double* in, double* out, int sign) {
  const fft_plan* p = get_plan(n);
  if (n == 1) { out[0] = in[0]; out[1] = in[1]; return; }
  if (in == out) {
    double* tmp = (double*)malloc(sizeof(double) * 2 * (size_t)n);
    memcpy(tmp, in, sizeof(double) * 2 * (size_t)n);
    fft_rec(out, tmp, 1, p->fac, p->nf, n, 1, sign < 0 ? p->tw_fwd : p->tw_bwd);
    free(tmp);
  } else {
    fft_rec(out, in, 1, p->fac, p->nf, n, 1, sign < 0 ? p->tw_fwd : p->tw_bwd);
  }
}
