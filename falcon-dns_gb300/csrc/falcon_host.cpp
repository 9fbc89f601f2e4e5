// Host runtime of the GB300 FAlCon-DNS time step: parameters and namelist,
// operator construction from the reference's LU factors, grouped device
// state, step sequencing, batching, serving and the C ABI of falcon_gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/falcon_gpu.h"
#include "falcon_internal.h"
#include "falcon_tc.h"
#include "imexrk_tables.h"

using namespace falcon;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CK(call)                                                                  \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return fail(FALCON_ECUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

std::atomic<long long> g_launches(0);
std::atomic<int> g_graphs(1);  // replay steady-state steps as CUDA graphs

// Optional per-launch CUDA-event timing (falcon_batch_profile).
enum KernelClass { KC_NONLIN = 0, KC_GEMM_RADIAL, KC_GEMM_MODE, KC_ELEMENTWISE, KC_COUNT };
const char* kClassNames[KC_COUNT] = {"nonlin_fft", "gemm_radial", "gemm_mode_solve", "elementwise"};
struct Prof {
  struct Rec { int cls; cudaEvent_t a, b; double flops; };
  std::vector<Rec> recs;
};

// ---------------------------------------------------------------------------
// Dense algebra on the host (operator construction only).  dgetrf/dgetrs
// restate LAPACK's partial-pivoting LU (src/algebra_lapack.F90:14-53).
// ---------------------------------------------------------------------------
int host_dgetrf(int n, double* a, int* ipiv) {
  int info = 0;
  for (int j = 0; j < n; ++j) {
    int p = j;
    double amax = std::fabs(a[j + (size_t)n * j]);
    for (int i = j + 1; i < n; ++i) {
      double v = std::fabs(a[i + (size_t)n * j]);
      if (v > amax) { amax = v; p = i; }
    }
    ipiv[j] = p + 1;
    if (a[p + (size_t)n * j] != 0.0) {
      if (p != j)
        for (int k = 0; k < n; ++k) std::swap(a[j + (size_t)n * k], a[p + (size_t)n * k]);
      const double piv = a[j + (size_t)n * j];
      if (std::fabs(piv) >= 2.2250738585072014e-308) {
        const double rp = 1.0 / piv;
        for (int i = j + 1; i < n; ++i) a[i + (size_t)n * j] *= rp;
      } else {
        for (int i = j + 1; i < n; ++i) a[i + (size_t)n * j] /= piv;
      }
    } else if (info == 0) {
      info = j + 1;
    }
    for (int k = j + 1; k < n; ++k) {
      const double akj = a[j + (size_t)n * k];
      if (akj != 0.0)
        for (int i = j + 1; i < n; ++i) a[i + (size_t)n * k] -= a[i + (size_t)n * j] * akj;
    }
  }
  return info;
}

void host_dgetrs(int n, const double* a, const int* ipiv, double* b) {
  for (int i = 0; i < n; ++i) {
    const int p = ipiv[i] - 1;
    if (p != i) std::swap(b[i], b[p]);
  }
  for (int j = 0; j < n; ++j) {
    const double bj = b[j];
    if (bj != 0.0)
      for (int i = j + 1; i < n; ++i) b[i] -= bj * a[i + (size_t)n * j];
  }
  for (int j = n - 1; j >= 0; --j) {
    if (b[j] != 0.0) {
      b[j] = b[j] / a[j + (size_t)n * j];
      const double bj = b[j];
      for (int i = 0; i < j; ++i) b[i] -= bj * a[i + (size_t)n * j];
    }
  }
}

template <class F>
void parallel_for(int n, F f) {
  unsigned nt = std::max(1u, std::thread::hardware_concurrency());
  nt = std::min<unsigned>(nt, (unsigned)std::max(1, n));
  std::atomic<int> next(0);
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&]() {
      for (int i = next++; i < n; i = next++) f(i);
    });
  for (auto& t : th) t.join();
}

// ---------------------------------------------------------------------------
// Chebyshev collocation (dcheb, src/chebyshev_fftw.F90:88-121) and grid
// (init_grid, src/init.F90:120-162).
// ---------------------------------------------------------------------------
struct Cheb {
  int R;
  std::vector<double> xp, t, D, D2;  // column-major (R,R): t(i,j) = T_{j}(x_i)
  std::vector<double> radius, inv_r, inv_r2, dr;
  double rmin, rmax;
};

Cheb make_cheb(int R, double eta) {
  Cheb c;
  c.R = R;
  c.rmin = eta / (1.0 - eta);
  c.rmax = 1.0 / (1.0 - eta);
  const double pi = 4.0 * std::atan(1.0);
  c.xp.resize(R);
  c.t.assign((size_t)R * R, 0.0);
  c.D.assign((size_t)R * R, 0.0);
  c.D2.assign((size_t)R * R, 0.0);
  for (int i = 0; i < R; ++i) c.xp[i] = std::cos(((double)(R - 1 - i) * pi) / (double)(R - 1));
  std::vector<double> tt(R), dt(R), d2t(R);
  for (int i = 0; i < R; ++i) {
    tt[0] = 1.0; tt[1] = c.xp[i];
    dt[0] = 0.0; dt[1] = 1.0;
    d2t[0] = 0.0; d2t[1] = 0.0;
    for (int j = 2; j < R; ++j) {
      tt[j] = 2.0 * c.xp[i] * tt[j - 1] - tt[j - 2];
      dt[j] = 2.0 * tt[j - 1] + 2.0 * c.xp[i] * dt[j - 1] - dt[j - 2];
      d2t[j] = 4.0 * dt[j - 1] + 2.0 * c.xp[i] * d2t[j - 1] - d2t[j - 2];
    }
    for (int j = 0; j < R; ++j) {
      c.t[i + (size_t)R * j] = tt[j];
      c.D[i + (size_t)R * j] = 2.0 * dt[j];
      c.D2[i + (size_t)R * j] = 4.0 * d2t[j];
    }
  }
  c.radius.resize(R); c.inv_r.resize(R); c.inv_r2.resize(R); c.dr.resize(R);
  for (int i = 0; i < R; ++i) {
    c.radius[i] = (c.rmin + (0.5 * (1.0 + std::cos((double)(R - 1 - i) * pi / (double)(R - 1)))));
    c.inv_r[i] = 1.0 / c.radius[i];
  }
  for (int i = 0; i < R - 1; ++i) c.dr[i + 1] = c.radius[i + 1] - c.radius[i];
  c.dr[0] = c.dr[1];
  for (int i = 0; i < R; ++i) c.inv_r2[i] = c.inv_r[i] * c.inv_r[i];
  return c;
}

// ---------------------------------------------------------------------------
// Operator key and shared operator sets
// ---------------------------------------------------------------------------
struct OpKey {
  int R, Nm, mbc, type, imp, exp;
  double dt, pr, eta, wt;
  int needs_lap, lagpts;
  // Grouping only (0 for operator sets): a variable-dt instance carries a
  // unique tag so that it never shares a group (its dt is its own).
  long long tag;
  bool operator<(const OpKey& o) const {
    return std::tie(R, Nm, mbc, type, imp, exp, dt, pr, eta, wt, needs_lap, lagpts, tag) <
           std::tie(o.R, o.Nm, o.mbc, o.type, o.imp, o.exp, o.dt, o.pr, o.eta, o.wt, o.needs_lap, o.lagpts, o.tag);
  }
};

struct OpSet {
  OpKey key;
  int R = 0, M = 0;
  // device, column-major (lda = rows)
  double* D1p = nullptr;   // R x R physical d/dr
  double* Lp = nullptr;    // R x R physical d2/dr2 + r^-1 d/dr
  double* ST = nullptr;    // M blocks of R x R: chebinvtran o AT_m^-1
  double* G = nullptr;     // M blocks of 3R x R: [Tinv X_w; Tinv X_psi; -D1inv X_psi]
  double* U = nullptr;      // 2R x R: [Tinv A_u^-1; D1inv A_u^-1]
  double* LAP = nullptr;    // M blocks of (2R+2) x R: [Tinv; -D1inv; wall omega rows] o LAPpsi_m^-1
  double* inv_r = nullptr;
  double* inv_r2 = nullptr;
  double* wq = nullptr;     // radInt weights (src/integ.F90:36-76) on values
  double* d1_0 = nullptr;   // rows 0 and R-1 of D1p
  double* d1_R = nullptr;
  // Explicit RK only: chebinvtranD1 and chebinvtranD2 + r^-1 chebinvtranD1
  // applied to values taken as scaled coefficients (C D H, C (D2 + r^-1 D) H),
  // for the first stage of a run, where the reference's upFC holds upFR
  // (src/init.F90:252, used by src/rhs_create_rk.F90:158-161).
  double* D1c = nullptr;
  double* Lc = nullptr;
  // Exact bf16 slices of each operator for the tensor-core GEMM (one entry
  // per operator array: its FP64 base, shape and slice arrays).
  struct Oz {
    const double* base = nullptr;
    long lda = 0, sA = 0;
    int rows = 0, K = 0, nb = 0, rowsP = 0, KP = 0, w = 6;
    uint16_t* s = nullptr;
    int* ex = nullptr;
    CUtensorMap tmap{};     // the slices for the tcgen05 kernel's copies
    bool tmap_ok = false;
  };
  std::vector<Oz> oz;
  size_t bytes = 0;
  ~OpSet() {
    // the last group holding the set is gone, but a kernel of any group's
    // stream that read it may still run: every stream drains first
    cudaDeviceSynchronize();
    cudaFree(D1p); cudaFree(Lp); cudaFree(ST); cudaFree(G); cudaFree(U); cudaFree(LAP);
    cudaFree(inv_r); cudaFree(inv_r2); cudaFree(wq); cudaFree(d1_0); cudaFree(d1_R);
    cudaFree(D1c); cudaFree(Lc);
    for (auto& o : oz) { cudaFree(o.s); cudaFree(o.ex); }
  }
};

// Contraction paths (the modes of gemm() below): 4 (default) measured per
// shape by the autotuner; 3 tcgen05 wherever possible; 2 tcgen05 where a
// contraction fills the GPU, mma.sync otherwise; 1 mma.sync only; 0 FP64
// FMA tiles.  The two sliced kernels give the same bits; all paths are
// FP64-accurate.
std::atomic<int> g_gemm_mode{4};

// Slices of one column-major operator array (rows x K, lda = rows, nb
// entries of stride sA) for the tensor-core GEMM.
int add_oz(OpSet* ops, const double* base, int rows, int K, int nb, long sA) {
  if (!base || K > 257) return 0;
  OpSet::Oz o;
  o.base = base; o.lda = rows; o.sA = sA; o.rows = rows; o.K = K; o.nb = nb;
  o.rowsP = oz_rows_padded(rows);
  o.KP = ((K + 15) / 16) * 16;
  o.w = oz_width_for(o.KP);
  const size_t ns = (size_t)nb * oz_slices(o.w) * o.rowsP * o.KP, ne = (size_t)nb * o.rowsP;
  CK(cudaMalloc(&o.s, ns * sizeof(uint16_t)));
  CK(cudaMalloc(&o.ex, ne * sizeof(int)));
  CK(cudaMemset(o.s, 0, ns * sizeof(uint16_t)));
  CK(cudaMemset(o.ex, 0, ne * sizeof(int)));
  CK(launch_oz_slice_rows(base, rows, sA, rows, K, nb, o.s, o.ex, o.rowsP, o.KP, o.w, 0));
  o.tmap_ok = tc_stage_layout_check(o.w, o.KP) == 0 &&
              tc_make_operator_map(&o.tmap, o.s, nb, oz_slices(o.w), o.KP, o.rowsP) == 0;
  ops->bytes += ns * sizeof(uint16_t) + ne * sizeof(int);
  ops->oz.push_back(o);
  return 0;
}

std::mutex g_ops_mu;
std::map<OpKey, std::weak_ptr<OpSet>> g_ops;

// Physical-space derivative matrices (the composition chebtransform ->
// derivative recurrence -> inverse transform of src/chebyshev_fftw.F90 is
// linear; its matrix is D H t^T diag(c') / (R-1), H = diag(1/2,1,..,1,1/2),
// c' = (1,2,..,2,1), by discrete orthogonality at the Gauss-Lobatto points).
void phys_deriv(const Cheb& c, std::vector<double>& D1p, std::vector<double>& Lp) {
  const int R = c.R;
  std::vector<double> W((size_t)R * R);  // W(j,i) = h_j t(i,j) c'_i / (R-1), coefficient j from value i
  for (int j = 0; j < R; ++j) {
    const double h = (j == 0 || j == R - 1) ? 0.5 : 1.0;
    for (int i = 0; i < R; ++i) {
      const double cp = (i == 0 || i == R - 1) ? 1.0 : 2.0;
      W[j + (size_t)R * i] = h * c.t[i + (size_t)R * j] * cp / (double)(R - 1);
    }
  }
  D1p.assign((size_t)R * R, 0.0);
  Lp.assign((size_t)R * R, 0.0);
  for (int i = 0; i < R; ++i)      // output point
    for (int k = 0; k < R; ++k) {  // input point
      double s1 = 0.0, s2 = 0.0;
      for (int j = 0; j < R; ++j) {
        const double w = W[j + (size_t)R * k];
        s1 += c.D[i + (size_t)R * j] * w;
        s2 += c.D2[i + (size_t)R * j] * w;
      }
      D1p[i + (size_t)R * k] = s1;
      Lp[i + (size_t)R * k] = s2 + c.inv_r[i] * s1;
    }
}

// mat_build_uphibar(_IRK) (src/mat_assembly.F90:189-240, :361-413)
void assemble_Au(const Cheb& c, int mbc, double dt, double wt, std::vector<double>& A) {
  const int R = c.R;
  const double C = std::pow(2.0 / (double)(R - 1), 0.5);
  A.assign((size_t)R * R, 0.0);
  for (int j = 0; j < R; ++j) {
    for (int i = 0; i < R; ++i)
      A[i + (size_t)R * j] = c.t[i + (size_t)R * j] -
                             wt * dt * (c.inv_r[i] * c.D[i + (size_t)R * j] + c.D2[i + (size_t)R * j] -
                                        c.inv_r2[i] * c.t[i + (size_t)R * j]);
    if (mbc == 0) {
      A[0 + (size_t)R * j] = c.t[0 + (size_t)R * j];
      A[R - 1 + (size_t)R * j] = c.t[R - 1 + (size_t)R * j];
    } else {
      A[0 + (size_t)R * j] = c.D[0 + (size_t)R * j] - c.inv_r[0] * c.t[0 + (size_t)R * j];
      A[R - 1 + (size_t)R * j] = c.D[R - 1 + (size_t)R * j] - c.inv_r[R - 1] * c.t[R - 1 + (size_t)R * j];
    }
  }
  for (int i = 0; i < R; ++i) { A[i] *= 0.5; A[i + (size_t)R * (R - 1)] *= 0.5; }
  for (auto& v : A) v = C * v;
}

// Coefficients -> values (chebinvtran) and -> d/dr values (chebinvtranD1)
// as matrices: Tinv = C t H, D1inv = C D H.
void apply_inv(const Cheb& c, const double* coef, double* val, double* dval) {
  const int R = c.R;
  const double C = std::pow(2.0 / (double)(R - 1), 0.5);
  for (int i = 0; i < R; ++i) {
    double s = 0.0, d = 0.0;
    for (int j = 0; j < R; ++j) {
      const double h = (j == 0 || j == R - 1) ? 0.5 : 1.0;
      s += c.t[i + (size_t)R * j] * h * coef[j];
      d += c.D[i + (size_t)R * j] * h * coef[j];
    }
    if (val) val[i] = C * s;
    if (dval) dval[i] = C * d;
  }
}

// dlagrange / d2lagrange (src/chebyshev_fftw.F90:449-517): derivatives at x
// of the Lagrange basis on the points xp.
void dlagrange(int n, const double* xp, double x, double* dw) {
  std::vector<double> w(n, 1.0), ww(n, 0.0);
  for (int i = 0; i < n; ++i) dw[i] = 0.0;
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
}

void d2lagrange(int n, const double* xp, double x, double* d2w) {
  std::vector<double> w(n, 1.0), ww(n, 0.0), mw(n, 0.0);
  for (int i = 0; i < n; ++i) d2w[i] = 0.0;
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
}

// Wall vorticity of the Johnston strategy (src/fourierloop_imexrk.F90:
// 586-637) as weights on the physical psi values: omega(wall) = sum_i
// win[i] psi(i), over the lm interior points next to each wall.
void johnston_weights(const Cheb& c, int lagpts, int mbc, std::vector<double>& win, std::vector<double>& wout) {
  const int R = c.R;
  int lm = std::min(lagpts, R - 2);
  if (lm < 1) lm = 1;
  std::vector<double> pts(lm), dwmin(lm), d2wmin(lm), dwmax(lm), d2wmax(lm);
  for (int i = 0; i < lm; ++i) pts[i] = c.radius[1 + i];
  dlagrange(lm, pts.data(), c.rmin, dwmin.data());
  d2lagrange(lm, pts.data(), c.rmin, d2wmin.data());
  for (int i = 0; i < lm; ++i) pts[i] = c.radius[R - 2 - i];
  dlagrange(lm, pts.data(), c.rmax, dwmax.data());
  d2lagrange(lm, pts.data(), c.rmax, d2wmax.data());
  win.assign(R, 0.0);
  wout.assign(R, 0.0);
  for (int i = 0; i < lm; ++i) {
    if (mbc == 0) {
      win[1 + i] += -1.0 * (d2wmin[i] - 2.0 * dwmin[0] * dwmin[i]);
      wout[R - 2 - i] += -1.0 * (d2wmax[i] - 2.0 * dwmax[0] * dwmax[i]);
    } else {
      win[1 + i] += -2.0 / c.radius[0] * dwmin[i];
      wout[R - 2 - i] += -2.0 / c.radius[R - 1] * dwmax[i];
    }
  }
}

template <class T>
int upload(T** dst, const std::vector<T>& v, size_t* acc) {
  CK(cudaMalloc(dst, sizeof(T) * v.size()));
  CK(cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice));
  // a copy from pageable memory may return before its DMA has landed, and
  // the kernels that read these tables run on non-blocking streams, which
  // do not wait for the legacy stream
  CK(cudaStreamSynchronize(0));
  if (acc) *acc += sizeof(T) * v.size();
  return 0;
}

// LU factors and 1-based pivots of the implicit operators made by the
// caller's own mat_build* + dgetrf, in the reference's layouts
// (src/mat_assembly.F90): AT_all (R,R,M), IPIV1 (R,M); AF_all (2R,2R,M),
// IPIV2 (2R,M); A_uphi_all (R,R,1), IPIV_uphi (R); LAPpsi_all (R,R,M),
// IPIV1_lap (R,M).  A null block is built on the device instead.
struct HostFactors {
  const double *AT = nullptr, *AF = nullptr, *Au = nullptr, *LAP = nullptr;
  const int *pT = nullptr, *pF = nullptr, *pu = nullptr, *pL = nullptr;
};

// The per-mode combined operators of one key, built on the device:
//   ST[m] = chebinvtran o AT_m^-1                          (R x R)
//   G[m]  = [chebinvtran; chebinvtran; -chebinvtranD1] o the omega, psi and
//           psi rows of AF_m^-1 on the vorticity right-hand side (3R x R)
//   LAP[m] = [chebinvtran; -chebinvtranD1; wall omega] o LAPpsi_m^-1
// Factorisations: batched dgetf2/dgetrs (falcon_ops.cu) on modes in chunks
// that keep the workspace near 256 MB.  Products: the DFMA GEMM.  G[0] and
// LAP[0] stay zero (the m = 0 flow is the u_phi_bar equation).
int build_mode_operators(const OpKey& k, const Cheb& c, OpSet* ops, const HostFactors* hf) {
  const int R = c.R, M = k.Nm + 1;
  const size_t RR = (size_t)R * R;
  cudaStream_t s = nullptr;
  const double C = std::pow(2.0 / (double)(R - 1), 0.5);
  // chebinvtran / chebinvtranD1 on scaled coefficients as column-major
  // matrices: Tinv = C t H, D1inv = C D H (negated for u_phi = -dpsi/dr).
  std::vector<double> tinv(RR), mdinv(RR);
  for (int j = 0; j < R; ++j) {
    const double h = (j == 0 || j == R - 1) ? 0.5 : 1.0;
    for (int i = 0; i < R; ++i) {
      tinv[i + (size_t)R * j] = C * c.t[i + (size_t)R * j] * h;
      mdinv[i + (size_t)R * j] = -(C * c.D[i + (size_t)R * j] * h);
    }
  }
  std::vector<double> win, wout, pin(R, 0.0), pout(R, 0.0);
  if (k.needs_lap) {
    johnston_weights(c, k.lagpts, k.mbc, win, wout);
    for (int kk = 0; kk < R; ++kk)
      for (int i = 0; i < R; ++i) {
        pin[kk] += win[i] * tinv[i + (size_t)R * kk];
        pout[kk] += wout[i] * tinv[i + (size_t)R * kk];
      }
  }
  const size_t per_mode = 6 * RR;  // AF (4 RR) + its right-hand sides (2 RR)
  const int mc = (int)std::max<size_t>(1, std::min<size_t>((size_t)M, ((size_t)256 << 20) / (per_mode * 8)));
  double *d_t = nullptr, *d_D = nullptr, *d_D2 = nullptr, *d_ir = nullptr, *d_ir2 = nullptr, *d_tinv = nullptr,
         *d_mdinv = nullptr, *d_pin = nullptr, *d_pout = nullptr, *Wm = nullptr, *Wr = nullptr;
  int *d_info = nullptr, *d_piv = nullptr;
  auto cleanup = [&]() {
    for (void* q : {(void*)d_t, (void*)d_D, (void*)d_D2, (void*)d_ir, (void*)d_ir2, (void*)d_tinv, (void*)d_mdinv,
                    (void*)d_pin, (void*)d_pout, (void*)Wm, (void*)Wr, (void*)d_info, (void*)d_piv})
      cudaFree(q);
  };
  int rc = 0;
  if ((rc = upload(&d_t, c.t, nullptr)) || (rc = upload(&d_D, c.D, nullptr)) || (rc = upload(&d_D2, c.D2, nullptr)) ||
      (rc = upload(&d_ir, c.inv_r, nullptr)) || (rc = upload(&d_ir2, c.inv_r2, nullptr)) ||
      (rc = upload(&d_tinv, tinv, nullptr)) || (rc = upload(&d_mdinv, mdinv, nullptr)) ||
      (rc = upload(&d_pin, pin, nullptr)) || (rc = upload(&d_pout, pout, nullptr))) {
    cleanup();
    return rc;
  }
  auto dev_alloc = [&](double** q, size_t n) -> int {
    if (cudaMalloc(q, sizeof(double) * n) != cudaSuccess) return fail(FALCON_ENOMEM, "operator workspace");
    if (cudaMemset(*q, 0, sizeof(double) * n) != cudaSuccess) return fail(FALCON_ECUDA, "operator workspace");
    return 0;
  };
  const long lap_rows = 2L * R + 2;
  const bool implicit = (k.type != FALCON_RK);  // explicit RK needs only LAPpsi
  if ((rc = dev_alloc(&Wm, 4 * RR * mc)) || (rc = dev_alloc(&Wr, 2 * RR * mc)) ||
      (implicit && (rc = dev_alloc(&ops->ST, RR * M))) || (implicit && (rc = dev_alloc(&ops->G, 3 * RR * M))) ||
      (k.needs_lap && (rc = dev_alloc(&ops->LAP, (size_t)lap_rows * R * M)))) {
    cleanup();
    return rc;
  }
  ops->bytes += (implicit ? sizeof(double) * 4 * RR * M : 0) + (k.needs_lap ? sizeof(double) * lap_rows * R * M : 0);
  if (cudaMalloc(&d_info, sizeof(int) * mc) != cudaSuccess) { cleanup(); return fail(FALCON_ENOMEM, "info"); }
  if (hf && cudaMalloc(&d_piv, sizeof(int) * 2 * (size_t)R * mc) != cudaSuccess) {
    cleanup();
    return fail(FALCON_ENOMEM, "pivots");
  }
  // the caller's factors of modes [m, m + nb) of one operator (order n):
  // factors into Wm, pivots into d_piv, then dgetrs on the unit right-hand
  // sides in Wr
  auto solve_given = [&](const double* lu, const int* piv, int n, int m, int nb, int off) -> int {
    const size_t nn = (size_t)n * n;
    cudaError_t e = cudaMemcpy(Wm, lu + (size_t)m * nn, sizeof(double) * nn * nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_piv, piv + (size_t)m * n, sizeof(int) * (size_t)n * nb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_unit_rhs(n, R, off, nb, Wr, s);
    if (e == cudaSuccess) e = launch_getrs_rows(n, nb, Wm, nn, d_piv, (size_t)n, Wr, (size_t)n * R, R, s);
    if (e != cudaSuccess) return fail(FALCON_ECUDA, std::string("solve with given factors: ") + cudaGetErrorString(e));
    return 0;
  };
  auto ck = [&](cudaError_t e, const char* what) -> int {
    if (e != cudaSuccess) return fail(FALCON_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return 0;
  };
  auto check_info = [&](int nb, int m_first, const char* what) -> int {
    std::vector<int> info(nb);
    const cudaError_t e = cudaMemcpy(info.data(), d_info, sizeof(int) * nb, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(FALCON_ECUDA, std::string("operator build (") + what + "): " + cudaGetErrorString(e));
    for (int m = 0; m < nb; ++m)
      if (info[m] != 0)
        return fail(FALCON_ESINGULAR, std::string("dgetrf: singular ") + what + " for mode " + std::to_string(m_first + m));
    return 0;
  };
  // out (column-major, leading dimension ldy) = P X for each mode, with X the
  // row-major solutions (stride sA) and P column-major (nrows_p x R).
  auto prod = [&](const double* Xrm, long sA, const double* Pcm, double* out, long ldy, int nrows_p, int nb) {
    GemmArgs g{};
    g.A = Xrm; g.lda = R; g.sA = sA;
    g.X = Pcm; g.ldx = nrows_p; g.sX = 0;
    g.Y = out; g.ldy = ldy; g.sY = ldy * R;
    g.K = R; g.rows = R; g.N = nrows_p; g.batch = nb; g.alpha = 1.0;
    return launch_gemm(g, s);
  };
  const double wdt = k.wt * k.dt;
  const int irk = (k.type == FALCON_IMEXRK) ? 1 : 0;
  const long L2 = (long)2 * RR, L3 = (long)3 * RR;
  for (int m0 = 0; m0 < M && rc == 0; m0 += mc) {
    const int nm = std::min(mc, M - m0);
    const int a0 = std::max(m0, 1), na = m0 + nm - a0;
    // temperature: ST[m] = Tinv AT_m^-1
    if (implicit && hf && hf->AT) {
      if ((rc = solve_given(hf->AT, hf->pT, R, m0, nm, 0)) ||
          (rc = ck(prod(Wr, (long)RR, d_tinv, ops->ST + (size_t)m0 * RR, R, R, nm), "ST product")))
        break;
    } else if (implicit && ((rc = ck(launch_assemble(0, R, m0, nm, d_t, d_D, d_D2, d_ir, d_ir2, wdt, 1.0 / k.pr, C, Wm, s), "assemble AT")) ||
        (rc = ck(launch_unit_rhs(R, R, 0, nm, Wr, s), "unit rhs")) ||
        (rc = ck(launch_lu_solve(R, nm, Wm, RR, Wr, RR, R, d_info, s), "lu AT")) ||
        (rc = check_info(nm, m0, "AT")) ||
        (rc = ck(prod(Wr, (long)RR, d_tinv, ops->ST + (size_t)m0 * RR, R, R, nm), "ST product"))))
      break;
    if (na <= 0) continue;
    // psi-omega: AF_m^-1 on [0; e_j], unknowns [psi; omega]
    double* Gm = implicit ? ops->G + (size_t)a0 * L3 : nullptr;
    const bool given_af = hf && hf->AF;
    if (implicit && given_af && (rc = solve_given(hf->AF, hf->pF, 2 * R, a0, na, R))) break;
    if (implicit && ((!given_af && ((rc = ck(launch_assemble_af(R, a0, na, k.mbc, irk, d_t, d_D, d_D2, d_ir, d_ir2, wdt, C, Wm, s), "assemble AF")) ||
        (rc = ck(launch_unit_rhs(2 * R, R, R, na, Wr, s), "unit rhs")) ||
        (rc = ck(launch_lu_solve(2 * R, na, Wm, 4 * RR, Wr, L2, R, d_info, s), "lu AF")) ||
        (rc = check_info(na, a0, "psi-omega operator")))) ||
        (rc = ck(prod(Wr + RR, L2, d_tinv, Gm, 3L * R, R, na), "G omega")) ||
        (rc = ck(prod(Wr, L2, d_tinv, Gm + R, 3L * R, R, na), "G psi")) ||
        (rc = ck(prod(Wr, L2, d_mdinv, Gm + 2 * R, 3L * R, R, na), "G uphi"))))
      break;
    if (!k.needs_lap) continue;
    double* Lm = ops->LAP + (size_t)a0 * lap_rows * R;
    const bool given_lap = hf && hf->LAP;
    if (given_lap && (rc = solve_given(hf->LAP, hf->pL, R, a0, na, 0))) break;
    if ((!given_lap && ((rc = ck(launch_assemble(4, R, a0, na, d_t, d_D, d_D2, d_ir, d_ir2, 0.0, 1.0, C, Wm, s), "assemble LAPpsi")) ||
        (rc = ck(launch_unit_rhs(R, R, 0, na, Wr, s), "unit rhs")) ||
        (rc = ck(launch_lu_solve(R, na, Wm, RR, Wr, RR, R, d_info, s), "lu LAPpsi")) ||
        (rc = check_info(na, a0, "psi Poisson operator")))) ||
        (rc = ck(prod(Wr, (long)RR, d_tinv, Lm, lap_rows, R, na), "LAP psi")) ||
        (rc = ck(prod(Wr, (long)RR, d_mdinv, Lm + R, lap_rows, R, na), "LAP uphi")) ||
        (rc = ck(prod(Wr, (long)RR, d_pin, Lm + 2 * R, lap_rows, 1, na), "LAP wall in")) ||
        (rc = ck(prod(Wr, (long)RR, d_pout, Lm + 2 * R + 1, lap_rows, 1, na), "LAP wall out")))
      break;
  }
  if (rc == 0) rc = ck(cudaDeviceSynchronize(), "operator build");
  cleanup();
  return rc;
}

// The operator set of key k: from the process-wide cache, else built on the
// device (and cached); with host factors hf, built from them and not cached
// (the set belongs to the one caller that gave them).
int build_opset(const OpKey& k, std::shared_ptr<OpSet>* out, const HostFactors* hf = nullptr) {
  if (!hf) {
    std::lock_guard<std::mutex> lk(g_ops_mu);
    auto it = g_ops.find(k);
    if (it != g_ops.end()) {
      if (auto sp = it->second.lock()) { *out = sp; return 0; }
    }
  }
  auto ops = std::make_shared<OpSet>();
  ops->key = k;
  const int R = k.R, M = k.Nm + 1;
  ops->R = R; ops->M = M;
  Cheb c = make_cheb(R, k.eta);
  std::vector<double> D1p, Lp;
  phys_deriv(c, D1p, Lp);
  std::vector<double> U((size_t)2 * R * R);
  int rc;
  if ((rc = build_mode_operators(k, c, ops.get(), hf))) return rc;
  {
    std::vector<double> Au;
    std::vector<int> pu(R);
    if (hf && hf->Au) {
      Au.assign(hf->Au, hf->Au + (size_t)R * R);
      pu.assign(hf->pu, hf->pu + R);
    } else {
      assemble_Au(c, k.mbc, k.dt, k.wt, Au);
      if (host_dgetrf(R, Au.data(), pu.data()) != 0) return fail(FALCON_ESINGULAR, "dgetrf: singular uphi_bar operator");
    }
    std::vector<double> x(R), v(R), dv(R);
    for (int j = 0; j < R; ++j) {
      std::fill(x.begin(), x.end(), 0.0);
      x[j] = 1.0;
      host_dgetrs(R, Au.data(), pu.data(), x.data());
      apply_inv(c, x.data(), v.data(), dv.data());
      for (int i = 0; i < R; ++i) {
        U[i + (size_t)2 * R * j] = v[i];
        U[R + i + (size_t)2 * R * j] = dv[i];
      }
    }
  }
  if ((rc = upload(&ops->D1p, D1p, &ops->bytes))) return rc;
  if ((rc = upload(&ops->Lp, Lp, &ops->bytes))) return rc;
  if ((rc = upload(&ops->U, U, &ops->bytes))) return rc;
  if ((rc = upload(&ops->inv_r, c.inv_r, &ops->bytes))) return rc;
  if ((rc = upload(&ops->inv_r2, c.inv_r2, &ops->bytes))) return rc;
  if (k.type == FALCON_RK) {
    const double C = std::pow(2.0 / (double)(R - 1), 0.5);
    std::vector<double> D1c((size_t)R * R), Lc((size_t)R * R);
    for (int j = 0; j < R; ++j) {
      const double h = (j == 0 || j == R - 1) ? 0.5 : 1.0;
      for (int i = 0; i < R; ++i) {
        const size_t q = i + (size_t)R * j;
        D1c[q] = C * c.D[q] * h;
        Lc[q] = C * c.D2[q] * h + c.inv_r[i] * D1c[q];
      }
    }
    if ((rc = upload(&ops->D1c, D1c, &ops->bytes))) return rc;
    if ((rc = upload(&ops->Lc, Lc, &ops->bytes))) return rc;
  }
  {
    // radInt(f) = fac * sum_k w_k Re(chebtransform(f r))_k with w_k = -1/(k^2-1)
    // for even k (halved at k = 0, R-1), 0 for odd k; chebtransform is
    // t^T diag(c') / ((R-1) fac) on the values.
    const double fac = std::sqrt(2.0 / (double)(R - 1));
    std::vector<double> wq(R, 0.0), d10(R), d1R(R);
    for (int k = 0; k < R; ++k) {
      if (k % 2 != 0) continue;
      double qk = -1.0 / (double)(k * k - 1);
      if (k == 0 || k == R - 1) qk *= 0.5;
      for (int j = 0; j < R; ++j) {
        const double cp = (j == 0 || j == R - 1) ? 1.0 : 2.0;
        wq[j] += qk * cp * c.t[j + (size_t)R * k] / ((double)(R - 1) * fac);
      }
    }
    for (int j = 0; j < R; ++j) {
      wq[j] *= fac * c.radius[j];
      d10[j] = D1p[0 + (size_t)R * j];
      d1R[j] = D1p[(R - 1) + (size_t)R * j];
    }
    if ((rc = upload(&ops->wq, wq, &ops->bytes))) return rc;
    if ((rc = upload(&ops->d1_0, d10, &ops->bytes))) return rc;
    if ((rc = upload(&ops->d1_R, d1R, &ops->bytes))) return rc;
  }
  {
    const long RR = (long)R * R;
    if ((rc = add_oz(ops.get(), ops->D1p, R, R, 1, RR)) || (rc = add_oz(ops.get(), ops->Lp, R, R, 1, RR)) ||
        (rc = add_oz(ops.get(), ops->ST, R, R, M, RR)) || (rc = add_oz(ops.get(), ops->G, 3 * R, R, M, 3 * RR)) ||
        (rc = add_oz(ops.get(), ops->U, 2 * R, R, 1, 2 * RR)) ||
        (rc = add_oz(ops.get(), ops->LAP, 2 * R + 2, R, M, (long)(2 * R + 2) * R)) ||
        (rc = add_oz(ops.get(), ops->D1c, R, R, 1, RR)) || (rc = add_oz(ops.get(), ops->Lc, R, R, 1, RR)))
      return rc;
    CK(cudaDeviceSynchronize());
  }
  if (!hf) {
    std::lock_guard<std::mutex> lk(g_ops_mu);
    g_ops[k] = ops;
  }
  *out = ops;
  return 0;
}

// ---------------------------------------------------------------------------
// Scheme tables (src/timeschemes.F90)
// ---------------------------------------------------------------------------
struct Scheme {
  int type = 0, imp = 0, exp = 0;
  int n_imp = 0, n_exp = 0;       // IMEX orders, or IMEXRK stages (n_exp)
  double w_imp[4] = {0}, w_exp[4] = {0}, wt_lhs = 0;
  double aD[kMaxStages][kMaxStages] = {{0}}, aA[kMaxStages][kMaxStages] = {{0}};
  double bD[kMaxStages] = {0}, bA[kMaxStages] = {0};
  bool check_A = false, check_D = false;
  bool diag_diff = false;         // implicit diagonal varies by stage
  int diag = 1;
};

// Multistep weights of rhs_update_wts_imp/_exp (src/timeschemes.F90:
// 1004-1052, 1621-1701) for the time-step history dta = dt_array(1..4)
// (dta[0] the newest); all-equal entries give the constant-dt weights.
int imex_weights(int imp, int exp, const double* dta, Scheme* s) {
  {
    const double* d = dta;
    switch (imp) {
      case FALCON_IMP_CN:
        s->n_imp = 2; s->w_imp[0] = 0.5; s->wt_lhs = 0.5;
        if (exp == FALCON_EXP_AB2) {
          s->n_exp = 2;
          s->w_exp[0] = 1.0 + 0.5 * d[0] / d[1];
          s->w_exp[1] = -0.5 * d[0] / d[1];
        } else if (exp == FALCON_EXP_AB3) {
          s->n_exp = 3;
          s->w_exp[1] = (d[0] * d[2] * 0.5 + (1.0 / 6.0) * d[0] * d[0]) / (d[1] * d[1] * 0.5 - d[1] * d[2]);
          s->w_exp[2] = (-d[0] * 0.5 - d[1] * s->w_exp[1]) * 0.5 / (d[2]);
          s->w_exp[0] = 1.0 - s->w_exp[1] - s->w_exp[2];
        } else return -1;
        return 0;
      case FALCON_IMP_BDF2: {
        if (exp != FALCON_EXP_AB2) return -1;
        const double r1 = d[1] / d[0], a0 = (2.0 + r1) / (1.0 + r1), a1 = 1.0 + 1.0 / r1;
        const double a2 = -1.0 * (1.0 / r1 / (1.0 + r1));
        s->n_imp = 2; s->n_exp = 2;
        s->wt_lhs = 1.0 / a0; s->w_imp[0] = a1 / a0; s->w_imp[1] = a2 / a0;
        s->w_exp[0] = (1.0 + 1.0 / r1) / a0; s->w_exp[1] = (-1.0 / r1) / a0;
        return 0;
      }
      case FALCON_IMP_BDF3: {
        if (exp != FALCON_EXP_AB3) return -1;
        const double r1 = d[1] / d[0], r2 = d[2] / d[0];
        const double a0 = (1.0 + 1.0 / (1.0 + r1) + 1.0 / (1.0 + r1 + r2));
        const double a1 = (((1.0 + r1) * (1.0 + r1 + r2)) / (r1 * (r1 + r2)));
        const double a2 = (-1.0 * (1.0 + r1 + r2) / (r1 * r2 * (1.0 + r1)));
        const double a3 = ((1.0 + r1) / (r2 * (r1 + r2) * (1.0 + r1 + r2)));
        const double b0 = 1.0 * ((1.0 + r1) * (1.0 + r1 + r2)) / (r1 * (r1 + r2));
        const double b1 = 1.0 * (-(1.0 + r1 + r2) / (r1 * r2));
        const double b2 = 1.0 * (1.0 + r1) / (r2 * (r1 + r2));
        s->n_imp = 3; s->n_exp = 3;
        s->wt_lhs = 1.0 / a0;
        s->w_imp[0] = a1 / a0; s->w_imp[1] = a2 / a0; s->w_imp[2] = a3 / a0;
        s->w_exp[0] = b0 / a0; s->w_exp[1] = b1 / a0; s->w_exp[2] = b2 / a0;
        return 0;
      }
      case FALCON_IMP_BDF4: {
        if (exp != FALCON_EXP_AB4) return -1;
        const double r1 = d[0] / d[1], r2 = d[1] / d[2], r3 = d[2] / d[3];
        const double c1 = 1.0 + r3 * (1.0 + r2), c2 = 1.0 + r2 * (1.0 + r1), c3 = 1.0 + r3 * c2;
        const double a0 = 1.0 + r1 / (1.0 + r1) + r2 * r1 / c2 + r3 * r2 * r1 / c3;
        const double a1 = -1.0 - r1 * (1.0 + r2 * (1.0 + r1) * (1.0 + r3 * c2 / c1) / (1.0 + r2));
        const double a2 = r1 * (r1 / (1.0 + r1) + r2 * r1 * (c3 + r3) / (1.0 + r3));
        const double a3 = -std::pow(r2, 3) * std::pow(r1, 2) * (1.0 + r1) / (1.0 + r2) * c3 / c2;
        const double a4 = (1.0 + r1) / (1.0 + r3) * c2 / c1 / c3 * (std::pow(r3, 4) * std::pow(r2, 3) * std::pow(r1, 2));
        const double b3 = -std::pow(r3, 3) * std::pow(r2, 2) * r1 * (1.0 + r1) / (1.0 + r3) * c2 / c1;
        const double b2 = std::pow(r2, 2) * r1 * (1.0 + r1) / (1.0 + r2) * c3;
        const double b1 = -c2 * c3 * r1 / (1.0 + r3);
        const double b0 = r2 * (1.0 + r1) / (1.0 + r2) * ((1.0 + r1) * (c3 + r3) + (1.0 + r3) / r2) / c1;
        s->n_imp = 4; s->n_exp = 4;
        s->wt_lhs = 1.0 / a0;
        s->w_imp[0] = -a1 / a0; s->w_imp[1] = -a2 / a0; s->w_imp[2] = -a3 / a0; s->w_imp[3] = -a4 / a0;
        s->w_exp[0] = b0 / a0; s->w_exp[1] = b1 / a0; s->w_exp[2] = b2 / a0; s->w_exp[3] = b3 / a0;
        return 0;
      }
      default: return -1;
    }
  }
}

// Scheme tables with dt_array(:) = dt (constant time step).
int scheme_weights(int type, int imp, int exp, Scheme* s) {
  s->type = type; s->imp = imp; s->exp = exp;
  if (type == FALCON_IMEX) {
    const double ones[4] = {1, 1, 1, 1};
    return imex_weights(imp, exp, ones, s);
  }
  if (type == FALCON_RK) {
    // butcher_a / butcher_b (src/timeschemes.F90:1701-1720); the implicit
    // tables stay zero.  RK4's a(2,3) = 1/2 of the reference is never read
    // (stage 2 sums i < 2) and is left out.
    if (imp != FALCON_IMP_NONE) return -1;
    if (exp == FALCON_EXP_RK2) {
      s->n_imp = s->n_exp = 2;
      s->aA[1][0] = 0.5;
      s->bA[0] = 0.0; s->bA[1] = 1.0;
    } else if (exp == FALCON_EXP_RK4) {
      s->n_imp = s->n_exp = 4;
      s->aA[1][0] = 0.5; s->aA[2][1] = 0.5; s->aA[3][2] = 1.0;
      s->bA[0] = 1.0 / 6.0; s->bA[1] = 1.0 / 3.0; s->bA[2] = 1.0 / 3.0; s->bA[3] = 1.0 / 6.0;
    } else {
      return -1;
    }
    return 0;
  }
  if (type == FALCON_IMEXRK) {
    // Butcher tables and the reference's ars_eqn_check / diag_diff /
    // diag_index flags (imexrk_tables.h).
    imexrk_table t;
    if (imexrk_table_get(imp, exp, &t) != 0 || t.n > kMaxStages) return -1;
    s->n_imp = s->n_exp = t.n;
    for (int i = 0; i < t.n; ++i) {
      for (int j = 0; j < t.n; ++j) { s->aD[i][j] = t.aD[i][j]; s->aA[i][j] = t.aA[i][j]; }
      s->bD[i] = t.bD[i]; s->bA[i] = t.bA[i];
    }
    s->check_D = t.check_D != 0; s->check_A = t.check_A != 0;
    s->diag_diff = t.diag_diff != 0;
    s->diag = t.diag_index - 1;
    return 0;
  }
  return -1;
}

// ---------------------------------------------------------------------------
// Azimuthal FFT plan (P = 3 Nm) and its device tables
// ---------------------------------------------------------------------------
}  // namespace

void falcon::fft_tables_host(const FftPlan& plan, double2* tw, int* pos) {
  const int P = plan.P;
  const double two_pi = 8.0 * std::atan(1.0);
  for (int i = 0; i < P; ++i) {
    pos[i] = fft_position(plan, i);
    const double a = two_pi * (double)i / (double)P;
    tw[i] = make_double2(std::cos(a), -std::sin(a));
  }
}

namespace {

struct FftTables {
  FftPlan plan{};
  double2* tw = nullptr;
  int* pos = nullptr;
  ~FftTables() { cudaFree(tw); cudaFree(pos); }
};

int make_fft(int P, std::unique_ptr<FftTables>* out) {
  auto f = std::make_unique<FftTables>();
  if (make_fft_plan(P, &f->plan) != 0)
    return fail(FALCON_EINVAL, "azimuthal length 3*Nm has a prime factor above 64 or too many factors");
  std::vector<int> pos(P);
  std::vector<double2> tw(P);
  fft_tables_host(f->plan, tw.data(), pos.data());
  int rc;
  if ((rc = upload(&f->tw, tw, nullptr))) return rc;
  if ((rc = upload(&f->pos, pos, nullptr))) return rc;
  *out = std::move(f);
  return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// Groups: instances sharing one operator set, stepped together
// ---------------------------------------------------------------------------
struct Group {
  falcon_params p{};           // parameters of the first instance (shared part)
  Scheme sch;
  int R = 0, M = 0, Nm = 0, P = 0, B = 0;
  std::shared_ptr<OpSet> ops;
  // IMEXRK with a stage-dependent implicit diagonal: the operators of each
  // stage whose diagonal differs from that of stage diag_index (null: ops)
  std::shared_ptr<OpSet> stage_ops[kMaxStages];
  std::unique_ptr<FftTables> fft;
  std::vector<int> members;    // batch indices
  std::vector<double> ra_pr_h; // per instance Ra/Pr
  std::vector<double> pr_h;    // per instance Pr
  // Pr enters only the temperature operator (AT, src/mat_assembly.F90), so
  // instances of one grid, dt and scheme that differ in Pr step together:
  // each run of equal Pr (a "sub", instance columns [b0, b1)) has its own
  // temperature solve, and every other kernel covers all of them.  Sub 0
  // takes its operators from ops / stage_ops; subs[k].ops for k >= 1.
  struct Sub {
    int b0 = 0, b1 = 0;
    std::shared_ptr<OpSet> ops;
    std::shared_ptr<OpSet> stage_ops[kMaxStages];
  };
  std::vector<Sub> subs;
  cudaStream_t stream = nullptr;
  // device state
  std::vector<void*> allocs;
  double2 *th[4] = {}, *wh[4] = {}, *nth[4] = {}, *nwh[4] = {};
  double *ubh[4] = {}, *uromh[4] = {};
  double2 *up = nullptr, *ur = nullptr, *psi = nullptr;
  double2 *ntp = nullptr, *ntr = nullptr, *nwp = nullptr, *nwr = nullptr, *dntr = nullptr, *dnwr = nullptr;
  double2 *lt = nullptr, *lw = nullptr, *lu0 = nullptr, *rhs_t = nullptr, *rhs_w = nullptr;
  double* ub = nullptr;        // 2R x 2B doubles (alias of ub2)
  double2* ub2 = nullptr;
  double* ra_pr = nullptr;
  double* inv_pr = nullptr;    // [b] 1/Pr
  double2 *fat[kMaxStages] = {}, *fdt[kMaxStages] = {}, *faw[kMaxStages] = {}, *fdw[kMaxStages] = {},
          *buo[kMaxStages] = {};
  double2 *t0 = nullptr, *w0 = nullptr;
  double* u0 = nullptr;
  double* us = nullptr;        // explicit RK: stage uphi_bar (R x B)
  double2* t_grid = nullptr;   // temperature seen by the last nonlinear pass (IMEXRK)
  double* up0_prev = nullptr;  // [r][b] Re u_phi(m = 0) at the start of the step (upFR_prev)
  double* spec_dev = nullptr;  // [2][b][m] KE and temperature spectra
  double* ubal_dev = nullptr;  // [b][r][3] u_phi balance
  double2* d1up = nullptr;     // d(u_phi)/dr of every mode (made on the first balance request)
  double* diag_dev = nullptr;  // 8 per instance
  double* diag_part = nullptr;  // 8 R per instance: diagnostics partial sums
  std::vector<double> diag_host;
  double2* stage_buf = nullptr;  // host staging (pinned) for one instance
  Prof* prof = nullptr;
  int head = 0, head_e = 0;
  int n_step = 0;
  double tot_time = 0.0;
  size_t bytes = 0;
  // Steady-state steps replayed as CUDA graphs, one per ring-buffer phase
  // (the kernel arguments of a step depend only on the history heads).
  struct StepGraph { int phase; cudaGraphExec_t exec; long long kernels; };
  std::vector<StepGraph> graphs;
  bool own_stream = false;
  cudaEvent_t done = nullptr;  // joins the group's stream back to its batch's stream
  // Variable time step (l_vartimestep, one instance per group): the dt
  // history dt_array(1..4), the current dt, the per-line velocity maxima of
  // the last nonlinear pass, and the grid spacing for get_dtvals.
  bool vardt = false;
  // restored from a checkpoint: the operators are rebuilt for the restored
  // dt at the next step, and (IMEXRK, RK) the velocity maxima of the restored
  // state are taken by an extra nonlinear pass before compute_new_dt
  bool force_rebuild = false;
  bool need_cfl_pass = false;
  bool restart_first = false;  // the next step is the first after a restart (l_restart)
  // Slice planes of the X operand of the tensor-core contractions, and the
  // operand they hold (reused while it is unchanged).
  uint16_t* oz_xs = nullptr;
  int* oz_cexp = nullptr;
  size_t oz_xs_cap = 0, oz_cexp_cap = 0;
  struct { const double* X = nullptr; long ldx = 0, sX = 0; int K = 0, N = 0, batch = 0, w = 0; bool valid = false; } oz_key;
  double dt_array[4] = {0, 0, 0, 0};
  double dt_new = 0.0;
  double* umax = nullptr;
  std::vector<double> umax_h, dr_h, radius_h;
  std::vector<double> spec_host, ubal_host;
  double cur_dt() const { return vardt ? dt_new : p.dt; }

  // The next step runs uncaptured (its contraction shapes may be new to
  // the autotuner, which measures only outside capture): set when the
  // captured steps are dropped.
  bool direct_next = false;
  void drop_graphs() {
    // a step launched from one of these graphs may still run on the stream
    if (stream && !graphs.empty()) cudaStreamSynchronize(stream);
    for (auto& sg : graphs) cudaGraphExecDestroy(sg.exec);
    graphs.clear();
    direct_next = true;
  }
  ~Group() {
    // work queued on the stream may still read or write the arrays
    if (stream) cudaStreamSynchronize(stream);
    drop_graphs();
    cudaFree(oz_xs);
    cudaFree(oz_cexp);
    for (void* q : allocs) cudaFree(q);
    if (stage_buf) cudaFreeHost(stage_buf);
    if (done) cudaEventDestroy(done);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
  size_t nel() const { return (size_t)R * M * B; }
  // Every per-instance array is [rows][B] elements of `ew` doubles; the
  // registry lets the serving loop repack instance columns when members
  // join or leave.
  struct Field { void** ptr; size_t rows; int ew; };
  std::vector<Field> fields;
  template <class T>
  int alloc(T** q, size_t n) {
    CK(cudaMalloc(q, sizeof(T) * (n ? n : 1)));
    // on the group's stream: its kernels (on a non-blocking stream) would
    // not wait for a legacy-stream memset
    CK(cudaMemsetAsync(*q, 0, sizeof(T) * (n ? n : 1), stream));
    allocs.push_back(*q);
    bytes += sizeof(T) * n;
    const int ew = (int)(sizeof(T) / sizeof(double));
    fields.push_back(Field{reinterpret_cast<void**>(q), n / (size_t)std::max(B, 1), ew});
    return 0;
  }
  double2* T() const { return th[head]; }
  double2* W() const { return wh[head]; }
};

namespace {

OpKey key_of(const falcon_params& p, const Scheme& s) {
  OpKey k{};
  k.R = p.nr_max; k.Nm = p.nm_max; k.mbc = p.mbc; k.type = p.scheme_type;
  k.imp = p.scheme_imp; k.exp = p.scheme_exp; k.dt = p.dt; k.pr = p.pr; k.eta = p.eta;
  k.wt = (p.scheme_type == FALCON_IMEX) ? s.wt_lhs : s.aD[s.diag][s.diag];
  k.needs_lap = (p.scheme_type == FALCON_RK || (p.scheme_type == FALCON_IMEXRK && !(s.check_A && s.check_D))) ? 1 : 0;
  k.lagpts = k.needs_lap ? p.lagpts : 0;
  return k;
}

int validate(const falcon_params& p) {
  if (p.nr_max < 4 || p.nr_max > 257) return fail(FALCON_EINVAL, "Nr_max must be in [4, 257]");
  if (p.nm_max < 1 || p.nm_max > 4096) return fail(FALCON_EINVAL, "Nm_max must be in [1, 4096]");
  if (!(p.eta > 0.0 && p.eta < 1.0)) return fail(FALCON_EINVAL, "eta must be in (0,1)");
  if (!(p.dt > 0.0) || !std::isfinite(p.dt)) return fail(FALCON_EINVAL, "dt must be positive");
  if (!(p.pr > 0.0)) return fail(FALCON_EINVAL, "Pr must be positive");
  if (p.mbc != 0 && p.mbc != 1) return fail(FALCON_EINVAL, "mBC must be NS or SF");
  if (p.l_vartimestep && !(p.cfl > 0.0 && p.dt_coef > 0.0 && p.dt_max > 0.0))
    return fail(FALCON_EINVAL, "l_vartimestep needs CFL, dt_coef and dt_max > 0");
  Scheme s;
  if (scheme_weights(p.scheme_type, p.scheme_imp, p.scheme_exp, &s) != 0)
    return fail(FALCON_EINVAL, "unsupported time scheme combination");
  // With diag_diff a stage solves with its own weight butcher_aD(st,st).  A
  // zero weight leaves the coupled omega-psi operator of mat_build_IRK
  // (src/mat_assembly.F90:131-160) singular: the omega wall coefficients
  // enter no row.  The reference factorises it regardless and its run
  // diverges in the first step (LZ3A4a, stages 2 and 4); refused here.
  if (p.scheme_type == FALCON_IMEXRK && s.diag_diff)
    for (int st = 1; st < s.n_exp; ++st)
      if (s.aD[st][st] == 0.0)
        return fail(FALCON_EINVAL, "IMEXRK scheme with a zero implicit diagonal at a stage (LZ3A4a): the reference's "
                                   "coupled omega-psi operator for that stage is singular");
  return 0;
}

// Scratch for the slice planes of the largest X operand of the group's
// contractions (allocated when the group is set up, before any capture).
int oz_scratch_init(Group* g) {
  const int R = g->R, M = g->M, B = g->B;
  const long KP = ((R + 15) / 16) * 16;
  auto np = [](long n) { return ((n + 31) / 32) * 32; };
  const long cols = std::max(np(2L * M * B), (long)M * np(2L * B));
  g->oz_xs_cap = (size_t)kOzS * KP * cols;
  g->oz_cexp_cap = (size_t)cols;
  CK(cudaMalloc(&g->oz_xs, g->oz_xs_cap * sizeof(uint16_t)));
  CK(cudaMalloc(&g->oz_cexp, g->oz_cexp_cap * sizeof(int)));
  g->bytes += g->oz_xs_cap * sizeof(uint16_t) + g->oz_cexp_cap * sizeof(int);
  return 0;
}

// Operators of the IMEXRK stages whose implicit diagonal differs from that
// of stage diag_index (diag_diff, src/fourierloop_imexrk.F90:134-160),
// built with the weight butcher_aD(rk_stage,rk_stage) at time step dt.
// Stages with equal diagonals share one set through the operator cache;
// LAPpsi comes from the main set.
int build_stage_ops_for(const Group* g, double pr, double dt, std::shared_ptr<OpSet> (&out)[kMaxStages]) {
  const Scheme& sc = g->sch;
  for (auto& so : out) so.reset();
  if (g->p.scheme_type != FALCON_IMEXRK || !sc.diag_diff) return 0;
  for (int st = 1; st < sc.n_exp; ++st) {
    if (sc.aD[st][st] == sc.aD[sc.diag][sc.diag]) continue;
    OpKey k = key_of(g->p, sc);
    k.pr = pr; k.dt = dt; k.wt = sc.aD[st][st]; k.needs_lap = 0; k.lagpts = 0;
    const int rc = build_opset(k, &out[st]);
    if (rc) return rc;
  }
  return 0;
}

int build_stage_ops(Group* g, double dt) {
  int rc = build_stage_ops_for(g, g->p.pr, dt, g->stage_ops);
  for (size_t k = 1; k < g->subs.size() && !rc; ++k)
    rc = build_stage_ops_for(g, g->pr_h[g->subs[k].b0], dt, g->subs[k].stage_ops);
  return rc;
}

// Operators of sub k (stage st of an IMEXRK step with stage-dependent
// diagonal, or -1): its temperature solve; the Pr-free operators of sub 0
// serve every sub.
const OpSet* sub_ops(const Group* g, int k, int st) {
  if (k == 0) return (st >= 0 && g->stage_ops[st]) ? g->stage_ops[st].get() : g->ops.get();
  const Group::Sub& u = g->subs[k];
  return (st >= 0 && u.stage_ops[st]) ? u.stage_ops[st].get() : u.ops.get();
}

// Subs of a group from its instances' Pr (runs of equal Pr).
void make_subs(Group* g) {
  g->subs.clear();
  for (int b = 0; b < g->B; ++b)
    if (b == 0 || g->pr_h[b] != g->pr_h[b - 1]) {
      if (!g->subs.empty()) g->subs.back().b1 = b;
      g->subs.push_back(Group::Sub{});
      g->subs.back().b0 = b;
    }
  if (!g->subs.empty()) g->subs.back().b1 = g->B;
}

// Per-instance Ra/Pr and 1/Pr of the group's columns, uploaded.
int upload_instance_params(Group* g) {
  const int B = g->B;
  std::vector<double> ip(B);
  for (int b = 0; b < B; ++b) ip[b] = 1.0 / g->pr_h[b];
  // stream-ordered before the group's kernels (a legacy-stream copy from
  // pageable memory may land after a kernel of a non-blocking stream read it)
  CK(cudaMemcpyAsync(g->ra_pr, g->ra_pr_h.data(), sizeof(double) * B, cudaMemcpyHostToDevice, g->stream));
  CK(cudaMemcpyAsync(g->inv_pr, ip.data(), sizeof(double) * B, cudaMemcpyHostToDevice, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  return 0;
}

// After the members of a group changed (serving): its subs from the
// instances' Pr, and the operator sets of each (built or taken from the
// operator cache).  The group's parameters take the Pr of its first column.
int group_refresh_subs(Group* g) {
  make_subs(g);
  if (g->B == 0) return 0;
  int rc;
  if (g->pr_h[0] != g->p.pr) {
    g->p.pr = g->pr_h[0];
    if ((rc = build_opset(key_of(g->p, g->sch), &g->ops))) return rc;
  }
  for (size_t k = 1; k < g->subs.size(); ++k) {
    falcon_params q = g->p;
    q.pr = g->pr_h[g->subs[k].b0];
    if ((rc = build_opset(key_of(q, g->sch), &g->subs[k].ops))) return rc;
  }
  if ((rc = build_stage_ops(g, g->p.dt))) return rc;
  g->drop_graphs();
  return 0;
}

int group_init(Group* g, const std::vector<falcon_params>& ps, const std::vector<int>& members) {
  g->p = ps[members[0]];
  g->members = members;
  g->R = g->p.nr_max; g->Nm = g->p.nm_max; g->M = g->Nm + 1; g->P = 3 * g->Nm;
  g->B = (int)members.size();
  if (scheme_weights(g->p.scheme_type, g->p.scheme_imp, g->p.scheme_exp, &g->sch) != 0)
    return fail(FALCON_EINVAL, "unsupported scheme");
  g->ra_pr_h.resize(g->B);
  g->pr_h.resize(g->B);
  for (int i = 0; i < g->B; ++i) {
    g->ra_pr_h[i] = ps[members[i]].ra / ps[members[i]].pr;
    g->pr_h[i] = ps[members[i]].pr;
  }
  make_subs(g);
  int rc;
  if ((rc = build_opset(key_of(g->p, g->sch), &g->ops))) return rc;
  for (size_t k = 1; k < g->subs.size(); ++k)
    if ((rc = build_opset(key_of(ps[members[g->subs[k].b0]], g->sch), &g->subs[k].ops))) return rc;
  if ((rc = build_stage_ops(g, g->p.dt))) return rc;
  if ((rc = make_fft(g->P, &g->fft))) return rc;
  if ((rc = oz_scratch_init(g))) return rc;
  const size_t n = g->nel();
  const int R = g->R, B = g->B;
  if (g->p.scheme_type == FALCON_IMEX) {
    for (int i = 0; i < g->sch.n_imp; ++i) {
      if ((rc = g->alloc(&g->th[i], n)) || (rc = g->alloc(&g->wh[i], n)) ||
          (rc = g->alloc(&g->ubh[i], (size_t)R * B)))
        return rc;
    }
    for (int i = 0; i < g->sch.n_exp; ++i) {
      if ((rc = g->alloc(&g->nth[i], n)) || (rc = g->alloc(&g->nwh[i], n)) ||
          (rc = g->alloc(&g->uromh[i], (size_t)R * B)))
        return rc;
    }
  } else if (g->p.scheme_type == FALCON_RK) {
    // explicit RK: one right-hand side per stage for T and for omega (with
    // uphi_bar in the m = 0 column), the stage uphi_bar
    if ((rc = g->alloc(&g->th[0], n)) || (rc = g->alloc(&g->wh[0], n)) || (rc = g->alloc(&g->us, (size_t)R * B)))
      return rc;
    for (int i = 0; i < g->sch.n_exp; ++i)
      if ((rc = g->alloc(&g->fat[i], n)) || (rc = g->alloc(&g->faw[i], n))) return rc;
    if ((rc = g->alloc(&g->t0, n)) || (rc = g->alloc(&g->w0, n)) || (rc = g->alloc(&g->u0, (size_t)R * B)) ||
        (rc = g->alloc(&g->t_grid, n)))
      return rc;
  } else {
    if ((rc = g->alloc(&g->th[0], n)) || (rc = g->alloc(&g->wh[0], n))) return rc;
    for (int i = 0; i < g->sch.n_exp; ++i) {
      if ((rc = g->alloc(&g->fat[i], n)) || (rc = g->alloc(&g->fdt[i], n)) || (rc = g->alloc(&g->faw[i], n)) ||
          (rc = g->alloc(&g->fdw[i], n)) || (rc = g->alloc(&g->buo[i], n)))
        return rc;
    }
    if ((rc = g->alloc(&g->t0, n)) || (rc = g->alloc(&g->w0, n)) || (rc = g->alloc(&g->u0, (size_t)R * B)) ||
        (rc = g->alloc(&g->t_grid, n)))
      return rc;
  }
  if ((rc = g->alloc(&g->up, n)) || (rc = g->alloc(&g->ur, n)) || (rc = g->alloc(&g->psi, n)) ||
      (rc = g->alloc(&g->ntp, n)) || (rc = g->alloc(&g->ntr, n)) || (rc = g->alloc(&g->nwp, n)) ||
      (rc = g->alloc(&g->nwr, n)) || (rc = g->alloc(&g->dntr, n)) || (rc = g->alloc(&g->dnwr, n)) ||
      (rc = g->alloc(&g->lt, n)) || (rc = g->alloc(&g->lw, n)) || (rc = g->alloc(&g->lu0, (size_t)R * B)) ||
      (rc = g->alloc(&g->rhs_t, n)) || (rc = g->alloc(&g->rhs_w, n)) ||
      (rc = g->alloc(&g->ub2, (size_t)2 * R * B)) || (rc = g->alloc(&g->ra_pr, (size_t)B)) ||
      (rc = g->alloc(&g->inv_pr, (size_t)B)) ||
      (rc = g->alloc(&g->diag_dev, (size_t)8 * B)) || (rc = g->alloc(&g->diag_part, (size_t)8 * R * B)) ||
      (rc = g->alloc(&g->up0_prev, (size_t)R * B)) || (rc = g->alloc(&g->spec_dev, (size_t)2 * g->M * B)) ||
      (rc = g->alloc(&g->ubal_dev, (size_t)3 * R * B)))
    return rc;
  g->ub = reinterpret_cast<double*>(g->ub2);
  if (g->p.l_vartimestep) {
    if (B != 1) return fail(FALCON_EINVAL, "a variable-dt group holds one instance");
    g->vardt = true;
    if ((rc = g->alloc(&g->umax, (size_t)2 * R * B))) return rc;
    g->umax_h.resize((size_t)2 * R);
    Cheb c = make_cheb(R, g->p.eta);
    g->dr_h = c.dr;
    g->radius_h = c.radius;
    for (int i = 0; i < 4; ++i) g->dt_array[i] = g->p.dt;
    g->dt_new = g->p.dt;
  }
  if ((rc = upload_instance_params(g))) return rc;
  CK(cudaMallocHost(&g->stage_buf, sizeof(double2) * (size_t)g->M * R * 2));
  return 0;
}

// Radial GEMM over all modes and instances: Y = A (R x R) * X (R x 2MB).
GemmArgs radial(const double* A, const double2* X, double2* Y, int R, int M, int B) {
  GemmArgs g{};
  g.A = A; g.lda = R;
  g.X = reinterpret_cast<const double*>(X); g.ldx = 2L * M * B;
  g.Y = reinterpret_cast<double*>(Y); g.ldy = 2L * M * B;
  g.K = R; g.rows = R; g.N = 2 * M * B; g.batch = 1; g.alpha = 1.0;
  return g;
}

// Per-mode GEMM over modes [m0, m0+nm): Y[:, m, :] = A_m(rows x R) X[:, m, :].
GemmArgs per_mode(const double* A, long lda, long sA, const double2* X, double2* Y, int R, int M, int B,
                  int m0, int nm, int rows) {
  GemmArgs g{};
  g.A = A + (size_t)m0 * sA; g.lda = lda; g.sA = sA;
  g.X = reinterpret_cast<const double*>(X) + 2L * m0 * B; g.ldx = 2L * M * B; g.sX = 2L * B;
  g.Y = reinterpret_cast<double*>(Y) + 2L * m0 * B; g.ldy = 2L * M * B; g.sY = 2L * B;
  g.K = R; g.rows = rows; g.N = 2 * B; g.batch = nm; g.alpha = 1.0;
  return g;
}

// Every kernel launch of a step goes through here: counted, and timed with
// events on the group's stream when profiling.
template <class F>
int launch(Group* g, int cls, double flops, F f) {
  cudaEvent_t a = nullptr, b = nullptr;
  if (g->prof) {
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, g->stream));
  }
  cudaError_t e = f();
  if (e != cudaSuccess)
    return fail(FALCON_ECUDA, std::string("kernel launch (") + kClassNames[cls] + "): " + cudaGetErrorString(e));
  g_launches++;
  if (g->prof) {
    CK(cudaEventRecord(b, g->stream));
    g->prof->recs.push_back({cls, a, b, flops});
  }
  return 0;
}

double gemm_flops(const GemmArgs& q) { return 2.0 * q.rows * (double)q.K * q.N * q.batch; }

// The slice view of q.A when it lies in an operator of the group's sets
// and q walks that operator with its own leading dimension and stride.
bool attach_oz(const OpSet* o, GemmArgs* q) {
  if (!o) return false;
  for (const auto& z : o->oz) {
    const long span = (z.nb > 1) ? z.nb * z.sA : z.lda * z.K;
    const long delta = q->A - z.base;
    if (delta < 0 || delta >= span) continue;
    const long z0 = (z.nb > 1) ? delta / z.sA : 0;
    const long row0 = delta - z0 * z.sA;
    if (q->lda != z.lda || q->K != z.K || row0 >= z.lda || row0 + q->rows > z.rows) return false;
    if (q->batch > 1 && (q->sA != z.sA || z0 + q->batch > z.nb)) return false;
    q->oz_s = z.s + (size_t)z0 * oz_slices(z.w) * z.rowsP * z.KP;
    q->oz_ex = z.ex + (size_t)z0 * z.rowsP;
    q->oz_sz = (long)oz_slices(z.w) * z.rowsP * z.KP;
    q->oz_w = z.w;
    q->oz_rowsP = z.rowsP;
    q->oz_KP = z.KP;
    q->oz_row0 = (int)row0;
    q->oz_tmap = z.tmap_ok ? &z.tmap : nullptr;
    q->oz_z0 = (int)z0;
    return true;
  }
  return false;
}

// The slice view of q.A in any operator set of the group (its subs' and
// their stages' included).
bool attach_group(const Group* g, GemmArgs* q) {
  for (size_t k = 0; k < std::max<size_t>(g->subs.size(), 1); ++k) {
    if (k > 0 && attach_oz(g->subs[k].ops.get(), q)) return true;
    if (k == 0 && attach_oz(g->ops.get(), q)) return true;
    for (int st = 0; st < kMaxStages; ++st) {
      const OpSet* o = k == 0 ? g->stage_ops[st].get() : g->subs[k].stage_ops[st].get();
      if (attach_oz(o, q)) return true;
    }
  }
  return false;
}

// Contractions that take the tcgen05 kernel: at least two of its
// 128 x 24 tiles per SM.  Smaller ones (one instance, small groups) are
// faster on the mma.sync kernel that slices its own X columns, whose
// per-launch cost is lower; both give the same bits.
bool tc_worth_it(const GemmArgs& q) {
  static std::atomic<int> nsm{0};
  int n = nsm.load();
  if (n == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      n = 152;
    nsm.store(n);
  }
  const long tiles = (long)q.batch * ((q.rows + kTcBM - 1) / kTcBM) * ((q.N + kTcBN - 1) / kTcBN);
  return tiles >= 2L * n;
}

// The tcgen05 contraction of one GEMM with an attached slice view.
TcArgs tc_args(const GemmArgs& q) {
  TcArgs t{};
  t.X = q.X; t.ldx = q.ldx; t.sX = q.sX;
  t.K = q.K; t.KP = q.oz_KP; t.N = q.N; t.batch = q.batch; t.rows = q.rows; t.w = q.oz_w;
  t.nout = 1; t.rend[0] = q.rows; t.Y[0] = q.Y; t.ldy = q.ldy; t.sY = q.sY;
  t.alpha = q.alpha;
  t.aex = q.oz_ex + q.oz_row0; t.rowsP = q.oz_rowsP;
  t.row0 = q.oz_row0; t.z0 = q.oz_z0;
  return t;
}

// ---------------------------------------------------------------------------
// Contraction paths and their autotuner.  A contraction with an attached
// slice view can run as FP64 FMA tiles (PATH_FMA), on the mma.sync slice
// kernel (PATH_MMA; X sliced in the kernel, or into slice planes first) or on
// the tcgen05 kernel (PATH_TC).  PATH_MMA and PATH_TC give the same bits;
// PATH_FMA differs from them by rounding (all are FP64-accurate).
// ---------------------------------------------------------------------------
// PATH_FMA16/32/64: the FMA tiles with the best tile shape of that column
// width (the same bits as PATH_FMA, whose shape a cost model picks).
enum { PATH_FMA = 0, PATH_MMA = 1, PATH_TC = 2, PATH_FMA16 = 3, PATH_FMA32 = 4, PATH_FMA64 = 5, PATH_COUNT = 6 };
inline bool is_fma_path(int p) { return p == PATH_FMA || p >= PATH_FMA16; }

// Slice planes of q.X for the mma.sync kernel when it does not slice X
// itself (made unless `reuse` finds them already made for the same X).
// false: they do not fit the group's scratch (the FMA tiles then run).
int mma_planes(Group* g, GemmArgs* q, bool reuse, bool* fits) {
  *fits = true;
  if (oz_fused_x(q->rows, q->N, q->batch)) return 0;
  const int KP = q->oz_KP, Np = (int)(((long)q->N + 31) / 32 * 32);
  if ((size_t)oz_slices(q->oz_w) * KP * Np * q->batch > g->oz_xs_cap || (size_t)Np * q->batch > g->oz_cexp_cap) {
    *fits = false;
    return 0;
  }
  auto& k = g->oz_key;
  const bool same = reuse && k.valid && k.X == q->X && k.ldx == q->ldx && k.sX == q->sX && k.K == q->K &&
                    k.N == q->N && k.batch == q->batch && k.w == q->oz_w;
  if (!same) {
    int rc = launch(g, KC_ELEMENTWISE, 0.0, [&]() {
      return launch_oz_slice_cols(q->X, q->ldx, q->sX, q->K, q->N, q->batch, g->oz_xs, g->oz_cexp, KP, Np, q->oz_w,
                                  g->stream);
    });
    if (rc) return rc;
    k.X = q->X; k.ldx = q->ldx; k.sX = q->sX; k.K = q->K; k.N = q->N; k.batch = q->batch; k.w = q->oz_w;
    k.valid = true;
  }
  q->oz_xs = g->oz_xs;
  q->oz_cexp = g->oz_cexp;
  q->oz_Np = Np;
  return 0;
}

// One contraction on the given path (q carries its slice view for MMA/TC).
int run_path_once(Group* g, int cls, GemmArgs q, int path, bool reuse);
int run_path(Group* g, int cls, GemmArgs q, int path, bool reuse) {
  const int rc = run_path_once(g, cls, q, path, reuse);
  if (rc == FALCON_ECUDA)  // the shape and path of the failed contraction
    g_err += " [contraction path " + std::to_string(path) + ": rows " + std::to_string(q.rows) + ", K " +
             std::to_string(q.K) + ", N " + std::to_string(q.N) + ", batch " + std::to_string(q.batch) + ", w " +
             std::to_string(q.oz_w) + ", group of " + std::to_string(g->B) + " at Nr " + std::to_string(g->R) +
             ", Nm " + std::to_string(g->Nm) + "]";
  return rc;
}
int run_path_once(Group* g, int cls, GemmArgs q, int path, bool reuse) {
  if (path == PATH_TC) {
    const TcArgs t = tc_args(q);
    const CUtensorMap* map = static_cast<const CUtensorMap*>(q.oz_tmap);
    return launch(g, cls, gemm_flops(q), [&]() { return launch_tc_gemm(t, *map, g->stream); });
  }
  if (path == PATH_MMA) {
    bool fits = true;
    int rc = mma_planes(g, &q, reuse, &fits);
    if (rc) return rc;
    if (!fits) path = PATH_FMA;
  }
  if (is_fma_path(path)) {
    q.oz_s = nullptr;
    q.oz_xs = nullptr;
    q.fma_ncol = path == PATH_FMA16 ? 16 : path == PATH_FMA32 ? 32 : path == PATH_FMA64 ? 64 : 0;
  }
  return launch(g, cls, gemm_flops(q), [&]() { return launch_gemm(q, g->stream); });
}

// The autotuner's decisions, per device and contraction shape: the path
// measured fastest the first time the shape ran (outside graph capture),
// kept for the process and, with a cache file, across processes.  Cache file
// (text): a header line "falcon-contraction-tuning 2", then one decision per
// line:
//   <device> <rows> <K> <N> <batch> <w> <per_mode> <reuse> <path> <us_0> ... <us_5>
// device = the CUDA device name with blanks as '_' and "_sm<SM count>";
// per_mode = 1 when the batch entries have their own X (sX != 0); reuse = 1
// when X's slice planes were made by the contraction before; w = the slice
// format (6 or 7); path 0 FMA (cost-model tile shape), 1 mma.sync, 2
// tcgen05, 3/4/5 FMA with tiles of 16/32/64 columns; us_p = the measured
// microseconds per contraction on path p (-1: not measured).
struct TuneKey {
  std::string dev;
  int rows, K, N, batch, w, per_mode, reuse;
  bool operator<(const TuneKey& o) const {
    return std::tie(dev, rows, K, N, batch, w, per_mode, reuse) <
           std::tie(o.dev, o.rows, o.K, o.N, o.batch, o.w, o.per_mode, o.reuse);
  }
};
struct TuneEntry { int path; float us[PATH_COUNT]; };
std::mutex g_tune_mu;
std::map<TuneKey, TuneEntry> g_tune;
std::string g_tune_path;          // cache file ("" none)
bool g_tune_env_checked = false;
std::atomic<long long> g_tune_measured(0);
constexpr const char* kTuneHeader = "falcon-contraction-tuning 2";

int tune_load_locked(const std::string& path) {
  std::ifstream f(path);
  if (!f) return 0;  // no file yet: it is created with the first decision
  std::string line;
  if (!std::getline(f, line) || line != kTuneHeader)
    return fail(FALCON_EINVAL, "tuning cache " + path + ": not a falcon contraction tuning file (header)");
  int n = 0;
  while (std::getline(f, line)) {
    if (line.empty() || line[0] == '#') continue;
    std::istringstream is(line);
    TuneKey k;
    TuneEntry e;
    bool good = (bool)(is >> k.dev >> k.rows >> k.K >> k.N >> k.batch >> k.w >> k.per_mode >> k.reuse >> e.path);
    for (int p = 0; p < PATH_COUNT && good; ++p) good = (bool)(is >> e.us[p]);
    if (!good || e.path < 0 || e.path >= PATH_COUNT || k.rows <= 0 || k.K <= 0 || k.N <= 0 || k.batch <= 0)
      return fail(FALCON_EINVAL, "tuning cache " + path + ": malformed line " + std::to_string(n + 2));
    g_tune[k] = e;
    ++n;
  }
  return 0;
}

void tune_store_locked(const TuneKey& k, const TuneEntry& e) {
  if (g_tune_path.empty()) return;
  std::FILE* f = std::fopen(g_tune_path.c_str(), "a+");
  if (!f) return;
  std::fseek(f, 0, SEEK_END);
  if (std::ftell(f) == 0) std::fprintf(f, "%s\n", kTuneHeader);
  std::fprintf(f, "%s %d %d %d %d %d %d %d %d", k.dev.c_str(), k.rows, k.K, k.N, k.batch, k.w, k.per_mode, k.reuse,
               e.path);
  for (int p = 0; p < PATH_COUNT; ++p) std::fprintf(f, " %.3f", e.us[p]);
  std::fprintf(f, "\n");
  std::fclose(f);
}

const std::string& device_tag() {
  static std::mutex mu;
  static std::map<int, std::string> tags;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  auto it = tags.find(dev);
  if (it != tags.end()) return it->second;
  cudaDeviceProp pr{};
  std::string t = cudaGetDeviceProperties(&pr, dev) == cudaSuccess ? std::string(pr.name) : std::string("device");
  for (auto& ch : t)
    if (std::isspace((unsigned char)ch)) ch = '_';
  t += "_sm" + std::to_string(pr.multiProcessorCount);
  return tags[dev] = t;
}

bool spans_overlap(const double* a, long na, const double* b, long nb) {
  const double *a1 = a + na, *b1 = b + nb;
  return a < b1 && b < a1;
}

// Extent in doubles of an operand addressed as base[k*ld + n + z*sz].
long operand_span(long ld, long sz, int K, int N, int batch) {
  return (long)(K - 1) * ld + N + (long)(batch - 1) * sz;
}

// A device buffer larger than L2 (129 MB on GB300), written before each
// timed run of the tuner: in a step the operators and operands of a
// contraction come from HBM (the step's working set is larger than L2), so
// the candidates are timed with a cold L2 too.  One per device, kept for
// the process.
constexpr size_t kTuneFlushBytes = (size_t)256 << 20;
void* tune_flush_buffer() {
  static std::mutex mu;
  static std::map<int, void*> bufs;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  void*& b = bufs[dev];
  if (!b && cudaMalloc(&b, kTuneFlushBytes) != cudaSuccess) b = nullptr;
  return b;
}

// The fastest of three timed runs of `run` (after one untimed run), each
// after a write of the flush buffer that evicts L2, timed by CUDA events on
// the group's stream: microseconds in *us.
int time_fastest(Group* g, void* flush, cudaEvent_t a, cudaEvent_t b, const std::function<int()>& run, float* us) {
  int rc = run();
  if (rc) return rc;
  float fastest = 0.f;
  for (int r = 0; r < 3; ++r) {
    float ms = 0.f;
    if (cudaMemsetAsync(flush, r + 1, kTuneFlushBytes, g->stream) != cudaSuccess ||
        cudaEventRecord(a, g->stream) != cudaSuccess)
      return fail(FALCON_ECUDA, "tuning: flush or event");
    if ((rc = run())) return rc;
    if (cudaEventRecord(b, g->stream) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
        cudaEventElapsedTime(&ms, a, b) != cudaSuccess)
      return fail(FALCON_ECUDA, "tuning timing");
    if (r == 0 || ms < fastest) fastest = ms;
  }
  *us = fastest * 1000.f;
  return 0;
}

// The path of a contraction under mode 4: the cached decision, or a
// measurement of every available path (each run once to warm up, then three
// times with L2 flushed before each, timed by CUDA events on the group's
// stream with the device otherwise idle; the fastest of the three counts),
// keeping the fixed rule's path unless another is at least 10 % faster.
// Shapes met inside graph capture or profiling, or whose output overlaps
// X, are not measured: they take the fixed rule of mode 2.
int tuned_path(Group* g, int cls, const GemmArgs& q, bool reuse, bool tc_ok, int fixed, int* path) {
  *path = fixed;
  TuneKey k{device_tag(), q.rows, q.K, q.N, q.batch, q.oz_w, q.sX != 0 ? 1 : 0, reuse ? 1 : 0};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    if (!g_tune_env_checked) {
      g_tune_env_checked = true;
      const char* env = std::getenv("FALCON_TUNE_CACHE");
      if (g_tune_path.empty() && env && *env) {
        g_tune_path = env;
        int rc = tune_load_locked(g_tune_path);
        if (rc) return rc;
      }
    }
    auto it = g_tune.find(k);
    if (it != g_tune.end()) {
      *path = it->second.path;
      if (*path == PATH_TC && !tc_ok) *path = PATH_MMA;
      return 0;
    }
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(g->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone || g->prof) return 0;
  const long xs = operand_span(q.ldx, q.sX, q.K, q.N, q.batch), ys = operand_span(q.ldy, q.sY, q.rows, q.N, q.batch);
  if (spans_overlap(q.X, xs, q.Y, ys)) return 0;
  TuneEntry e{};
  void* flush = tune_flush_buffer();
  if (!flush) return fail(FALCON_ENOMEM, "contraction tuning: no device memory for the L2 flush buffer");
  CK(cudaDeviceSynchronize());
  cudaEvent_t a = nullptr, b = nullptr;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  float best = 0.f;
  int rc = 0;
  for (int p = 0; p < PATH_COUNT && !rc; ++p) {
    e.us[p] = -1.f;
    if (p == PATH_TC && !tc_ok) continue;
    if (p >= PATH_FMA16 && q.N <= 8) continue;  // one-warp GEMV, no tile shapes
    if ((rc = time_fastest(g, flush, a, b, [&]() { return run_path(g, cls, q, p, reuse); }, &e.us[p]))) break;
    if (p == PATH_FMA || e.us[p] < best) {
      best = e.us[p];
      e.path = p;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  // the fixed rule's path unless another is at least 10 % faster: a
  // contraction inside a step pays launch and dependency costs that the
  // isolated timing does not see, so near-ties keep the rule's choice
  if (e.path != fixed && e.us[fixed] >= 0.f && e.us[fixed] <= 1.1f * e.us[e.path]) e.path = fixed;
  g_tune_measured++;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[k] = e;
  tune_store_locked(k, e);
  *path = e.path;
  return 0;
}

// reuse: the call follows a contraction with the same X operand, unchanged
// since (the blocks of one operator applied to one right-hand side); its
// slice planes are reused when they match.
//
// Modes: 0 FP64 FMA tiles; 1 mma.sync for every contraction with a slice
// view; 2 fixed rules: tcgen05 for contractions that fill the GPU (at least
// two 128 x 24 tiles per SM), mma.sync for the other ones of at least 16
// columns per batch entry, FMA for narrower ones (the per-mode solves of
// groups of up to 7 instances); 3 tcgen05 for every contraction with a
// slice view (the same bits as 1); 4 (default) the measured fastest of FMA,
// mma.sync and tcgen05 per shape.
int gemm(Group* g, int cls, const GemmArgs& q0, bool reuse = false) {
  GemmArgs q = q0;
  q.oz_s = nullptr;
  q.oz_xs = nullptr;
  // X may have changed since the planes were made: only a call that follows
  // one on the same, unchanged X may reuse them (the paths of two such
  // calls can differ under the autotuner, so the first one need not have
  // made them)
  if (!reuse) g->oz_key.valid = false;
  const int mode = g_gemm_mode.load();
  bool ok = false;
  if (mode && g->oz_xs && (q.N >= 16 || mode != 2)) ok = attach_group(g, &q);
  if (!ok) return run_path(g, cls, q, PATH_FMA, reuse);
  const bool tc_ok = mode >= 2 && q.oz_tmap != nullptr;
  int path = PATH_MMA;
  if (mode == 3 && tc_ok) path = PATH_TC;
  if ((mode == 2 || mode == 4) && tc_ok && tc_worth_it(q)) path = PATH_TC;
  if (mode == 4) {
    // the tuner weighs tcgen05 only for contractions that fill the GPU (at
    // least two tiles per SM): below that one 448-thread CTA per SM idles
    // most of its warps, and the narrow shapes stay on the kernels whose
    // launch cost is lower
    const int fixed = q.N >= 16 ? path : PATH_FMA;
    int rc = tuned_path(g, cls, q, reuse, tc_ok && tc_worth_it(q), fixed, &path);
    if (rc) return rc;
  }
  return run_path(g, cls, q, path, reuse);
}

// The merged tcgen05 launch of the row blocks v (one X, outputs after one
// another), from the merged view `all`.
int run_merged_tc(Group* g, int cls, const std::vector<GemmArgs>& v, const GemmArgs& all) {
  TcArgs t = tc_args(all);
  t.nout = (int)v.size();
  int r = 0;
  for (size_t o = 0; o < v.size(); ++o) {
    r += v[o].rows;
    t.rend[o] = r;
    t.Y[o] = v[o].Y;
  }
  const CUtensorMap* map = static_cast<const CUtensorMap*>(all.oz_tmap);
  return launch(g, cls, gemm_flops(all), [&]() { return launch_tc_gemm(t, *map, g->stream); });
}

// Mode 4, row blocks narrower than 16 columns per batch entry: one merged
// tcgen05 launch, or the blocks one after another on their own (autotuned)
// paths, whichever measures faster (the blocks unless the merged launch is
// 25 % faster: in a step graph the merged launch's 215 KB shared-memory
// configuration costs more than its isolated timing shows) with the
// autotuner's method; cached under per_mode = 2 + the
// number of blocks (path 2: merged, 0: the blocks).  The blocks run once
// untimed first, so that their own paths are measured before they are
// timed together.
int tuned_merge(Group* g, int cls, const std::vector<GemmArgs>& v, const GemmArgs& all, bool* merged) {
  *merged = false;
  TuneKey k{device_tag(), all.rows, all.K, all.N, all.batch, all.oz_w, 2 + (int)v.size(), 0};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(k);
    if (it != g_tune.end()) {
      *merged = it->second.path == PATH_TC;
      return 0;
    }
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(g->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone || g->prof) return 0;
  void* flush = tune_flush_buffer();
  if (!flush) return fail(FALCON_ENOMEM, "contraction tuning: no device memory for the L2 flush buffer");
  auto blocks = [&]() {
    for (size_t o = 0; o < v.size(); ++o) {
      const int rc = gemm(g, cls, v[o], o > 0);
      if (rc) return rc;
    }
    return 0;
  };
  int rc0 = blocks();  // the blocks' own paths, measured where new
  if (rc0) return rc0;
  auto one = [&]() { return run_merged_tc(g, cls, v, all); };
  TuneEntry e{};
  for (float& t : e.us) t = -1.f;
  CK(cudaDeviceSynchronize());
  cudaEvent_t a = nullptr, b = nullptr;
  CK(cudaEventCreate(&a));
  CK(cudaEventCreate(&b));
  int rc = time_fastest(g, flush, a, b, blocks, &e.us[PATH_FMA]);
  if (!rc) rc = time_fastest(g, flush, a, b, one, &e.us[PATH_TC]);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  e.path = e.us[PATH_TC] * 1.25f < e.us[PATH_FMA] ? PATH_TC : PATH_FMA;
  g_tune_measured++;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[k] = e;
  tune_store_locked(k, e);
  *merged = e.path == PATH_TC;
  return 0;
}

// Consecutive row blocks of one operator applied to one X, each written to
// its own output (G: omega, psi, u_phi; LAP: psi, u_phi and the two wall
// vorticity rows).  With the tcgen05 contractions they run as one launch
// over all the rows (fewer, fuller 128-row tiles, X sliced once), unless an
// output overlaps X (then a later block reads what an earlier one wrote,
// and the blocks run one after another as before).  Blocks narrower than
// 16 columns merge under mode 3, and under mode 4 where measured faster.
int gemm_blocks(Group* g, int cls, std::initializer_list<GemmArgs> blocks) {
  const std::vector<GemmArgs> v(blocks);
  const int mode = g_gemm_mode.load();
  if (mode >= 2 && g->oz_xs && !v.empty() && v.size() <= 4 && (v[0].N >= 16 || mode >= 3)) {
    const GemmArgs& f = v[0];
    const char* x0 = reinterpret_cast<const char*>(f.X);
    const char* x1 = reinterpret_cast<const char*>(f.X + (size_t)(f.batch - 1) * f.sX + (size_t)f.K * f.ldx);
    bool merge = true;
    int rows = 0;
    for (const GemmArgs& q : v) {
      const char* y = reinterpret_cast<const char*>(q.Y);
      if (q.A != f.A + rows || q.lda != f.lda || q.sA != f.sA || q.X != f.X || q.ldx != f.ldx || q.sX != f.sX ||
          q.K != f.K || q.N != f.N || q.batch != f.batch || q.ldy != f.ldy || q.sY != f.sY || q.alpha != f.alpha ||
          (y >= x0 && y < x1))
        merge = false;
      rows += q.rows;
    }
    if (merge) {
      GemmArgs all = f;
      all.rows = rows;
      all.oz_s = nullptr;
      all.oz_xs = nullptr;
      const bool ok = attach_group(g, &all);
      bool use = ok && all.oz_tmap && (mode == 3 || tc_worth_it(all));
      if (use && mode == 4 && f.N < 16) {
        g->oz_key.valid = false;  // the blocks' own X slicing starts afresh
        const int rc = tuned_merge(g, cls, v, all, &use);
        if (rc) return rc;
      }
      if (use) return run_merged_tc(g, cls, v, all);
    }
  }
  for (size_t o = 0; o < v.size(); ++o) {
    const int rc = gemm(g, cls, v[o], o > 0);
    if (rc) return rc;
  }
  return 0;
}

int elementwise(Group* g, double flops_per_el, std::function<cudaError_t()> f) {
  return launch(g, KC_ELEMENTWISE, flops_per_el * (double)g->nel(), f);
}

int run_nonlin(Group* g) {
  NonlinArgs a{};
  a.R = g->R; a.M = g->M; a.B = g->B; a.Nm = g->Nm;
  a.plan = g->fft->plan; a.tw = g->fft->tw; a.pos = g->fft->pos;
  a.t = g->T(); a.w = g->W(); a.up = g->up; a.ur = g->ur;
  a.ntp = g->ntp; a.ntr = g->ntr; a.nwp = g->nwp; a.nwr = g->nwr;
  a.umax = g->vardt ? g->umax : nullptr;
  const double P = g->P;
  const double flops = (double)g->R * g->B * (4.0 * 5.0 * P * std::log2(P) + 6.0 * P);
  const int rc = launch(g, KC_NONLIN, flops, [&]() { return launch_nonlin(a, g->stream); });
  if (rc == FALCON_ECUDA)
    g_err += " [nonlinear pass: group of " + std::to_string(g->B) + " at Nr " + std::to_string(g->R) + ", Np " +
             std::to_string(g->P) + "]";
  return rc;
}

// The implicit solves shared by IMEX and IMEXRK: temperature, then
// buoyancy, then (omega, psi, u_phi) for m >= 1 and uphi_bar for m = 0.
// st: the IMEXRK stage whose own implicit diagonal the operators take (-1:
// the scheme's diagonal).  The temperature solve runs once per sub (its Pr),
// the rest once for all instances.
int solve_all(Group* g, double2* t_out, double2* w_out, double buo_scale, double2* buo_store,
              double* ubar_store, int st = -1) {
  const int R = g->R, M = g->M, B = g->B;
  const OpSet* o = sub_ops(g, 0, st);
  cudaStream_t s = g->stream;
  int rc;
  for (size_t k = 0; k < g->subs.size(); ++k) {
    const Group::Sub& u = g->subs[k];
    GemmArgs q = per_mode(sub_ops(g, (int)k, st)->ST, R, (long)R * R, g->rhs_t + u.b0, t_out + u.b0, R, M, B, 0, M, R);
    q.N = 2 * (u.b1 - u.b0);
    if ((rc = gemm(g, KC_GEMM_MODE, q))) return rc;
  }
  if ((rc = elementwise(g, 6.0, [&]() {
         return launch_add_buoyancy(R, M, B, o->inv_r, g->ra_pr, buo_scale, t_out, g->rhs_w, buo_store, s);
       })))
    return rc;
  if (M > 1) {
    const long sG = 3L * R * R;
    if ((rc = gemm_blocks(g, KC_GEMM_MODE, {per_mode(o->G, 3 * R, sG, g->rhs_w, w_out, R, M, B, 1, M - 1, R),
                                            per_mode(o->G + R, 3 * R, sG, g->rhs_w, g->psi, R, M, B, 1, M - 1, R),
                                            per_mode(o->G + 2 * R, 3 * R, sG, g->rhs_w, g->up, R, M, B, 1, M - 1, R)})))
      return rc;
  }
  GemmArgs gu{};
  gu.A = o->U; gu.lda = 2 * R;
  gu.X = reinterpret_cast<const double*>(g->rhs_w); gu.ldx = 2L * M * B;
  gu.Y = g->ub; gu.ldy = 2L * B;
  gu.K = R; gu.rows = 2 * R; gu.N = 2 * B; gu.batch = 1; gu.alpha = 1.0;
  if ((rc = gemm(g, KC_GEMM_MODE, gu))) return rc;
  return elementwise(g, 3.0, [&]() {
    return launch_post_w(R, M, B, o->inv_r, g->psi, g->ur, g->up, w_out, g->ub, ubar_store, s);
  });
}

// compute_new_dt from the get_dtvals time scales (src/nonlin.F90:93-106) of
// the last nonlinear pass: the CFL step, bounded by dt_max, changed only
// when needed with l_optimizedt, and the dt_array history shifted.
//   multistep (src/steptime.F90:313-370): the whole history shifts;
//   IMEXRK (src/steptime_imexrk.F90:248-308): only dt_array(2);
//   RK (src/steptime_rk.F90:180-238): dt and dt_array reset to the namelist
//   dt first, the diffusive scales dr^2, (r dphi)^2 included, and the
//   "optimize" branch always taken.
// Before the second step of a run, dt = the namelist dt.
int vardt_update(Group* g, int nstep) {
  const falcon_params& p = g->p;
  const bool rk = (p.scheme_type == FALCON_RK);
  // First step after a restart (l_restart, n_step-n_restart == 1): dt_new
  // starts from the namelist dt; the IMEXRK and RK loops also reset
  // dt_array(:) (src/steptime_imexrk.F90:102-106, src/steptime_rk.F90:92-98)
  // while the multistep loop keeps the restored history; compute_new_dt
  // then sets dt_array(1) only, none of the "optimize" branches applying.
  const bool first = g->restart_first;
  g->restart_first = false;
  if (rk || nstep <= 1 || (first && p.scheme_type == FALCON_IMEXRK)) {
    g->dt_new = p.dt;
    for (int i = 0; i < 4; ++i) g->dt_array[i] = p.dt;
  }
  if (first) g->dt_new = p.dt;
  if (nstep <= 1 || (first && rk)) return 0;
  const int R = g->R;
  CK(cudaMemcpyAsync(g->umax_h.data(), g->umax, sizeof(double) * 2 * R, cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  const double pi = 4.0 * std::atan(1.0);
  double mr = 0.0, mp = 0.0, mrr = 0.0, mpp = 0.0;
  for (int r = 0; r < R; ++r) {
    const double rp = g->radius_h[r] * pi;
    const double dtr = g->dr_h[r] / g->umax_h[2 * r];
    const double dtp = (2.0 / 3.0) * rp / ((double)g->Nm * g->umax_h[2 * r + 1]);
    const double dtrr = g->dr_h[r] * g->dr_h[r];
    const double dtpp = (2.0 / 3.0) * rp / (double)g->Nm * (2.0 / 3.0) * rp / (double)g->Nm;
    mr = (r == 0) ? dtr : std::fmin(mr, dtr);
    mp = (r == 0) ? dtp : std::fmin(mp, dtp);
    mrr = (r == 0) ? dtrr : std::fmin(mrr, dtrr);
    mpp = (r == 0) ? dtpp : std::fmin(mpp, dtpp);
  }
  double dt_cal = std::fmin(mr, mp);
  if (rk) dt_cal = std::fmin(dt_cal, std::fmin(mrr, mpp));
  double dt_n;
  if (p.pr == 1.0 || p.pr > 1.0) dt_n = std::fmax(1.0 / p.pr, 1.0) * p.cfl * dt_cal;
  else dt_n = std::fmin(1.0 / p.pr, 1.0) * p.cfl * dt_cal;
  const double dt2 = std::fmin(0.5 * (1.0 / p.dt_coef + 1.0) * dt_n, p.dt_max);
  if (rk || p.l_optimizedt) {
    // dt keeps its previous value when no branch applies
    if (first) {
    } else if (g->dt_array[1] > p.dt_max) g->dt_new = p.dt_max;
    else if (g->dt_array[1] >= dt_cal) g->dt_new = dt2;
    else if (p.dt_coef * g->dt_array[1] < dt_cal && g->dt_array[1] < p.dt_max)
      g->dt_new = (g->dt_array[0] < dt2) ? dt2 : g->dt_array[0];
  } else {
    g->dt_new = dt2;
  }
  if (first) {
    g->dt_array[0] = g->dt_new;
    return 0;
  }
  const int nmax = (p.scheme_type == FALCON_IMEX) ? std::max(g->sch.n_imp, g->sch.n_exp) : 2;
  for (int i = nmax - 1; i >= 1; --i) g->dt_array[i] = g->dt_array[i - 1];
  g->dt_array[0] = g->dt_new;
  return 0;
}

int step_imex(Group* g) {
  const int R = g->R, M = g->M, B = g->B;
  const size_t n = g->nel();
  cudaStream_t s = g->stream;
  const int nstep = g->n_step + 1;
  int rc;
  if (nstep > 1) {
    if ((rc = run_nonlin(g))) return rc;
  } else {
    CK(cudaMemsetAsync(g->ntp, 0, sizeof(double2) * n, s));
    CK(cudaMemsetAsync(g->ntr, 0, sizeof(double2) * n, s));
    CK(cudaMemsetAsync(g->nwp, 0, sizeof(double2) * n, s));
    CK(cudaMemsetAsync(g->nwr, 0, sizeof(double2) * n, s));
  }
  // Variable time step: new dt, weights of the dt history, and the
  // operators rebuilt when dt_array(1) /= dt_array(2) (src/fourierloop.F90:
  // 74-91; the matrices keep their previous weight otherwise, as there).
  Scheme vs = g->sch;
  if (g->vardt) {
    if ((rc = vardt_update(g, nstep))) return rc;
    if (imex_weights(vs.imp, vs.exp, g->dt_array, &vs) != 0) return fail(FALCON_EINVAL, "unsupported time scheme");
    const bool rebuild = nstep == 1 || g->dt_array[0] != g->dt_array[1] || g->force_rebuild;
    g->force_rebuild = false;
    if (rebuild) {
      OpKey k = key_of(g->p, vs);
      k.dt = g->dt_array[0];
      k.wt = vs.wt_lhs;
      if (k < g->ops->key || g->ops->key < k) {
        std::shared_ptr<OpSet> fresh;
        if ((rc = build_opset(k, &fresh))) return rc;
        g->ops = fresh;
      }
    }
  }
  const Scheme& sc = vs;
  OpSet* o = g->ops.get();
  if ((rc = gemm(g, KC_GEMM_RADIAL, radial(o->D1p, g->ntr, g->dntr, R, M, B))) ||
      (rc = gemm(g, KC_GEMM_RADIAL, radial(o->D1p, g->nwr, g->dnwr, R, M, B))))
    return rc;
  const bool cn = (sc.imp == FALCON_IMP_CN);
  if (cn) {
    GemmArgs gl = radial(o->Lp, g->up, g->lu0, R, M, B);
    gl.N = 2 * B; gl.ldy = 2L * B;
    if ((rc = gemm(g, KC_GEMM_RADIAL, radial(o->Lp, g->T(), g->lt, R, M, B))) ||
        (rc = gemm(g, KC_GEMM_RADIAL, radial(o->Lp, g->W(), g->lw, R, M, B))) ||
        (rc = gemm(g, KC_GEMM_RADIAL, gl)))
      return rc;
  }
  const int ni = sc.n_imp, ne = sc.n_exp;
  const int he_new = (g->head_e + ne - 1) % ne;
  const int h_new = (g->head + ni - 1) % ni;
  RhsArgs a{};
  a.R = R; a.M = M; a.B = B;
  a.up = g->up; a.up0_prev = g->up0_prev;
  a.inv_r = o->inv_r; a.inv_r2 = o->inv_r2; a.ra_pr = g->ra_pr;
  a.dt = g->cur_dt(); a.inv_pr = g->inv_pr;
  a.scheme_cn = cn ? 1 : 0;
  a.n_imp = ni; a.n_exp = ne; a.wt_lhs = sc.wt_lhs;
  for (int i = 0; i < 4; ++i) { a.w_imp[i] = sc.w_imp[i]; a.w_exp[i] = sc.w_exp[i]; }
  for (int i = 0; i < ni; ++i) {
    a.th[i] = g->th[(g->head + i) % ni];
    a.wh[i] = g->wh[(g->head + i) % ni];
    a.ubh[i] = g->ubh[(g->head + i) % ni];
  }
  a.nt_new = g->nth[he_new]; a.nw_new = g->nwh[he_new]; a.urom_new = g->uromh[he_new];
  for (int i = 0; i < ne; ++i) {
    a.nth[i] = g->nth[(he_new + i) % ne];
    a.nwh[i] = g->nwh[(he_new + i) % ne];
    a.uromh[i] = g->uromh[(he_new + i) % ne];
  }
  a.ntp = g->ntp; a.ntr = g->ntr; a.dntr = g->dntr; a.nwp = g->nwp; a.nwr = g->nwr; a.dnwr = g->dnwr;
  a.lt = g->lt; a.lw = g->lw; a.lu0 = g->lu0;
  a.rhs_t = g->rhs_t; a.rhs_w = g->rhs_w;
  if ((rc = elementwise(g, 10.0 + 8.0 * (ni + ne), [&]() { return launch_imex_rhs(a, s); }))) return rc;
  const double buo_scale = g->cur_dt() * (cn ? 0.5 : sc.wt_lhs);
  if ((rc = solve_all(g, g->th[h_new], g->wh[h_new], buo_scale, nullptr, g->ubh[h_new]))) return rc;
  g->head = h_new;
  g->head_e = he_new;
  g->n_step = nstep;
  g->tot_time += g->cur_dt();
  return 0;
}

int step_imexrk(Group* g) {
  const int R = g->R, M = g->M, B = g->B;
  const size_t n = g->nel();
  cudaStream_t s = g->stream;
  const Scheme& sc = g->sch;
  const int ns = sc.n_exp;
  const int nstep = g->n_step + 1;
  const bool sa = sc.check_A && sc.check_D;
  int rc;
  // Variable time step (src/steptime_imexrk.F90:102-137): the CFL step from
  // a nonlinear pass on the assembled state (not stiffly accurate) or from
  // the last stage pass (stiffly accurate); operators rebuilt when dt
  // changed (src/fourierloop_imexrk.F90:117-125).
  if (g->vardt) {
    if (nstep > 1 && (!sa || g->need_cfl_pass)) {
      if ((rc = run_nonlin(g))) return rc;
      CK(cudaMemcpyAsync(g->t_grid, g->T(), sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
    }
    g->need_cfl_pass = false;
    if ((rc = vardt_update(g, nstep))) return rc;
    const bool rebuild = nstep == 1 || g->dt_array[0] != g->dt_array[1] || g->force_rebuild;
    g->force_rebuild = false;
    if (rebuild) {
      OpKey k = key_of(g->p, sc);
      k.dt = g->dt_array[0];
      if (k < g->ops->key || g->ops->key < k) {
        std::shared_ptr<OpSet> fresh;
        if ((rc = build_opset(k, &fresh))) return rc;
        g->ops = fresh;
        if ((rc = build_stage_ops(g, k.dt))) return rc;
      }
    }
  }
  OpSet* o = g->ops.get();
  StageArgs a{};
  a.R = R; a.M = M; a.B = B;
  a.inv_r = o->inv_r; a.inv_r2 = o->inv_r2; a.ra_pr = g->ra_pr;
  a.dt = g->cur_dt(); a.inv_pr = g->inv_pr; a.buo_imp = g->p.buo_imp;
  a.t0 = g->t0; a.w0 = g->w0; a.u0 = g->u0;
  for (int i = 0; i < ns; ++i) {
    a.fat[i] = g->fat[i]; a.fdt[i] = g->fdt[i]; a.faw[i] = g->faw[i]; a.fdw[i] = g->fdw[i]; a.buo[i] = g->buo[i];
  }
  a.rhs_t = g->rhs_t; a.rhs_w = g->rhs_w;
  a.ntp = g->ntp; a.ntr = g->ntr; a.dntr = g->dntr; a.nwp = g->nwp; a.nwr = g->nwr; a.dnwr = g->dnwr;
  a.lt = g->lt; a.lw = g->lw; a.lu0 = g->lu0; a.t = g->T(); a.w = g->W(); a.up = g->up;
  for (int st = 0; st < ns; ++st) {
    a.st = st;
    for (int i = 0; i < kMaxStages; ++i) { a.aD[i] = sc.aD[st][i]; a.aA[i] = sc.aA[st][i]; }
    a.aD_ss = sc.aD[st][st];
    if (st > 0) {
      if ((rc = elementwise(g, 12.0 * st + 8.0, [&]() { return launch_stage_rhs(a, s); }))) return rc;
      const double scale = g->p.buo_imp ? g->cur_dt() * sc.aD[st][st] : 0.0;
      if ((rc = solve_all(g, g->T(), g->W(), scale, g->buo[st], nullptr, st))) return rc;
    }
    double colsum = 0.0;
    for (int i = 0; i < ns; ++i) colsum += sc.aA[i][st];
    if ((nstep > 1 || st > 0) && (colsum + sc.bA[st] != 0.0)) {
      if ((rc = run_nonlin(g))) return rc;
      CK(cudaMemcpyAsync(g->t_grid, g->T(), sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
    } else if (nstep == 1 && st == 0) {
      CK(cudaMemsetAsync(g->ntp, 0, sizeof(double2) * n, s));
      CK(cudaMemsetAsync(g->ntr, 0, sizeof(double2) * n, s));
      CK(cudaMemsetAsync(g->nwp, 0, sizeof(double2) * n, s));
      CK(cudaMemsetAsync(g->nwr, 0, sizeof(double2) * n, s));
    }
    if (sa && st == ns - 1) break;  // last-stage derivatives are unused by the SA assembly
    GemmArgs gl = radial(o->Lp, g->up, g->lu0, R, M, B);
    gl.N = 2 * B; gl.ldy = 2L * B;
    if ((rc = gemm(g, KC_GEMM_RADIAL, radial(o->D1p, g->ntr, g->dntr, R, M, B))) ||
        (rc = gemm(g, KC_GEMM_RADIAL, radial(o->D1p, g->nwr, g->dnwr, R, M, B))) ||
        (rc = gemm(g, KC_GEMM_RADIAL, radial(o->Lp, g->T(), g->lt, R, M, B))) ||
        (rc = gemm(g, KC_GEMM_RADIAL, radial(o->Lp, g->W(), g->lw, R, M, B))) ||
        (rc = gemm(g, KC_GEMM_RADIAL, gl)))
      return rc;
    a.fat_out = g->fat[st]; a.fdt_out = g->fdt[st]; a.faw_out = g->faw[st]; a.fdw_out = g->fdw[st];
    a.buo_out = (st == 0) ? g->buo[0] : nullptr;
    if ((rc = elementwise(g, 20.0, [&]() { return launch_stage_deriv(a, s); }))) return rc;
  }
  if (sa) {
    // Assembly_stage_SA (src/fourierloop_imexrk.F90:653-665)
    CK(cudaMemcpyAsync(g->t0, g->T(), sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(g->w0, g->W(), sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
    if ((rc = launch(g, KC_ELEMENTWISE, 0.0, [&]() { return launch_extract_mode0(R, M, B, g->up, g->u0, s); }))) return rc;
  } else {
    // Assembly_stage (src/fourierloop_imexrk.F90:499-651)
    AsmArgs q{};
    q.R = R; q.M = M; q.B = B; q.ns = ns; q.dt = g->cur_dt();
    for (int i = 0; i < ns; ++i) {
      q.bA[i] = sc.bA[i]; q.bD[i] = sc.bD[i];
      q.fat[i] = g->fat[i]; q.fdt[i] = g->fdt[i]; q.faw[i] = g->faw[i]; q.fdw[i] = g->fdw[i]; q.buo[i] = g->buo[i];
    }
    q.t0 = g->t0; q.w0 = g->w0; q.rhs_w = g->rhs_w; q.u0 = g->u0;
    if ((rc = elementwise(g, 8.0 * ns + 6.0, [&]() { return launch_assembly(q, s); }))) return rc;
    if (M > 1) {
      const int rows = 2 * R + 2;
      const long sL = (long)rows * R;
      double2* psi_tmp = g->rhs_t;  // the reference leaves psii at its last-stage value
      if ((rc = gemm_blocks(g, KC_GEMM_MODE,
                            {per_mode(o->LAP, rows, sL, g->rhs_w, psi_tmp, R, M, B, 1, M - 1, R),
                             per_mode(o->LAP + R, rows, sL, g->rhs_w, g->up, R, M, B, 1, M - 1, R),
                             per_mode(o->LAP + 2 * R, rows, sL, g->rhs_w, g->w0, R, M, B, 1, M - 1, 1),
                             per_mode(o->LAP + 2 * R + 1, rows, sL, g->rhs_w, g->w0 + (size_t)(R - 1) * M * B, R, M,
                                      B, 1, M - 1, 1)})))
        return rc;
    }
    GemmArgs gd{};
    gd.A = o->D1p; gd.lda = R;
    gd.X = g->u0; gd.ldx = B;
    gd.Y = reinterpret_cast<double*>(g->lu0); gd.ldy = B;
    gd.K = R; gd.rows = R; gd.N = B; gd.batch = 1; gd.alpha = 1.0;
    if ((rc = gemm(g, KC_GEMM_RADIAL, gd))) return rc;
    if ((rc = elementwise(g, 3.0, [&]() {
           return launch_assembly_post(R, M, B, o->inv_r, g->rhs_t, g->u0, reinterpret_cast<const double*>(g->lu0),
                                       g->ur, g->up, g->w0, s);
         })))
      return rc;
    CK(cudaMemcpyAsync(g->T(), g->t0, sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(g->W(), g->w0, sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
  }
  g->n_step = nstep;
  g->tot_time += g->cur_dt();
  return 0;
}

// Explicit RK (timeloop_rk, src/steptime_rk.F90:103-141): per stage the
// stage values (Get_stage_var: psi through LAPpsi, Johnston wall vorticity,
// mode 0 from uphi_bar), the nonlinear pass, and the explicit right-hand
// sides; then Assembly_stage with the b weights.
int step_rk(Group* g) {
  const int R = g->R, M = g->M, B = g->B;
  const size_t n = g->nel();
  OpSet* o = g->ops.get();
  cudaStream_t s = g->stream;
  const Scheme& sc = g->sch;
  const int ns = sc.n_exp;
  const int nstep = g->n_step + 1;
  int rc;
  // variable time step (src/steptime_rk.F90:103-115); LAPpsi does not depend on dt
  if (g->vardt) {
    if (g->need_cfl_pass && nstep > 1 && (rc = run_nonlin(g))) return rc;
    g->need_cfl_pass = false;
    if ((rc = vardt_update(g, nstep))) return rc;
  }
  double2* dup = g->rhs_t;  // d(u_phi)/dr of every mode (rhs_t is unused by RK)
  auto combine = [&](int nf, const double* coef, double2* t_out, double2* w_out, double* u_out) {
    RkCombineArgs a{};
    a.R = R; a.M = M; a.B = B; a.nf = nf; a.dt = g->cur_dt();
    for (int i = 0; i < nf; ++i) { a.c[i] = coef[i]; a.ft[i] = g->fat[i]; a.fw[i] = g->faw[i]; }
    a.t0 = g->t0; a.w0 = g->w0; a.u0 = g->u0;
    a.t_out = t_out; a.w_out = w_out; a.u_out = u_out; a.rhs_w = g->rhs_w;
    return elementwise(g, 8.0 * nf + 4.0, [&]() { return launch_rk_combine(a, s); });
  };
  // psi, u_phi, u_r and the wall vorticity of modes >= 1 from rhs_w; mode 0
  // from uphi_bar (omega_0 = u/r + du/dr, u_phi = u, u_r = 0)
  auto psi_update = [&](double2* w_out, double* u_in) -> int {
    if (M > 1) {
      const int rows = 2 * R + 2;
      const long sL = (long)rows * R;
      if ((rc = gemm(g, KC_GEMM_MODE, per_mode(o->LAP, rows, sL, g->rhs_w, g->psi, R, M, B, 1, M - 1, R))) ||
          (rc = gemm(g, KC_GEMM_MODE, per_mode(o->LAP + R, rows, sL, g->rhs_w, g->up, R, M, B, 1, M - 1, R), true)) ||
          (rc = gemm(g, KC_GEMM_MODE, per_mode(o->LAP + 2 * R, rows, sL, g->rhs_w, w_out, R, M, B, 1, M - 1, 1),
                     w_out != g->rhs_w)) ||
          (rc = gemm(g, KC_GEMM_MODE, per_mode(o->LAP + 2 * R + 1, rows, sL, g->rhs_w, w_out + (size_t)(R - 1) * M * B,
                                               R, M, B, 1, M - 1, 1), w_out != g->rhs_w)))
        return rc;
    }
    GemmArgs gd{};
    gd.A = o->D1p; gd.lda = R;
    gd.X = u_in; gd.ldx = B;
    gd.Y = reinterpret_cast<double*>(g->lu0); gd.ldy = B;
    gd.K = R; gd.rows = R; gd.N = B; gd.batch = 1; gd.alpha = 1.0;
    if ((rc = gemm(g, KC_GEMM_RADIAL, gd))) return rc;
    return elementwise(g, 3.0, [&]() {
      return launch_assembly_post(R, M, B, o->inv_r, g->psi, u_in, reinterpret_cast<const double*>(g->lu0), g->ur,
                                  g->up, w_out, s);
    });
  };
  for (int st = 0; st < ns; ++st) {
    if (st > 0) {
      if ((rc = combine(st, sc.aA[st], g->T(), g->W(), g->us)) || (rc = psi_update(g->W(), g->us))) return rc;
    }
    if (nstep > 1 || st > 0) {
      if ((rc = run_nonlin(g))) return rc;
      CK(cudaMemcpyAsync(g->t_grid, g->T(), sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
    } else {
      CK(cudaMemsetAsync(g->ntp, 0, sizeof(double2) * n, s));
      CK(cudaMemsetAsync(g->ntr, 0, sizeof(double2) * n, s));
      CK(cudaMemsetAsync(g->nwp, 0, sizeof(double2) * n, s));
      CK(cudaMemsetAsync(g->nwr, 0, sizeof(double2) * n, s));
    }
    // the first stage of a run reads upFC as initialised (= upFR)
    const bool coef = (nstep == 1 && st == 0);
    GemmArgs gl = radial(coef ? o->Lc : o->Lp, g->up, g->lu0, R, M, B);
    gl.N = 2 * B; gl.ldy = 2L * B;
    if ((rc = gemm(g, KC_GEMM_RADIAL, radial(o->D1p, g->ntr, g->dntr, R, M, B))) ||
        (rc = gemm(g, KC_GEMM_RADIAL, radial(o->D1p, g->nwr, g->dnwr, R, M, B))) ||
        (rc = gemm(g, KC_GEMM_RADIAL, radial(o->Lp, g->T(), g->lt, R, M, B))) ||
        (rc = gemm(g, KC_GEMM_RADIAL, radial(o->Lp, g->W(), g->lw, R, M, B))) ||
        (rc = gemm(g, KC_GEMM_RADIAL, radial(coef ? o->D1c : o->D1p, g->up, dup, R, M, B))) ||
        (rc = gemm(g, KC_GEMM_RADIAL, gl)))
      return rc;
    RkRhsArgs a{};
    a.R = R; a.M = M; a.B = B; a.inv_pr = g->inv_pr;
    a.inv_r = o->inv_r; a.inv_r2 = o->inv_r2; a.ra_pr = g->ra_pr;
    a.t = g->T(); a.w = g->W(); a.lt = g->lt; a.lw = g->lw;
    a.ntp = g->ntp; a.ntr = g->ntr; a.dntr = g->dntr; a.nwp = g->nwp; a.nwr = g->nwr; a.dnwr = g->dnwr;
    a.up = g->up; a.ur = g->ur; a.dup = dup; a.lub = g->lu0;
    a.ft = g->fat[st]; a.fw = g->faw[st];
    if ((rc = elementwise(g, 30.0, [&]() { return launch_rk_rhs(a, s); })) ||
        (rc = launch(g, KC_ELEMENTWISE, 8.0 * M * R * B, [&]() { return launch_rk_ubar(a, s); })))
      return rc;
  }
  // Assembly_stage: y_n = y_0 + dt sum_i b_i F_i, in place
  if ((rc = combine(ns, sc.bA, g->t0, g->w0, g->u0)) || (rc = psi_update(g->w0, g->u0))) return rc;
  CK(cudaMemcpyAsync(g->T(), g->t0, sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(g->W(), g->w0, sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
  g->n_step = nstep;
  g->tot_time += g->cur_dt();
  return 0;
}

int group_step_direct(Group* g) {
  switch (g->p.scheme_type) {
    case FALCON_IMEX: return step_imex(g);
    case FALCON_IMEXRK: return step_imexrk(g);
    default: return step_rk(g);
  }
}

// Host-side bookkeeping of one step (what step_imex / step_imexrk update).
void group_advance(Group* g) {
  if (g->p.scheme_type == FALCON_IMEX) {
    g->head = (g->head + g->sch.n_imp - 1) % g->sch.n_imp;
    g->head_e = (g->head_e + g->sch.n_exp - 1) % g->sch.n_exp;
  }
  g->n_step += 1;
  g->tot_time += g->cur_dt();
}

// One time step.  From the second step on, the launch sequence of a step is
// fixed up to the ring-buffer phase, so each phase is captured once into a
// CUDA graph and replayed: one launch instead of 11 (IMEX) to ~60 (IMEXRK)
// kernel launches, which lets many small groups keep the GPU busy.
int group_step(Group* g) {
  // upFR_prev = upFR at the start of a run (src/init.F90:253); the IMEX
  // loop renews it every step after the nonlinear pass (in imex_rhs_kernel),
  // the IMEXRK and RK loops keep it
  if (g->n_step == 0 || g->restart_first)
    CK(launch_extract_mode0(g->R, g->M, g->B, g->up, g->up0_prev, g->stream));
  if (!g_graphs.load() || g->prof || g->n_step < 1 || g->vardt || g->direct_next) {
    g->direct_next = false;
    return group_step_direct(g);
  }
  const int phase = g->head * 8 + g->head_e;
  for (auto& sg : g->graphs)
    if (sg.phase == phase) {
      CK(cudaGraphLaunch(sg.exec, g->stream));
      g_launches += sg.kernels;
      group_advance(g);
      return 0;
    }
  const long long before = g_launches.load();
  CK(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
  const int rc = group_step_direct(g);  // advances the host state once
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(g->stream, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return fail(FALCON_ECUDA, std::string("step capture: ") + cudaGetErrorString(e));
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) return fail(FALCON_ECUDA, std::string("step graph: ") + cudaGetErrorString(ei));
  g->graphs.push_back({phase, exec, g_launches.load() - before});
  CK(cudaGraphLaunch(exec, g->stream));
  return 0;
}

// After a state is loaded: histories zeroed, current slot = state,
// Y0 = state (src/init.F90:393-395, src/timeschemes.F90:51-53).
int group_reset_arrays(Group* g);
int group_reset(Group* g) {
  g->n_step = 0;
  g->tot_time = 0.0;
  return group_reset_arrays(g);
}

// The array part of group_reset: every column restarted from its state,
// step count and time kept (group_reset_instance on all columns at once).
int group_reset_arrays(Group* g) {
  const int R = g->R, M = g->M, B = g->B;
  const size_t n = g->nel();
  cudaStream_t s = g->stream;
  if (g->p.scheme_type == FALCON_IMEX) {
    const int ni = g->sch.n_imp, ne = g->sch.n_exp;
    for (int i = 0; i < ni; ++i)
      if (i != g->head) {
        CK(cudaMemsetAsync(g->th[i], 0, sizeof(double2) * n, s));
        CK(cudaMemsetAsync(g->wh[i], 0, sizeof(double2) * n, s));
        CK(cudaMemsetAsync(g->ubh[i], 0, sizeof(double) * R * B, s));
      }
    CK(launch_extract_mode0(R, M, B, g->up, g->ubh[g->head], s));
    for (int i = 0; i < ne; ++i) {
      CK(cudaMemsetAsync(g->nth[i], 0, sizeof(double2) * n, s));
      CK(cudaMemsetAsync(g->nwh[i], 0, sizeof(double2) * n, s));
      CK(cudaMemsetAsync(g->uromh[i], 0, sizeof(double) * R * B, s));
    }
  } else {
    CK(cudaMemcpyAsync(g->t0, g->T(), sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(g->w0, g->W(), sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(g->t_grid, g->T(), sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
    CK(launch_extract_mode0(R, M, B, g->up, g->u0, s));
    for (int i = 0; i < g->sch.n_exp; ++i)
      for (double2* q : {g->fat[i], g->fdt[i], g->faw[i], g->fdw[i], g->buo[i]})
        if (q) CK(cudaMemsetAsync(q, 0, sizeof(double2) * n, s));
  }
  CK(cudaMemsetAsync(g->psi, 0, sizeof(double2) * n, s));
  return 0;
}

// Upload one instance's Fortran-layout fields (host) into the group.  The
// copies read the caller's arrays directly: from pageable memory the copy
// has taken the data when the call returns, from pinned memory it is still
// in flight, so callers synchronise the stream before they return (every
// C-ABI caller does, through group_reset_instance or falcon_batch sync).
int group_set_instance(Group* g, int b, const double* t, const double* w, const double* up, const double* ur) {
  const int R = g->R, M = g->M, B = g->B;
  const size_t ne = (size_t)M * R, nb = sizeof(double2) * ne;
  double2* d = nullptr;
  CK(cudaMallocAsync(&d, 4 * nb, g->stream));
  const double* src[4] = {t, w, up, ur};
  double2* dst[4] = {g->T(), g->W(), g->up, g->ur};
  for (int f = 0; f < 4; ++f) {
    if (src[f]) CK(cudaMemcpyAsync(d + f * ne, src[f], nb, cudaMemcpyHostToDevice, g->stream));
    else CK(cudaMemsetAsync(d + f * ne, 0, nb, g->stream));
    CK(launch_scatter_instance(R, M, B, b, d + f * ne, dst[f], g->stream));
  }
  CK(cudaFreeAsync(d, g->stream));
  return 0;
}

// Every column of the group from host arrays: each run gives `len`
// consecutive slots from `slot0` on, its instances back to back in the host
// arrays (2 M R doubles each; a null field is zeros).  One copy per run and
// field, one scatter per field.
struct HostRun {
  int slot0, len;
  const double* src[4];
};
int group_set_columns(Group* g, const std::vector<HostRun>& runs) {
  const int R = g->R, M = g->M, B = g->B;
  const size_t ne = (size_t)M * R, nb = sizeof(double2) * ne;
  double2* d = nullptr;
  CK(cudaMallocAsync(&d, nb * B, g->stream));
  double2* dst[4] = {g->T(), g->W(), g->up, g->ur};
  for (int f = 0; f < 4; ++f) {
    for (const HostRun& k : runs) {
      double2* to = d + (size_t)k.slot0 * ne;
      if (k.src[f]) CK(cudaMemcpyAsync(to, k.src[f], nb * k.len, cudaMemcpyHostToDevice, g->stream));
      else CK(cudaMemsetAsync(to, 0, nb * k.len, g->stream));
    }
    CK(launch_scatter_columns(R, M, B, d, dst[f], g->stream));
  }
  CK(cudaFreeAsync(d, g->stream));
  return 0;
}

int group_get_instance(Group* g, int b, double* t, double* w, double* up, double* ur, double* psi) {
  const int R = g->R, M = g->M, B = g->B;
  const size_t nb = sizeof(double2) * (size_t)M * R;
  double2* d = nullptr;
  CK(cudaMallocAsync(&d, nb, g->stream));
  double* dst[5] = {t, w, up, ur, psi};
  const double2* src[5] = {g->T(), g->W(), g->up, g->ur, g->psi};
  for (int f = 0; f < 5; ++f) {
    if (!dst[f]) continue;
    CK(launch_gather_instance(R, M, B, b, src[f], d, g->stream));
    CK(cudaMemcpyAsync(g->stage_buf, d, nb, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    std::memcpy(dst[f], g->stage_buf, nb);
  }
  CK(cudaFreeAsync(d, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  return 0;
}

// Repack the instance columns of every per-instance array: slot j of the
// new layout takes old slot map[j] (or zeros when map[j] < 0).
int group_resize(Group* g, const std::vector<int>& map) {
  const int Bn = (int)map.size();
  CK(cudaStreamSynchronize(g->stream));  // the last step of the group reads the arrays
  g->drop_graphs();  // the arrays move
  for (int j = 0; j < Bn; ++j)
    if (map[j] < -1 || map[j] >= g->B) return fail(FALCON_EINVAL, "column map entry out of range");
  int* dmap = nullptr;
  CK(cudaMalloc(&dmap, sizeof(int) * std::max(Bn, 1)));
  // on the group's stream, so that the remap kernels below read the map
  // only after it has landed (a legacy-stream copy from pageable memory may
  // return before its DMA completes, and this stream does not wait for it)
  CK(cudaMemcpyAsync(dmap, map.data(), sizeof(int) * Bn, cudaMemcpyHostToDevice, g->stream));
  size_t bytes = 0;
  for (auto& f : g->fields) {
    double* old = reinterpret_cast<double*>(*f.ptr);
    double* nw = nullptr;
    const size_t n = f.rows * (size_t)std::max(Bn, 1) * f.ew;
    CK(cudaMalloc(&nw, sizeof(double) * n));
    CK(launch_remap_cols(old, nw, f.rows, g->B, Bn, f.ew, dmap, g->stream));
    CK(cudaStreamSynchronize(g->stream));
    for (auto& a : g->allocs)
      if (a == old) a = nw;
    cudaFree(old);
    *f.ptr = nw;
    bytes += sizeof(double) * f.rows * (size_t)Bn * f.ew;
  }
  cudaFree(dmap);
  g->ub = reinterpret_cast<double*>(g->ub2);
  std::vector<double> ra(Bn, 0.0), pr(Bn, g->p.pr);
  for (int j = 0; j < Bn; ++j)
    if (map[j] >= 0) { ra[j] = g->ra_pr_h[map[j]]; pr[j] = g->pr_h[map[j]]; }
  g->ra_pr_h = ra;
  g->pr_h = pr;
  g->B = Bn;
  make_subs(g);
  g->bytes = bytes;
  return 0;
}

// Per-instance fresh start (the column of `b`): its histories and stage
// stores zeroed, its current-slot uphi_bar and Y0 taken from its state.
int group_reset_instance(Group* g, int b) {
  const int R = g->R, M = g->M, B = g->B;
  const size_t n = (size_t)R * M;
  cudaStream_t s = g->stream;
  auto zero = [&](void* q, size_t rows, int ew) {
    return launch_col_op(nullptr, reinterpret_cast<double*>(q), rows, B, b, ew, s);
  };
  auto copy = [&](const void* src, void* dst, size_t rows, int ew) {
    return launch_col_op(reinterpret_cast<const double*>(src), reinterpret_cast<double*>(dst), rows, B, b, ew, s);
  };
  if (g->p.scheme_type == FALCON_IMEX) {
    for (int i = 0; i < g->sch.n_imp; ++i)
      if (i != g->head) {
        CK(zero(g->th[i], n, 2)); CK(zero(g->wh[i], n, 2)); CK(zero(g->ubh[i], R, 1));
      }
    for (int i = 0; i < g->sch.n_exp; ++i) {
      CK(zero(g->nth[i], n, 2)); CK(zero(g->nwh[i], n, 2)); CK(zero(g->uromh[i], R, 1));
    }
    CK(launch_extract_mode0(R, M, B, g->up, g->ubh[g->head], s));
  } else {
    for (int i = 0; i < g->sch.n_exp; ++i)
      for (double2* q : {g->fat[i], g->fdt[i], g->faw[i], g->fdw[i], g->buo[i]})
        if (q) CK(zero(q, n, 2));
    CK(copy(g->T(), g->t0, n, 2));
    CK(copy(g->W(), g->w0, n, 2));
    CK(copy(g->T(), g->t_grid, n, 2));
    CK(launch_extract_mode0(R, M, B, g->up, g->u0, s));
  }
  CK(zero(g->psi, n, 2));
  CK(cudaStreamSynchronize(s));
  return 0;
}

// ---------------------------------------------------------------------------
// Checkpoint and snapshot files (store_checkpoint, store_snapshot of
// src/output.F90:359-516): Fortran unformatted sequential records, each
// framed by its byte length as a 4-byte integer before and after.
// ---------------------------------------------------------------------------
struct RecordWriter {
  std::FILE* f = nullptr;
  std::vector<char> buf;
  template <class T>
  void put(const T& v) {
    const char* p = reinterpret_cast<const char*>(&v);
    buf.insert(buf.end(), p, p + sizeof(T));
  }
  void put_array(const double* v, size_t n) {
    const char* p = reinterpret_cast<const char*>(v);
    buf.insert(buf.end(), p, p + n * sizeof(double));
  }
  bool end_record() {
    const int32_t len = (int32_t)buf.size();
    const bool ok = std::fwrite(&len, 4, 1, f) == 1 && std::fwrite(buf.data(), 1, buf.size(), f) == buf.size() &&
                    std::fwrite(&len, 4, 1, f) == 1;
    buf.clear();
    return ok;
  }
};

int read_record(std::FILE* f, std::vector<char>* out) {
  int32_t a = 0, b = 0;
  if (std::fread(&a, 4, 1, f) != 1 || a < 0) return fail(FALCON_EIO, "checkpoint: truncated record header");
  out->resize((size_t)a);
  if (a > 0 && std::fread(out->data(), 1, (size_t)a, f) != (size_t)a) return fail(FALCON_EIO, "checkpoint: truncated record");
  if (std::fread(&b, 4, 1, f) != 1 || b != a) return fail(FALCON_EIO, "checkpoint: corrupt record marker");
  return 0;
}

// One instance's (M, R) complex field, Fortran layout (mode fastest).
int gather_field(Group* g, int b, const double2* src, std::vector<double>* out) {
  const size_t nb = sizeof(double2) * (size_t)g->M * g->R;
  out->assign((size_t)2 * g->M * g->R, 0.0);
  if (!src) return 0;
  double2* d = nullptr;
  CK(cudaMallocAsync(&d, nb, g->stream));
  CK(launch_gather_instance(g->R, g->M, g->B, b, src, d, g->stream));
  CK(cudaMemcpyAsync(g->stage_buf, d, nb, cudaMemcpyDeviceToHost, g->stream));
  CK(cudaFreeAsync(d, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  std::memcpy(out->data(), g->stage_buf, nb);
  return 0;
}

int scatter_field(Group* g, int b, const double* in, double2* dst) {
  const size_t nb = sizeof(double2) * (size_t)g->M * g->R;
  double2* d = nullptr;
  CK(cudaMallocAsync(&d, nb, g->stream));
  std::memcpy(g->stage_buf, in, nb);
  CK(cudaMemcpyAsync(d, g->stage_buf, nb, cudaMemcpyHostToDevice, g->stream));
  CK(launch_scatter_instance(g->R, g->M, g->B, b, d, dst, g->stream));
  CK(cudaFreeAsync(d, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  return 0;
}

// One instance's column of an R x B real array, as R complex values.
int gather_real(Group* g, int b, const double* src, std::vector<double>* out) {
  const int R = g->R, B = g->B;
  out->assign((size_t)2 * R, 0.0);
  if (!src) return 0;
  std::vector<double> all((size_t)R * B);
  CK(cudaMemcpyAsync(all.data(), src, sizeof(double) * all.size(), cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  for (int r = 0; r < R; ++r) (*out)[2 * r] = all[(size_t)r * B + b];
  return 0;
}

int scatter_real(Group* g, int b, const double* in /* R complex */, double* dst) {
  const int R = g->R, B = g->B;
  for (int r = 0; r < R; ++r)
    CK(cudaMemcpyAsync(dst + (size_t)r * B + b, in + 2 * r, sizeof(double), cudaMemcpyHostToDevice, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  return 0;
}

// Orders written in the header (n_order_tscheme_imp / _exp / _max) and the
// number of levels of the rhs_imp_* / rhs_exp_* records: the multistep
// orders; for IMEXRK the stage count in the header and single-level arrays
// (store_checkpoint_imexrk, src/output.F90:404-447); for RK the stage count
// for both (store_checkpoint with the RK orders).
struct CkptShape { int ni, ne, nmax, li, le; };
CkptShape checkpoint_shape(const Group* g) {
  if (g->p.scheme_type == FALCON_IMEX) {
    const int ni = g->sch.n_imp, ne = g->sch.n_exp;
    return {ni, ne, std::max(ni, ne), ni, ne};
  }
  const int ns = g->sch.n_exp;
  if (g->p.scheme_type == FALCON_IMEXRK) return {ns, ns, ns, 1, 1};
  return {ns, ns, ns, ns, ns};
}

// store_checkpoint (src/output.F90:359-402) for instance b.  Multistep runs
// write the history arrays rhs_imp_* (T, omega, uphi_bar at the previous
// steps) and rhs_exp_* (the explicit terms): entry i of rhs_imp is the
// state i steps before the current one, except that the oldest entry, which
// the next step shifts out before any use, is not kept on the device and is
// written as zero; the Runge-Kutta loops write their arrays as zero (they
// carry no history between steps).
int group_store_checkpoint(Group* g, int b, const char* path) {
  const int R = g->R, M = g->M;
  const CkptShape sh = checkpoint_shape(g);
  const int ni = sh.li, ne = sh.le, nmax = sh.nmax;
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return fail(FALCON_EIO, std::string("cannot write checkpoint ") + path);
  RecordWriter w;
  w.f = f;
  int rc = 0;
  auto done = [&](int e) { std::fclose(f); return e; };
  w.put(g->cur_dt()); w.put(g->tot_time);
  w.put((int32_t)g->Nm); w.put((int32_t)R); w.put((int32_t)sh.ni); w.put((int32_t)sh.ne); w.put((int32_t)nmax);
  if (!w.end_record()) return done(fail(FALCON_EIO, "checkpoint write failed"));
  for (int i = 0; i < nmax; ++i) w.put((g->vardt && i < 4) ? g->dt_array[i] : g->p.dt);
  if (!w.end_record()) return done(fail(FALCON_EIO, "checkpoint write failed"));
  std::vector<double> v;
  for (const double2* fld : std::initializer_list<const double2*>{g->T(), g->W(), g->ur, g->up}) {
    if ((rc = gather_field(g, b, fld, &v))) return done(rc);
    w.put_array(v.data(), v.size());
    if (!w.end_record()) return done(fail(FALCON_EIO, "checkpoint write failed"));
  }
  const bool ms = (g->p.scheme_type == FALCON_IMEX);
  // (order, M, R) complex arrays, the order index fastest; the vorticity
  // histories hold modes m >= 1 (mode 0 is the uphi_bar equation and the
  // reference leaves its entries zero)
  auto hist3 = [&](int n, std::function<const double2*(int)> level, bool modes1) -> int {
    std::vector<std::vector<double>> lv(n);
    for (int io = 0; io < n; ++io) {
      if ((rc = gather_field(g, b, ms ? level(io) : nullptr, &lv[io]))) return rc;
      if (modes1)
        for (int r = 0; r < R; ++r) lv[io][2 * ((size_t)r * M)] = lv[io][2 * ((size_t)r * M) + 1] = 0.0;
    }
    std::vector<double> out((size_t)2 * n * M * R);
    for (size_t rm = 0; rm < (size_t)M * R; ++rm)
      for (int io = 0; io < n; ++io) {
        out[2 * (io + (size_t)n * rm)] = lv[io][2 * rm];
        out[2 * (io + (size_t)n * rm) + 1] = lv[io][2 * rm + 1];
      }
    w.put_array(out.data(), out.size());
    return w.end_record() ? 0 : fail(FALCON_EIO, "checkpoint write failed");
  };
  auto hist2 = [&](int n, std::function<const double*(int)> level) -> int {
    std::vector<std::vector<double>> lv(n);
    for (int io = 0; io < n; ++io)
      if ((rc = gather_real(g, b, ms ? level(io) : nullptr, &lv[io]))) return rc;
    std::vector<double> out((size_t)2 * n * R);
    for (int r = 0; r < R; ++r)
      for (int io = 0; io < n; ++io) out[2 * (io + (size_t)n * r)] = lv[io][2 * r];
    w.put_array(out.data(), out.size());
    return w.end_record() ? 0 : fail(FALCON_EIO, "checkpoint write failed");
  };
  auto imp_slot = [&](int io) { return io + 1 < ni ? (g->head + io + 1) % ni : -1; };
  auto exp_slot = [&](int io) { return (g->head_e + io) % ne; };
  if ((rc = hist3(ni, [&](int io) -> const double2* { int k = imp_slot(io); return k < 0 ? nullptr : g->th[k]; },
                  false)) ||
      (rc = hist3(ne, [&](int io) -> const double2* { return g->nth[exp_slot(io)]; }, false)) ||
      (rc = hist3(ni, [&](int io) -> const double2* { int k = imp_slot(io); return k < 0 ? nullptr : g->wh[k]; },
                  true)) ||
      (rc = hist3(ne, [&](int io) -> const double2* { return g->nwh[exp_slot(io)]; }, true)) ||
      (rc = hist2(ni, [&](int io) -> const double* { int k = imp_slot(io); return k < 0 ? nullptr : g->ubh[k]; })) ||
      (rc = hist2(ne, [&](int io) -> const double* { return g->uromh[exp_slot(io)]; })))
    return done(rc);
  if (std::fclose(f) != 0) return fail(FALCON_EIO, "checkpoint close failed");
  return 0;
}

// Restores instance b from a checkpoint of the same grid and scheme: the
// state, the time, the time-step history and, for multistep runs, the
// history arrays, so that a constant-dt run continues bit for bit.  With a
// variable dt the operators are rebuilt for the restored dt at the next step
// (the reference's restart does the same, src/fourierloop.F90:87).  (The
// reference's read_checkpoint, src/init.F90:865-935, reads the state and dt
// only and rebuilds the histories from earlier checkpoints.)  The time and
// the step count are the group's: instances of one group are restored from
// checkpoints of the same run time.
int group_load_checkpoint(Group* g, int b, const char* path) {
  const int R = g->R, M = g->M;
  const CkptShape sh = checkpoint_shape(g);
  const int ni = sh.li, ne = sh.le, nmax = sh.nmax;
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return fail(FALCON_EIO, std::string("checkpoint not found: ") + path);
  auto done = [&](int e) { std::fclose(f); return e; };
  std::vector<char> rec;
  int rc;
  if ((rc = read_record(f, &rec))) return done(rc);
  if (rec.size() != 36) return done(fail(FALCON_EIO, "checkpoint: unexpected header record"));
  double dt_new, tot_time;
  int32_t hd[5];
  std::memcpy(&dt_new, rec.data(), 8);
  std::memcpy(&tot_time, rec.data() + 8, 8);
  std::memcpy(hd, rec.data() + 16, 20);
  if (hd[0] != g->Nm || hd[1] != R)
    return done(fail(FALCON_EINVAL, "checkpoint grid differs from the instance's (resolution change is not supported)"));
  if (hd[2] != sh.ni || hd[3] != sh.ne || hd[4] != nmax)
    return done(fail(FALCON_EINVAL, "checkpoint time-scheme orders differ from the instance's"));
  if ((rc = read_record(f, &rec))) return done(rc);
  if (rec.size() != sizeof(double) * nmax) return done(fail(FALCON_EIO, "checkpoint: dt_array size"));
  double dta[4] = {g->p.dt, g->p.dt, g->p.dt, g->p.dt};
  std::memcpy(dta, rec.data(), sizeof(double) * std::min(nmax, 4));
  const size_t fb = sizeof(double2) * (size_t)M * R;
  std::vector<std::vector<double>> fld(4);
  for (int k = 0; k < 4; ++k) {
    if ((rc = read_record(f, &rec))) return done(rc);
    if (rec.size() != fb) return done(fail(FALCON_EIO, "checkpoint: field size"));
    fld[k].resize((size_t)2 * M * R);
    std::memcpy(fld[k].data(), rec.data(), fb);
  }
  std::vector<std::vector<double>> hist(6);
  const int nh[6] = {ni, ne, ni, ne, ni, ne};
  for (int k = 0; k < 6; ++k) {
    if ((rc = read_record(f, &rec))) return done(rc);
    const size_t want = sizeof(double2) * (size_t)nh[k] * (k < 4 ? (size_t)M * R : (size_t)R);
    if (rec.size() != want) return done(fail(FALCON_EIO, "checkpoint: history size"));
    hist[k].resize(want / sizeof(double));
    std::memcpy(hist[k].data(), rec.data(), want);
  }
  std::fclose(f);
  // state (tFR, omgFR, urFR, upFR)
  if ((rc = scatter_field(g, b, fld[0].data(), g->T())) || (rc = scatter_field(g, b, fld[1].data(), g->W())) ||
      (rc = scatter_field(g, b, fld[2].data(), g->ur)) || (rc = scatter_field(g, b, fld[3].data(), g->up)))
    return rc;
  if ((rc = group_reset_instance(g, b))) return rc;  // Y0, uphi_bar slot, stage stores
  if (g->p.scheme_type == FALCON_IMEX) {
    auto level3 = [&](const std::vector<double>& h, int n, int io, std::vector<double>* out) {
      out->resize((size_t)2 * M * R);
      for (size_t rm = 0; rm < (size_t)M * R; ++rm) {
        (*out)[2 * rm] = h[2 * (io + (size_t)n * rm)];
        (*out)[2 * rm + 1] = h[2 * (io + (size_t)n * rm) + 1];
      }
    };
    auto level2 = [&](const std::vector<double>& h, int n, int io, std::vector<double>* out) {
      out->assign((size_t)2 * R, 0.0);
      for (int r = 0; r < R; ++r) (*out)[2 * r] = h[2 * (io + (size_t)n * r)];
    };
    std::vector<double> v;
    for (int io = 0; io + 1 < ni; ++io) {
      const int k = (g->head + io + 1) % ni;
      level3(hist[0], ni, io, &v);
      if ((rc = scatter_field(g, b, v.data(), g->th[k]))) return rc;
      level3(hist[2], ni, io, &v);
      if ((rc = scatter_field(g, b, v.data(), g->wh[k]))) return rc;
      level2(hist[4], ni, io, &v);
      if ((rc = scatter_real(g, b, v.data(), g->ubh[k]))) return rc;
    }
    for (int io = 0; io < ne; ++io) {
      const int k = (g->head_e + io) % ne;
      level3(hist[1], ne, io, &v);
      if ((rc = scatter_field(g, b, v.data(), g->nth[k]))) return rc;
      level3(hist[3], ne, io, &v);
      if ((rc = scatter_field(g, b, v.data(), g->nwh[k]))) return rc;
      level2(hist[5], ne, io, &v);
      if ((rc = scatter_real(g, b, v.data(), g->uromh[k]))) return rc;
    }
  }
  // continue as a running step sequence (the first step after a restart
  // takes the nonlinear pass, src/steptime.F90:205)
  g->n_step = std::max(g->n_step, 1);
  g->tot_time = tot_time;
  if (g->vardt) {
    for (int i = 0; i < 4; ++i) g->dt_array[i] = dta[i];
    g->dt_new = dt_new;
    g->force_rebuild = true;
    g->need_cfl_pass = (g->p.scheme_type != FALCON_IMEX);
  }
  return 0;
}

// store_snapshot (src/output.F90:487-516) for instance b.
// ---------------------------------------------------------------------------
// Restart (l_restart): get_checkpoint_data and read_checkpoint
// (src/init.F90:447-935), the restart branch of init_fields (:183-204) and
// the multistep bootstrap of timeloop_imex (src/steptime.F90:87-193 with
// rhs_*_from_restart, src/rhs_create.F90:387-573).
// ---------------------------------------------------------------------------
struct CkptData {
  double dt_new = 0.0, tot_time = 0.0;
  int nm = 0, nr = 0, ni = 0, ne = 0, nmax = 0;
  double dta[8] = {0};
  std::vector<double> fld[4];        // tFR, omgFR, urFR, upFR: complex (nm+1, nr)
  std::vector<double> h3[4], h2[2];  // rhs_imp/exp_temp, _vort (order, M, R); _uphi_bar (order, R)
};

// One record, or false at the end of the file or on a malformed frame.
bool try_record(std::FILE* f, std::vector<char>* out) {
  int32_t a = 0, b = 0;
  if (std::fread(&a, 4, 1, f) != 1 || a < 0) return false;
  out->resize((size_t)a);
  if (a > 0 && std::fread(out->data(), 1, (size_t)a, f) != (size_t)a) return false;
  return std::fread(&b, 4, 1, f) == 1 && b == a;
}

// read_checkpoint reads the header, dt_array and the four fields; the
// history records after them are kept when they hold ni / ne levels (files
// of the multistep loop) and left empty otherwise.
int read_checkpoint_file(const std::string& path, CkptData* c) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return fail(FALCON_EIO, "checkpoint not found: " + path);
  auto bad = [&](const char* what) {
    std::fclose(f);
    return fail(FALCON_EIO, std::string("checkpoint ") + path + ": " + what);
  };
  std::vector<char> rec;
  if (!try_record(f, &rec) || rec.size() != 36) return bad("unexpected header record");
  int32_t hd[5];
  std::memcpy(&c->dt_new, rec.data(), 8);
  std::memcpy(&c->tot_time, rec.data() + 8, 8);
  std::memcpy(hd, rec.data() + 16, 20);
  c->nm = hd[0]; c->nr = hd[1]; c->ni = hd[2]; c->ne = hd[3]; c->nmax = hd[4];
  if (c->nm < 1 || c->nm > 4096 || c->nr < 4 || c->nr > 257 || c->ni < 1 || c->ne < 1 || c->ni > 8 ||
      c->ne > 8 || c->nmax < 1 || c->nmax > 8)
    return bad("invalid header");
  if (!try_record(f, &rec) || rec.size() != sizeof(double) * c->nmax) return bad("dt_array size");
  std::memcpy(c->dta, rec.data(), rec.size());
  const size_t cf = (size_t)2 * (c->nm + 1) * c->nr;
  for (int k = 0; k < 4; ++k) {
    if (!try_record(f, &rec) || rec.size() != sizeof(double) * cf) return bad("field size");
    c->fld[k].resize(cf);
    std::memcpy(c->fld[k].data(), rec.data(), rec.size());
  }
  const int lv[6] = {c->ni, c->ne, c->ni, c->ne, c->ni, c->ne};
  for (int k = 0; k < 6; ++k) {
    if (!try_record(f, &rec)) break;
    const size_t want = sizeof(double) * 2 * (size_t)lv[k] * (k < 4 ? (size_t)(c->nm + 1) * c->nr : (size_t)c->nr);
    if (rec.size() != want) continue;
    std::vector<double>& h = (k < 4) ? c->h3[k] : c->h2[k - 4];
    h.resize(want / sizeof(double));
    std::memcpy(h.data(), rec.data(), want);
  }
  std::fclose(f);
  return 0;
}

// Fields of a checkpoint on a smaller grid (src/init.F90:726-861): per
// radial line the unnormalised DCT-I of the old values, zero padding, the
// DCT-I at the new length divided by 2(Nr-1), times (Nr-1)/(Nr_old-1); the
// three steps are one Nr x Nr_old matrix, applied on the device to the four
// fields at once.  Modes above the old Nm are zero.
int resample_fields(Group* g, const CkptData& c, std::vector<double> out[4]) {
  const int R = g->R, M = g->M, Ro = c.nr, Mo = c.nm + 1;
  const double pi = 4.0 * std::atan(1.0);
  auto cosn = [&](long a, long n) { return std::cos(pi * (double)(a % (2 * n)) / (double)n); };
  std::vector<double> Q((size_t)R * Ro);
  for (int i = 0; i < Ro; ++i)
    for (int j = 0; j < R; ++j) {
      double acc = 0.0;
      for (int k = 0; k < Ro; ++k) {
        const double wo = (i == 0) ? 1.0 : (i == Ro - 1) ? ((k & 1) ? -1.0 : 1.0) : 2.0 * cosn((long)i * k, Ro - 1);
        const double wn = (k == 0) ? 1.0 : (k == R - 1) ? ((j & 1) ? -1.0 : 1.0) : 2.0 * cosn((long)k * j, R - 1);
        acc += wn * wo;
      }
      Q[j + (size_t)R * i] = acc / (2.0 * (double)(R - 1)) * ((2.0 * (double)(R - 1)) / (2.0 * (double)(Ro - 1)));
    }
  const size_t nx = (size_t)2 * Ro * M * 4, ny = (size_t)2 * R * M * 4;
  std::vector<double> X(nx, 0.0), Y(ny);
  for (int r = 0; r < Ro; ++r)
    for (int m = 0; m < Mo; ++m)
      for (int f = 0; f < 4; ++f) {
        X[2 * (((size_t)r * M + m) * 4 + f)] = c.fld[f][2 * (m + (size_t)Mo * r)];
        X[2 * (((size_t)r * M + m) * 4 + f) + 1] = c.fld[f][2 * (m + (size_t)Mo * r) + 1];
      }
  double *dQ = nullptr, *dX = nullptr, *dY = nullptr;
  cudaStream_t s = g->stream;
  CK(cudaMallocAsync(&dQ, sizeof(double) * Q.size(), s));
  CK(cudaMallocAsync(&dX, sizeof(double) * nx, s));
  CK(cudaMallocAsync(&dY, sizeof(double) * ny, s));
  CK(cudaMemcpyAsync(dQ, Q.data(), sizeof(double) * Q.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(dX, X.data(), sizeof(double) * nx, cudaMemcpyHostToDevice, s));
  GemmArgs q{};
  q.A = dQ; q.lda = R;
  q.X = dX; q.ldx = 2L * M * 4;
  q.Y = dY; q.ldy = 2L * M * 4;
  q.K = Ro; q.rows = R; q.N = 2 * M * 4; q.batch = 1; q.alpha = 1.0;
  int rc = gemm(g, KC_GEMM_RADIAL, q);
  if (rc == 0) {
    CK(cudaMemcpyAsync(Y.data(), dY, sizeof(double) * ny, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  CK(cudaFreeAsync(dQ, s)); CK(cudaFreeAsync(dX, s)); CK(cudaFreeAsync(dY, s));
  CK(cudaStreamSynchronize(s));
  if (rc) return rc;
  for (int f = 0; f < 4; ++f) {
    out[f].assign((size_t)2 * M * R, 0.0);
    for (int r = 0; r < R; ++r)
      for (int m = 0; m < M; ++m) {
        out[f][2 * (m + (size_t)M * r)] = Y[2 * (((size_t)r * M + m) * 4 + f)];
        out[f][2 * (m + (size_t)M * r) + 1] = Y[2 * (((size_t)r * M + m) * 4 + f) + 1];
      }
  }
  return 0;
}

// Restart of every instance of group g, member b from the checkpoint files
// "<dirs[b]>/checkpoint_%05d" with the member's n_restart_point:
//  - a multistep scheme with l_imexrk_started (CN, BDF2, BDF3, BDF4) reads
//    the last n_imp checkpoints and builds its histories from them: for each,
//    oldest first, a nonlinear pass on that state, then its values as
//    implicit entry n_imp-j and its explicit terms as explicit entry
//    n_exp-j (1-based; j = 0 the oldest), so that for CN/AB3 the two
//    explicit entries used by the first step both come from the last two
//    states shifted by one, as in the reference;
//  - another multistep restart takes the histories of the file (the
//    reference's own reads of these records are commented out) with the
//    order rules of src/init.F90:593-716;
//  - IMEXRK and RK restart from one file, which may hold a smaller grid
//    (Chebyshev resampling, zero Fourier modes above the old Nm).
// The time step history follows src/init.F90:566-580; l_add_pert adds ampT
// to every temperature entry.  Members of one group must restart to the same
// time and dt history (they step together).
int group_restart(Group* g, const std::vector<std::string>& dirs, const std::vector<const falcon_params*>& mp) {
  const int R = g->R, M = g->M, B = g->B, Nm = g->Nm, type = g->p.scheme_type;
  const int ni = g->sch.n_imp, ne = g->sch.n_exp;
  const CkptShape sh = checkpoint_shape(g);
  const bool started = type == FALCON_IMEX && g->p.l_imexrk_started;
  const int nfiles = started ? ni : 1;
  cudaStream_t s = g->stream;
  int rc;
  std::vector<std::vector<CkptData>> cd(B, std::vector<CkptData>(nfiles));
  std::vector<std::array<double, 4>> dts(B);
  for (int b = 0; b < B; ++b) {
    if ((type == FALCON_IMEX) && ((mp[b]->l_imexrk_started != 0) != started))
      return fail(FALCON_EINVAL, "restart: l_imexrk_started differs between instances of one operator group");
    const int np = mp[b]->n_restart_point;
    if (np - nfiles + 1 < 0) return fail(FALCON_EINVAL, "restart: n_restart_point too small for the scheme");
    for (int j = 0; j < nfiles; ++j) {
      char name[64];
      std::snprintf(name, sizeof(name), "checkpoint_%05d", np - (nfiles - 1) + j);
      const std::string path = (dirs[b].empty() ? std::string(".") : dirs[b]) + "/" + name;
      if ((rc = read_checkpoint_file(path, &cd[b][j]))) return rc;
    }
    const CkptData& nw = cd[b][nfiles - 1];
    const bool same = nw.nm == Nm && nw.nr == R;
    if (!same && !(nw.nm <= Nm && nw.nr <= R))
      return fail(FALCON_EINVAL, "restart: the checkpoint's grid is larger than the instance's");
    if (!same && type == FALCON_IMEX)
      return fail(FALCON_EINVAL, "restart: a multistep scheme cannot change grid (its histories are per grid point)");
    for (int j = 0; j < nfiles; ++j)
      if (started && (cd[b][j].nm != Nm || cd[b][j].nr != R))
        return fail(FALCON_EINVAL, "restart: l_imexrk_started needs checkpoints of the instance's grid");
    if (type == FALCON_IMEX && !started) {
      for (int k = 0; k < 4; ++k)
        if (nw.h3[k].empty()) return fail(FALCON_EINVAL, "restart: the checkpoint holds no multistep histories");
      for (int k = 0; k < 2; ++k)
        if (nw.h2[k].empty()) return fail(FALCON_EINVAL, "restart: the checkpoint holds no multistep histories");
      if (ne > nw.ne && nw.ne > ni)
        return fail(FALCON_EINVAL, "restart: explicit order extension reads beyond the implicit history");
    }
    // dt_array
    std::array<double, 8> d;
    d.fill(g->p.dt);
    if (started) {
      for (int j = 0; j < nfiles; ++j) d[nfiles - 1 - j] = cd[b][j].dta[0];
    } else {
      const int mo = nw.nmax;
      for (int i = 0; i < std::min(sh.nmax, mo); ++i) d[i] = nw.dta[i];
      for (int i = mo; i < sh.nmax; ++i) d[i] = d[mo - 1];
    }
    for (int i = 0; i < 4; ++i) dts[b][i] = d[i];
    if (b > 0 && (dts[b] != dts[0] || nw.tot_time != cd[0][nfiles - 1].tot_time ||
                  nw.dt_new != cd[0][nfiles - 1].dt_new))
      return fail(FALCON_EINVAL, "restart: instances of one operator group must restart to the same time and dt");
  }
  g->drop_graphs();
  if (type == FALCON_IMEX) { g->head = 0; g->head_e = 1 % ne; }
  auto newest_fields = [&](int b, std::vector<double> f[4]) -> int {
    const CkptData& nw = cd[b][nfiles - 1];
    if (nw.nm == Nm && nw.nr == R) {
      for (int k = 0; k < 4; ++k) f[k] = nw.fld[k];
      return 0;
    }
    return resample_fields(g, nw, f);
  };
  auto put_state = [&](int b, std::vector<double> f[4]) -> int {
    int e;
    if ((e = scatter_field(g, b, f[0].data(), g->T())) || (e = scatter_field(g, b, f[1].data(), g->W())) ||
        (e = scatter_field(g, b, f[2].data(), g->ur)) || (e = scatter_field(g, b, f[3].data(), g->up)))
      return e;
    return 0;
  };
  auto add_pert = [&](int b, std::vector<double>& t) {
    if (!mp[b]->l_add_pert) return;
    for (size_t e = 0; e < t.size() / 2; ++e) t[2 * e] = mp[b]->ampT + t[2 * e];
  };
  for (int b = 0; b < B; ++b) {
    std::vector<double> f[4];
    if ((rc = newest_fields(b, f))) return rc;
    if (!started) add_pert(b, f[0]);
    if ((rc = put_state(b, f)) || (rc = group_reset_instance(g, b))) return rc;
  }
  if (started) {
    OpSet* o = g->ops.get();
    const bool cn = (g->sch.imp == FALCON_IMP_CN);
    for (int j = 0; j < nfiles; ++j) {
      const int si = ni - 1 - j, se = ne - 1 - j;
      for (int b = 0; b < B; ++b) {
        std::vector<double> f[4];
        for (int k = 0; k < 4; ++k) f[k] = cd[b][j].fld[k];
        if ((rc = put_state(b, f))) return rc;
      }
      if ((rc = run_nonlin(g)) || (rc = gemm(g, KC_GEMM_RADIAL, radial(o->D1p, g->ntr, g->dntr, R, M, B))) ||
          (rc = gemm(g, KC_GEMM_RADIAL, radial(o->D1p, g->nwr, g->dnwr, R, M, B))))
        return rc;
      // the explicit terms of this state, written by the right-hand-side
      // kernel into explicit entry se (its right-hand sides are discarded)
      RhsArgs a{};
      a.R = R; a.M = M; a.B = B;
      a.inv_r = o->inv_r; a.inv_r2 = o->inv_r2; a.ra_pr = g->ra_pr;
      a.dt = g->cur_dt(); a.inv_pr = g->inv_pr;
      a.scheme_cn = cn ? 1 : 0;
      a.n_imp = ni; a.n_exp = ne; a.wt_lhs = g->sch.wt_lhs;
      for (int i = 0; i < ni; ++i) { a.th[i] = g->th[i]; a.wh[i] = g->wh[i]; a.ubh[i] = g->ubh[i]; }
      for (int i = 0; i < ne; ++i) { a.nth[i] = g->nth[i]; a.nwh[i] = g->nwh[i]; a.uromh[i] = g->uromh[i]; }
      a.nt_new = g->nth[se]; a.nw_new = g->nwh[se]; a.urom_new = g->uromh[se];
      a.ntp = g->ntp; a.ntr = g->ntr; a.dntr = g->dntr; a.nwp = g->nwp; a.nwr = g->nwr; a.dnwr = g->dnwr;
      a.lt = g->lt; a.lw = g->lw; a.lu0 = g->lu0;
      a.rhs_t = g->rhs_t; a.rhs_w = g->rhs_w;
      if ((rc = launch(g, KC_ELEMENTWISE, 0.0, [&]() { return launch_imex_rhs(a, s); }))) return rc;
      // its values as implicit entry si (entry 0 is the current state itself)
      const size_t n = g->nel();
      if (si != 0) {
        CK(cudaMemcpyAsync(g->th[si], g->th[0], sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(g->wh[si], g->wh[0], sizeof(double2) * n, cudaMemcpyDeviceToDevice, s));
      }
      if ((rc = launch(g, KC_ELEMENTWISE, 0.0, [&]() { return launch_extract_mode0(R, M, B, g->up, g->ubh[si], s); })))
        return rc;
      CK(cudaStreamSynchronize(s));
    }
    for (int b = 0; b < B; ++b) {
      if (!mp[b]->l_add_pert) continue;
      std::vector<double> t = cd[b][nfiles - 1].fld[0];
      add_pert(b, t);
      if ((rc = scatter_field(g, b, t.data(), g->T()))) return rc;
    }
  } else if (type == FALCON_IMEX) {
    // histories of the file, with the order rules of src/init.F90:593-716
    for (int b = 0; b < B; ++b) {
      const CkptData& nw = cd[b][nfiles - 1];
      const int io_ = nw.ni, eo = nw.ne;
      auto level3 = [&](const std::vector<double>& h, int n, int io, std::vector<double>* out) {
        out->resize((size_t)2 * M * R);
        for (size_t rm = 0; rm < (size_t)M * R; ++rm) {
          (*out)[2 * rm] = h[2 * (io + (size_t)n * rm)];
          (*out)[2 * rm + 1] = h[2 * (io + (size_t)n * rm) + 1];
        }
      };
      auto level2 = [&](const std::vector<double>& h, int n, int io, std::vector<double>* out) {
        out->assign((size_t)2 * R, 0.0);
        for (int r = 0; r < R; ++r) (*out)[2 * r] = h[2 * (io + (size_t)n * r)];
      };
      std::vector<double> v;
      // implicit entry io (0-based) becomes entry io+1 of the first step;
      // the oldest is shifted out before any use
      for (int io = 0; io + 1 < ni; ++io) {
        const int src = std::min(io, io_ - 1);
        const int k = (g->head + io + 1) % ni;
        level3(nw.h3[0], io_, src, &v);
        if ((rc = scatter_field(g, b, v.data(), g->th[k]))) return rc;
        level3(nw.h3[2], io_, src, &v);
        if ((rc = scatter_field(g, b, v.data(), g->wh[k]))) return rc;
        level2(nw.h2[0], io_, src, &v);
        if ((rc = scatter_real(g, b, v.data(), g->ubh[k]))) return rc;
      }
      // explicit entries; beyond the file's order they are the implicit entry
      // n_exp_old (src/init.F90:673-679)
      for (int io = 0; io < ne; ++io) {
        const int k = (g->head_e + io) % ne;
        const bool have = io < eo;
        const int src = have ? io : std::min(eo - 1, io_ - 1);
        level3(have ? nw.h3[1] : nw.h3[0], have ? eo : io_, src, &v);
        if ((rc = scatter_field(g, b, v.data(), g->nth[k]))) return rc;
        level3(have ? nw.h3[3] : nw.h3[2], have ? eo : io_, src, &v);
        if ((rc = scatter_field(g, b, v.data(), g->nwh[k]))) return rc;
        level2(have ? nw.h2[1] : nw.h2[0], have ? eo : io_, src, &v);
        if ((rc = scatter_real(g, b, v.data(), g->uromh[k]))) return rc;
      }
    }
  }
  const CkptData& n0 = cd[0][nfiles - 1];
  g->n_step = 1;  // the first step after a restart takes the nonlinear pass
  g->tot_time = n0.tot_time;
  if (g->vardt) {
    for (int i = 0; i < 4; ++i) g->dt_array[i] = dts[0][i];
    g->dt_new = n0.dt_new;
    g->force_rebuild = true;
    g->need_cfl_pass = (type == FALCON_IMEXRK);
    g->restart_first = true;
  }
  CK(cudaStreamSynchronize(s));
  return 0;
}

int group_store_snapshot(Group* g, int b, const char* path) {
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return fail(FALCON_EIO, std::string("cannot write snapshot ") + path);
  auto done = [&](int e) { std::fclose(f); return e; };
  RecordWriter w;
  w.f = f;
  w.put(g->ra_pr_h[b] * g->pr_h[b]); w.put(g->pr_h[b]); w.put(g->p.eta);
  if (!w.end_record()) return done(fail(FALCON_EIO, "snapshot write failed"));
  w.put(g->cur_dt()); w.put(g->tot_time);
  if (!w.end_record()) return done(fail(FALCON_EIO, "snapshot write failed"));
  w.put((int32_t)g->Nm); w.put((int32_t)g->R);
  if (!w.end_record()) return done(fail(FALCON_EIO, "snapshot write failed"));
  Cheb c = make_cheb(g->R, g->p.eta);
  w.put_array(c.radius.data(), c.radius.size());
  if (!w.end_record()) return done(fail(FALCON_EIO, "snapshot write failed"));
  std::vector<double> v;
  int rc;
  for (const double2* fld : std::initializer_list<const double2*>{g->T(), g->W(), g->ur, g->up}) {
    if ((rc = gather_field(g, b, fld, &v))) return done(rc);
    w.put_array(v.data(), v.size());
    if (!w.end_record()) return done(fail(FALCON_EIO, "snapshot write failed"));
  }
  if (std::fclose(f) != 0) return fail(FALCON_EIO, "snapshot close failed");
  return 0;
}

// writeKE_spectral of every instance of the group on the device; fills
// g->diag_host (8 doubles per instance).
int group_diagnostics(Group* g) {
  OpSet* o = g->ops.get();
  DiagArgs a{};
  a.R = g->R; a.M = g->M; a.B = g->B; a.mbc_sf = g->p.mbc == 1;
  a.t = g->T(); a.w = g->W(); a.up = g->up; a.ur = g->ur;
  if (g->p.scheme_type == FALCON_IMEX) a.tprev = (g->n_step > 0) ? g->th[(g->head + 1) % g->sch.n_imp] : g->T();
  else a.tprev = g->t_grid;
  a.wq = o->wq; a.d1_0 = o->d1_0; a.d1_R = o->d1_R; a.ra_pr = g->ra_pr;
  const double eta = g->p.eta;
  a.nu_bot_den = (1.0 - eta) / (eta * std::log(eta));
  a.nu_top_den = (1.0 - eta) / std::log(eta);
  a.pi = 4.0 * std::atan(1.0);
  a.out = g->diag_dev;
  a.part = g->diag_part;
  CK(launch_diagnostics(a, g->stream));
  g->diag_host.resize((size_t)8 * g->B);
  CK(cudaMemcpyAsync(g->diag_host.data(), g->diag_dev, sizeof(double) * 8 * g->B, cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  return 0;
}

// calculate_spectra (src/output.F90:327-355) of every instance of the
// group, to the host: spec_host [2][B][M].
int group_spectra(Group* g) {
  OpSet* o = g->ops.get();
  const double four_pi = 16.0 * std::atan(1.0);
  const size_t nm = (size_t)g->M * g->B;
  CK(launch_spectra(g->R, g->M, g->B, g->T(), g->ur, g->up, o->wq, four_pi, g->spec_dev, g->spec_dev + nm,
                    g->stream));
  g->spec_host.resize(2 * nm);
  CK(cudaMemcpyAsync(g->spec_host.data(), g->spec_dev, sizeof(double) * 2 * nm, cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  return 0;
}

// The u_phi balance (src/output.F90:145-228) of every instance, to the host:
// ubal_host [B][R][3].
int group_upbalance(Group* g) {
  OpSet* o = g->ops.get();
  const int R = g->R, M = g->M, B = g->B;
  if (!g->d1up) {
    int rc = g->alloc(&g->d1up, g->nel());
    if (rc) return rc;
  }
  GemmArgs q = radial(o->D1p, g->up, g->d1up, R, M, B);  // FP64 FMA tiles (no slice view attached)
  CK(launch_gemm(q, g->stream));
  CK(launch_upbalance(R, M, B, g->ur, g->up, g->d1up, g->up0_prev, o->Lp, o->inv_r, o->inv_r2, g->cur_dt(),
                      g->ubal_dev, g->stream));
  g->ubal_host.resize((size_t)3 * R * B);
  CK(cudaMemcpyAsync(g->ubal_host.data(), g->ubal_dev, sizeof(double) * 3 * R * B, cudaMemcpyDeviceToHost,
                     g->stream));
  CK(cudaStreamSynchronize(g->stream));
  return 0;
}

void fill_diag(const Group* g, int b, double time, falcon_diag* d) {
  const double* v = &g->diag_host[(size_t)8 * b];
  d->time = time; d->dt = g->cur_dt();
  d->ke = v[0]; d->ke_r = v[1]; d->ke_phi = v[2]; d->ke_upbar = v[3];
  d->nu_top = v[4]; d->nu_bot = v[5]; d->vis = v[6]; d->buo = v[7];
}

// Seeded noise (host): splitmix64 keyed by (seed, m, i), Box-Muller in FP64.
uint64_t splitmix64(uint64_t* x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
void noise_pair(uint64_t seed, int m, int i, double* a, double* b) {
  uint64_t st = seed * 0xD1B54A32D192ED03ull ^ ((uint64_t)(unsigned)m << 32) ^ (uint64_t)(unsigned)i;
  splitmix64(&st);
  const double u1 = ((double)(splitmix64(&st) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
  const double u2 = (double)(splitmix64(&st) >> 11) * (1.0 / 9007199254740992.0);
  const double rad = std::sqrt(-2.0 * std::log(u1));
  const double ang = 2.0 * (4.0 * std::atan(1.0)) * u2;
  *a = rad * std::cos(ang);
  *b = rad * std::sin(ang);
}

// Host restatement of forfft (src/fourier_fftw.F90:39-57) by the direct sum,
// used once for the reference-style initial perturbation.
void host_forfft(int nm, int np, const double* ff, double* f) {
  const double two_pi = 8.0 * std::atan(1.0);
  for (int m = 0; m <= nm; ++m) {
    double sr = 0.0, si = 0.0;
    for (int j = 0; j < np; ++j) {
      const long idx = ((long)m * j) % np;
      const double a = two_pi * (double)idx / (double)np;
      sr += ff[j] * std::cos(a);
      si -= ff[j] * std::sin(a);
    }
    f[2 * m] = sr / (double)np;
    f[2 * m + 1] = si / (double)np;
  }
}

// Initial temperature of one instance in Fortran layout (M,R) complex.
void initial_temperature(const falcon_params& p, int kind, double amp, uint64_t seed, std::vector<double>& tFR) {
  const int R = p.nr_max, Nm = p.nm_max, M = Nm + 1, P = 3 * Nm;
  Cheb c = make_cheb(R, p.eta);
  tFR.assign((size_t)2 * M * R, 0.0);
  const double lrr = std::log(c.rmin / c.rmax), lrmax = std::log(c.rmax);
  const double pi = 4.0 * std::atan(1.0);
  if (kind == 1) {
    for (int r = 0; r < R; ++r) {
      tFR[2 * ((size_t)M * r)] = std::log(c.radius[r]) / lrr - lrmax / lrr;
      if (r == 0 || r == R - 1) continue;
      for (int m = 1; m <= Nm; ++m) {
        double a, b;
        noise_pair(seed, m, r, &a, &b);
        tFR[2 * ((size_t)m + (size_t)M * r)] = amp * a;
        tFR[2 * ((size_t)m + (size_t)M * r) + 1] = amp * b;
      }
    }
    return;
  }
  // init_perturbation (src/init.F90:277-399)
  std::vector<double> tt(P), phi(P, 0.0);
  for (int j = 1; j < P; ++j) phi[j] = phi[j - 1] + 2.0 * pi / (double)P;
  std::vector<double> gasp(R, 0.0);
  if (p.n_init == 0) {
    auto gm = [&](double r, double cc, double L) {
      return pi / 3.0 * L * r * (r + 3.0 * L) * std::exp(-r / L) +
             (2.0 * pi * L * L * (cc + L) * (cc + L)) / r * std::exp(-2.0 * cc / L) *
                 (1.0 - (1.0 - r / (cc + L)) * std::exp(r / L)) +
             pi * L * L * L * (std::exp(-r / L) - std::exp((r - 2.0 * cc) / L));
    };
    auto ge = [&](double r, double cc, double L) {
      return 2.0 * pi * L / r * std::exp(-r / L) *
             (0.5 * (r * (r + L) * (2.0 * cc - r)) + 1.0 / 3.0 * ((r - cc) * (r - cc) * (r - cc) - cc * cc * cc) -
              L * (cc + L) * (r - cc + L) + L * (cc + L) * (cc + L) * std::exp((r - 2.0 * cc) / L));
    };
    auto gc = [&](double cc, double L) {
      return pi * L * L * L * (1.0 - std::exp(-2.0 * cc / L)) - 2.0 * pi * cc * L * (cc + L) * std::exp(-2.0 * cc / L);
    };
    const double sigma_r = 0.1 / std::sqrt(2.0), sigma_p = 0.2;
    double rc = 0.5 * (c.rmax + c.rmin);
    int ir = 0;
    double best = std::fabs(c.radius[0] - rc);
    for (int i = 1; i < R; ++i)
      if (std::fabs(c.radius[i] - rc) < best) { best = std::fabs(c.radius[i] - rc); ir = i; }
    rc = c.radius[ir];
    const double c1 = 0.5 * (c.radius[R - 1] - rc), c2 = 0.5 * (rc - c.radius[0]), L = 0.5 * sigma_r;
    for (int i = 0; i < R; ++i) {
      const double rr = c.radius[i];
      if (i == ir) gasp[i] = 1.0;
      else if (rr < rc - c2) gasp[i] = ge(rc - rr, c2, L);
      else if (rr >= rc - c2 && rr < rc) gasp[i] = gm(rc - rr, c2, L);
      else if (rr > rc && rr <= rc + c1) gasp[i] = gm(rr - rc, c1, L);
      else if (rr > rc + c1) gasp[i] = ge(rr - rc, c1, L);
    }
    for (int i = 0; i < R; ++i) {
      if (i < ir) gasp[i] = gasp[i] / gc(c1, L);
      else if (i > ir) gasp[i] = gasp[i] / gc(c2, L);
    }
    for (int r = 0; r < R; ++r) {
      const double c_r = amp * gasp[r];
      const double tcon = std::log(c.radius[r]) / lrr - lrmax / lrr;
      for (int j = 0; j < P; ++j) {
        const double ph = (double)j * 2.0 * pi / (double)P;
        tt[j] = c_r * std::exp(-(ph - pi) * (ph - pi) / (sigma_p * sigma_p)) + tcon;
      }
      host_forfft(Nm, P, tt.data(), &tFR[(size_t)2 * M * r]);
    }
  } else {
    for (int r = 0; r < R; ++r) {
      const double tcon = std::log(c.radius[r]) / lrr - lrmax / lrr;
      const double rad = c.radius[r];
      for (int j = 0; j < P; ++j) {
        if (p.n_init < 0) {
          const double sp = 0.25, sr = 0.25, rmid = c.rmax - (c.rmax - c.rmin) / 2.0;
          if (phi[j] > 1.0 && phi[j] < 3.0)
            tt[j] = -1.0 * (c.rmax - rad) * (c.rmin - rad) * amp * (1.0 / (2.0 * pi * sp * sr)) *
                        std::exp(-1.0 * ((rad - rmid) * (rad - rmid) / (sr * sr) + (phi[j] - 2.0) * (phi[j] - 2.0) / (sp * sp))) +
                    tcon;
          else
            tt[j] = tcon;
        } else {
          tt[j] = amp * (c.rmax - rad) * (c.rmin - rad) * std::cos((double)p.n_init * phi[j]) + tcon;
        }
      }
      host_forfft(Nm, P, tt.data(), &tFR[(size_t)2 * M * r]);
    }
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Batches
// ---------------------------------------------------------------------------
struct falcon_batch {
  std::vector<falcon_params> params;
  bool restart_pending = false;  // l_restart set: falcon_batch_restart comes before the first step
  std::vector<std::unique_ptr<Group>> groups;
  std::vector<std::pair<int, int>> where;  // instance -> (group, slot)
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cudaEvent_t start = nullptr;  // fans the batch's stream out to the group streams
  ~falcon_batch() {
    if (stream) cudaStreamSynchronize(stream);
    groups.clear();
    if (start) cudaEventDestroy(start);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
  // Work of every group done and visible to the host.
  int sync() {
    for (auto& g : groups)
      if (g->own_stream) CK(cudaStreamSynchronize(g->stream));
    CK(cudaStreamSynchronize(stream));
    return 0;
  }
};

struct falcon_handle {
  falcon_batch* b = nullptr;
};

// Largest group of a new batch (0: one group per operator key).  Default
// 128: a uniform batch of 256 runs as two groups whose nonlinear passes
// (FP64 pipe) and contractions (tensor cores) overlap on the GPU, 3.6 %
// faster than one group of 256 (three groups of 86: 1.9 %).
std::atomic<int> g_max_group{128};

static int batch_create(const falcon_params* ps, int n, falcon_batch** out) {
  if (!ps || n <= 0 || !out) return fail(FALCON_EINVAL, "invalid batch arguments");
  for (int i = 0; i < n; ++i) {
    int rc = validate(ps[i]);
    if (rc) return rc;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(FALCON_ECUDA, "no CUDA device: the GB300 library has no CPU fallback");
  CK(init_dft_tables());
  std::unique_ptr<falcon_batch> b(new falcon_batch());
  b->params.assign(ps, ps + n);
  CK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  b->own_stream = true;
  // Instances step together whenever grid, dt and scheme match: Ra enters
  // only the buoyancy term, Pr only the temperature operator (one solve per
  // Pr within the group), both taken per instance.  Within a key the
  // instances are ordered by Pr, so that equal Pr form contiguous columns.
  std::map<OpKey, std::vector<int>> byk;
  for (int i = 0; i < n; ++i) {
    Scheme s;
    scheme_weights(ps[i].scheme_type, ps[i].scheme_imp, ps[i].scheme_exp, &s);
    OpKey k = key_of(ps[i], s);
    k.pr = 0.0;
    if (ps[i].l_vartimestep) k.tag = i + 1;
    byk[k].push_back(i);
  }
  for (auto& kv : byk)
    std::stable_sort(kv.second.begin(), kv.second.end(), [&](int a, int c) { return ps[a].pr < ps[c].pr; });
  b->where.resize(n);
  const int gmax = g_max_group.load();
  for (auto& kv : byk) {
    // instances of one key in ceil(n / gmax) balanced groups (they share
    // the operator set), each stepped on its own stream
    const int cnt = (int)kv.second.size();
    const int parts = gmax > 0 ? (cnt + gmax - 1) / gmax : 1;
    for (int pi = 0; pi < parts; ++pi) {
      const int lo = (int)((long)cnt * pi / parts), hi = (int)((long)cnt * (pi + 1) / parts);
      std::vector<int> mem(kv.second.begin() + lo, kv.second.begin() + hi);
      auto g = std::make_unique<Group>();
      g->stream = b->stream;
      int rc = group_init(g.get(), b->params, mem);
      if (rc) return rc;
      for (size_t j = 0; j < mem.size(); ++j) b->where[mem[j]] = {(int)b->groups.size(), (int)j};
      b->groups.push_back(std::move(g));
    }
  }
  for (int i = 0; i < n; ++i)
    if (b->params[i].l_restart) b->restart_pending = true;
  if (b->groups.size() > 1) {
    // groups of different operator keys run concurrently, one stream each,
    // ordered after (and joined back into) the batch's stream in every step call
    CK(cudaEventCreateWithFlags(&b->start, cudaEventDisableTiming));
    for (auto& g : b->groups) {
      CK(cudaStreamSynchronize(g->stream));
      CK(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
      g->own_stream = true;
      CK(cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming));
    }
  }
  *out = b.release();
  return 0;
}

namespace falcon {
// Error text for entry points defined in the kernels translation unit.
int set_error_message(const char* msg) {
  g_err = msg ? msg : "";
  return 0;
}
}  // namespace falcon

extern "C" {

const char* falcon_last_error(void) { return g_err.c_str(); }
const char* falcon_version(void) { return "falcon-gb300 0.1 (sm_103a, FP64)"; }

int falcon_params_default(falcon_params* p) {
  if (!p) return fail(FALCON_EINVAL, "null params");
  std::memset(p, 0, sizeof(*p));
  p->nr_max = 20; p->nm_max = 20;
  p->eta = 0.35; p->ra = 1000.0; p->pr = 1.0; p->mbc = 1; p->ampT = 0.00001;
  p->l_add_pert = 0; p->lagpts = 14; p->buo_imp = 1; p->n_init = 0;
  p->n_time_steps = 100; p->dt = 0.01; p->totaltime = 100.0;
  p->l_vartimestep = 0; p->l_optimizedt = 0;
  p->scheme_type = FALCON_IMEXRK; p->scheme_imp = FALCON_IMP_ARS222; p->scheme_exp = FALCON_EXP_ARS222;
  p->l_imexrk_started = 1; p->dt_coef = 2.0; p->dt_max = 3.e-5; p->cfl = 0.9;
  p->l_restart = 0; p->n_restart = 0; p->n_restart_point = 0; p->n_snapshot_point = 0;
  std::strcpy(p->tag, "");
  p->n_checkpoint = 500000; p->n_snapshot = 300000; p->n_KE = 1; p->n_KEspec = 100000;
  return 0;
}

int falcon_params_set_scheme(falcon_params* p, const char* type, const char* imp, const char* exp) {
  if (!p || !type || !imp || !exp) return fail(FALCON_EINVAL, "null argument");
  auto up = [](std::string s) {
    for (auto& ch : s) ch = (char)std::toupper((unsigned char)ch);
    return s;
  };
  const std::string t = up(type), i = up(imp), e = up(exp);
  if (t == "IMEX") p->scheme_type = FALCON_IMEX;
  else if (t == "IMEXRK") p->scheme_type = FALCON_IMEXRK;
  else if (t == "RK") p->scheme_type = FALCON_RK;
  else return fail(FALCON_EINVAL, "unknown time_scheme_type " + t);
  static const std::map<std::string, int> imps = {
      {"CN", FALCON_IMP_CN}, {"BDF2", FALCON_IMP_BDF2}, {"BDF3", FALCON_IMP_BDF3}, {"BDF4", FALCON_IMP_BDF4},
      {"NONE", FALCON_IMP_NONE}};
  static const std::map<std::string, int> exps = {
      {"AB2", FALCON_EXP_AB2}, {"AB3", FALCON_EXP_AB3}, {"AB4", FALCON_EXP_AB4},
      {"RK2", FALCON_EXP_RK2}, {"RK4", FALCON_EXP_RK4}};
  // IMEXRK pairs: "XXX" / "expXXX" (src/timeschemes.F90:186-962)
  int ii = -1, ie = -1;
  auto a = imps.find(i);
  auto b = exps.find(e);
  if (a != imps.end()) ii = a->second;
  else ii = imexrk_scheme_id(i.c_str());
  if (b != exps.end()) ie = b->second;
  else if (e.compare(0, 3, "EXP") == 0) ie = imexrk_scheme_id(e.c_str() + 3);
  if (ii < 0) return fail(FALCON_EINVAL, "unknown time_scheme_imp " + i);
  if (ie < 0) return fail(FALCON_EINVAL, "unknown time_scheme_exp " + e);
  p->scheme_imp = ii;
  p->scheme_exp = ie;
  return 0;
}

// Namelist reader: groups `&name ... /`, entries `key = value` separated by
// commas or newlines, `!` comments, Fortran logicals and quoted strings.
int falcon_params_read_namelist(const char* path, falcon_params* p) {
  if (!path || !p) return fail(FALCON_EINVAL, "null argument");
  std::ifstream in(path);
  if (!in) return fail(FALCON_EIO, std::string("Input namelist file not found: ") + path);
  falcon_params_default(p);
  std::string text, line;
  while (std::getline(in, line)) {
    bool inq = false;
    char q = 0;
    for (size_t i = 0; i < line.size(); ++i) {
      const char ch = line[i];
      if (inq) { if (ch == q) inq = false; }
      else if (ch == '"' || ch == '\'') { inq = true; q = ch; }
      else if (ch == '!') { line = line.substr(0, i); break; }
    }
    text += line + "\n";
  }
  std::string typ = "IMEXRK", imp = "ARS222", exp = "expARS222";
  auto lower = [](std::string s) {
    for (auto& ch : s) ch = (char)std::tolower((unsigned char)ch);
    return s;
  };
  auto trim = [](std::string s) {
    size_t a = s.find_first_not_of(" \t\r\n,");
    size_t b = s.find_last_not_of(" \t\r\n,");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
  };
  auto as_bool = [&](const std::string& v) {
    std::string s = lower(v);
    return s == ".true." || s == "t" || s == ".t." || s == "true";
  };
  auto as_str = [&](std::string v) {
    v = trim(v);
    if (v.size() >= 2 && (v[0] == '"' || v[0] == '\'')) v = v.substr(1, v.size() - 2);
    return v;
  };
  auto as_num = [&](std::string v) {
    v = trim(v);
    for (auto& ch : v) if (ch == 'd' || ch == 'D') ch = 'e';
    return std::strtod(v.c_str(), nullptr);
  };
  size_t pos = 0;
  while ((pos = text.find('&', pos)) != std::string::npos) {
    size_t end = pos + 1;
    bool inq = false;
    char qc = 0;
    for (; end < text.size(); ++end) {
      const char ch = text[end];
      if (inq) { if (ch == qc) inq = false; }
      else if (ch == '"' || ch == '\'') { inq = true; qc = ch; }
      else if (ch == '/') break;
    }
    std::string body = text.substr(pos + 1, end - pos - 1);
    pos = end;
    size_t sp = body.find_first_of(" \t\r\n");
    body = (sp == std::string::npos) ? std::string() : body.substr(sp);
    // split into key = value pairs: a key is an identifier followed by '='
    std::vector<std::pair<std::string, std::string>> kv;
    size_t i = 0;
    while (i < body.size()) {
      size_t eq = body.find('=', i);
      if (eq == std::string::npos) break;
      std::string key = lower(trim(body.substr(i, eq - i)));
      size_t ks = key.find_last_of(" \t\r\n,");
      if (ks != std::string::npos) key = key.substr(ks + 1);
      // value runs to the start of the next "ident =" outside quotes
      size_t j = eq + 1;
      bool q2 = false;
      char qq = 0;
      size_t val_end = body.size();
      for (; j < body.size(); ++j) {
        const char ch = body[j];
        if (q2) { if (ch == qq) q2 = false; continue; }
        if (ch == '"' || ch == '\'') { q2 = true; qq = ch; continue; }
        if (ch == '=') {
          size_t k = j;
          while (k > eq + 1 && std::isspace((unsigned char)body[k - 1])) --k;
          while (k > eq + 1 && (std::isalnum((unsigned char)body[k - 1]) || body[k - 1] == '_')) --k;
          val_end = k;
          break;
        }
      }
      kv.emplace_back(key, trim(body.substr(eq + 1, val_end - eq - 1)));
      i = val_end;
    }
    for (auto& e : kv) {
      const std::string& k = e.first;
      const std::string& v = e.second;
      if (k == "nr_max") p->nr_max = (int)as_num(v);
      else if (k == "nm_max") p->nm_max = (int)as_num(v);
      else if (k == "eta") p->eta = as_num(v);
      else if (k == "ra") p->ra = as_num(v);
      else if (k == "pr") p->pr = as_num(v);
      else if (k == "mbc") p->mbc = (lower(as_str(v)) == "sf") ? 1 : 0;
      else if (k == "ampt") p->ampT = as_num(v);
      else if (k == "l_add_pert") p->l_add_pert = as_bool(v);
      else if (k == "lagpts") p->lagpts = (int)as_num(v);
      else if (k == "n_init") p->n_init = (int)as_num(v);
      else if (k == "buo_tscheme") p->buo_imp = (lower(as_str(v)) == "imp") ? 1 : 0;
      else if (k == "n_time_steps") p->n_time_steps = (int)as_num(v);
      else if (k == "dt") p->dt = as_num(v);
      else if (k == "totaltime") p->totaltime = as_num(v);
      else if (k == "l_vartimestep") p->l_vartimestep = as_bool(v);
      else if (k == "l_optimizedt") p->l_optimizedt = as_bool(v);
      else if (k == "time_scheme_type") typ = as_str(v);
      else if (k == "time_scheme_imp") imp = as_str(v);
      else if (k == "time_scheme_exp") exp = as_str(v);
      else if (k == "l_imexrk_started") p->l_imexrk_started = as_bool(v);
      else if (k == "dt_coef") p->dt_coef = as_num(v);
      else if (k == "dt_max") p->dt_max = as_num(v);
      else if (k == "cfl") p->cfl = as_num(v);
      else if (k == "l_restart") p->l_restart = as_bool(v);
      else if (k == "n_restart") p->n_restart = (int)as_num(v);
      else if (k == "n_restart_point") p->n_restart_point = (int)as_num(v);
      else if (k == "n_snapshot_point") p->n_snapshot_point = (int)as_num(v);
      else if (k == "tag") std::snprintf(p->tag, sizeof(p->tag), "%s", as_str(v).c_str());
      else if (k == "n_checkpoint") p->n_checkpoint = (int)as_num(v);
      else if (k == "n_snapshot") p->n_snapshot = (int)as_num(v);
      else if (k == "n_ke") p->n_KE = (int)as_num(v);
      else if (k == "n_kespec") p->n_KEspec = (int)as_num(v);
    }
  }
  return falcon_params_set_scheme(p, typ.c_str(), imp.c_str(), exp.c_str());
}

int falcon_set_max_group_size(int n) { return g_max_group.exchange(n > 0 ? n : 0); }

int falcon_batch_create(const falcon_params* params, int n, falcon_batch** out) {
  return batch_create(params, n, out);
}

void falcon_batch_destroy(falcon_batch* b) {
  if (b) { b->sync(); delete b; }
}

int falcon_batch_size(const falcon_batch* b) { return b ? (int)b->params.size() : 0; }
int falcon_batch_ngroups(const falcon_batch* b) { return b ? (int)b->groups.size() : 0; }

size_t falcon_batch_device_bytes(const falcon_batch* b) {
  if (!b) return 0;
  size_t s = 0;
  std::vector<const OpSet*> seen;
  for (auto& g : b->groups) {
    s += g->bytes;
    std::vector<const OpSet*> sets{g->ops.get()};
    for (auto& so : g->stage_ops)
      if (so) sets.push_back(so.get());
    for (const OpSet* o : sets)
      if (std::find(seen.begin(), seen.end(), o) == seen.end()) {
        seen.push_back(o);
        s += o->bytes;
      }
  }
  return s;
}

int falcon_batch_set_stream(falcon_batch* b, void* stream) {
  if (!b) return fail(FALCON_EINVAL, "null batch");
  cudaStreamSynchronize(b->stream);
  if (b->own_stream) cudaStreamDestroy(b->stream);
  b->own_stream = false;
  b->stream = (cudaStream_t)stream;
  for (auto& g : b->groups)
    if (!g->own_stream) g->stream = b->stream;
  return 0;
}

int falcon_batch_set_state(falcon_batch* b, int i, const double* tFR, const double* omgFR, const double* upFR,
                           const double* urFR) {
  if (!b || i < 0 || i >= (int)b->params.size()) return fail(FALCON_EINVAL, "instance index out of range");
  Group* g = b->groups[b->where[i].first].get();
  int rc = group_set_instance(g, b->where[i].second, tFR, omgFR, upFR, urFR);
  if (rc) return rc;
  b->restart_pending = false;
  if (g->n_step == 0) g->tot_time = 0.0;
  return group_reset_instance(g, b->where[i].second);
}

int falcon_batch_set_states(falcon_batch* b, const double* tFR, const double* omgFR, const double* upFR,
                            const double* urFR) {
  if (!b || !tFR) return fail(FALCON_EINVAL, "null argument");
  const size_t n = b->params.size();
  const double* src[4] = {tFR, omgFR, upFR, urFR};
  std::vector<std::vector<HostRun>> runs(b->groups.size());
  std::vector<int> last(b->groups.size(), -2);  // host instance that ends each group's last run
  size_t off = 0;
  for (size_t i = 0; i < n; ++i) {
    const int gi = b->where[i].first, slot = b->where[i].second;
    auto& rv = runs[gi];
    if (!rv.empty() && last[gi] == (int)i - 1 && rv.back().slot0 + rv.back().len == slot) {
      rv.back().len += 1;
    } else {
      HostRun k{slot, 1, {}};
      for (int f = 0; f < 4; ++f) k.src[f] = src[f] ? src[f] + off : nullptr;
      rv.push_back(k);
    }
    last[gi] = (int)i;
    off += 2 * (size_t)b->params[i].nr_max * (b->params[i].nm_max + 1);
  }
  for (size_t gi = 0; gi < b->groups.size(); ++gi) {
    Group* g = b->groups[gi].get();
    int rc = group_set_columns(g, runs[gi]);
    if (!rc) rc = group_reset_arrays(g);
    if (rc) return rc;
    if (g->n_step == 0) g->tot_time = 0.0;
  }
  b->restart_pending = false;
  return b->sync();
}

int falcon_batch_init_state(falcon_batch* b, int kind, double amp, const uint64_t* seeds) {
  if (!b) return fail(FALCON_EINVAL, "null batch");
  for (size_t i = 0; i < b->params.size(); ++i) {
    std::vector<double> t;
    initial_temperature(b->params[i], kind, kind == 1 ? amp : b->params[i].ampT, seeds ? seeds[i] : (uint64_t)i, t);
    Group* g = b->groups[b->where[i].first].get();
    int rc = group_set_instance(g, b->where[i].second, t.data(), nullptr, nullptr, nullptr);
    if (rc) return rc;
  }
  for (auto& g : b->groups) {
    int rc = group_reset(g.get());
    if (rc) return rc;
  }
  b->restart_pending = false;
  return b->sync();
}

// The tensor-core contraction's bounded waits record a timeout in a device
// error word instead of hanging; read (and clear) it after a
// synchronisation.
static int check_device_waits() {
  const int v = tc_error_read_and_clear();
  if (v > 0)
    return fail(FALCON_ECUDA, "tensor-core contraction: a wait inside the kernel timed out (code " +
                                  std::to_string(v) + "); its results are invalid");
  return 0;
}

int falcon_batch_get_state(falcon_batch* b, int i, double* tFR, double* omgFR, double* upFR, double* urFR,
                           double* psi) {
  if (!b || i < 0 || i >= (int)b->params.size()) return fail(FALCON_EINVAL, "instance index out of range");
  Group* g = b->groups[b->where[i].first].get();
  const int rc = group_get_instance(g, b->where[i].second, tFR, omgFR, upFR, urFR, psi);
  return rc ? rc : check_device_waits();
}

int falcon_batch_step(falcon_batch* b, int nsteps) {
  if (!b || nsteps < 0) return fail(FALCON_EINVAL, "invalid step arguments");
  if (b->restart_pending)
    return fail(FALCON_EINVAL, "l_restart is set: restore the state with falcon_restart before stepping");
  const bool fan = b->start != nullptr;
  if (fan) {
    CK(cudaEventRecord(b->start, b->stream));
    for (auto& g : b->groups) CK(cudaStreamWaitEvent(g->stream, b->start, 0));
  }
  int rc = 0;
  for (int k = 0; k < nsteps && !rc; ++k)
    for (auto& g : b->groups) {
      rc = group_step(g.get());
      if (rc) break;
    }
  if (fan) {
    for (auto& g : b->groups) {
      CK(cudaEventRecord(g->done, g->stream));
      CK(cudaStreamWaitEvent(b->stream, g->done, 0));
    }
  }
  if (rc) return rc;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(FALCON_ECUDA, cudaGetErrorString(e));
  return 0;
}

int falcon_batch_diagnostics(falcon_batch* b, falcon_diag* out) {
  if (!b || !out) return fail(FALCON_EINVAL, "null argument");
  for (auto& g : b->groups) {
    int rc = group_diagnostics(g.get());
    if (rc) return rc;
  }
  int status = 0;
  for (size_t i = 0; i < b->params.size(); ++i) {
    const Group* g = b->groups[b->where[i].first].get();
    fill_diag(g, b->where[i].second, g->tot_time, &out[i]);
    if (!std::isfinite(out[i].ke) || !std::isfinite(out[i].nu_top) || !std::isfinite(out[i].nu_bot)) {
      status = fail(FALCON_ENONFINITE, "non-finite state in instance " + std::to_string(i));
    } else if (out[i].ke > 1e10 && status == 0) {
      // the reference stops the run here (src/output.F90:321-323)
      status = fail(FALCON_EBLOWUP, "kinetic energy above 1e10 in instance " + std::to_string(i));
    }
  }
  const int wr = check_device_waits();
  return wr ? wr : status;
}

int falcon_create(const falcon_params* p, falcon_handle** out) {
  if (!p || !out) return fail(FALCON_EINVAL, "null argument");
  falcon_batch* b = nullptr;
  int rc = batch_create(p, 1, &b);
  if (rc) return rc;
  auto* h = new falcon_handle();
  h->b = b;
  *out = h;
  return 0;
}

void falcon_destroy(falcon_handle* h) {
  if (!h) return;
  falcon_batch_destroy(h->b);
  delete h;
}

int falcon_init_state(falcon_handle* h, int kind, double amp, uint64_t seed) {
  if (!h) return fail(FALCON_EINVAL, "null handle");
  return falcon_batch_init_state(h->b, kind, amp, &seed);
}

int falcon_set_state(falcon_handle* h, const double* tFR, const double* omgFR, const double* upFR,
                     const double* urFR) {
  if (!h) return fail(FALCON_EINVAL, "null handle");
  return falcon_batch_set_state(h->b, 0, tFR, omgFR, upFR, urFR);
}

int falcon_get_state(falcon_handle* h, double* tFR, double* omgFR, double* upFR, double* urFR, double* psi) {
  if (!h) return fail(FALCON_EINVAL, "null handle");
  return falcon_batch_get_state(h->b, 0, tFR, omgFR, upFR, urFR, psi);
}

int falcon_upload_factors(falcon_handle* h, const double* AT, const int* ipiv_T, const double* AF, const int* ipiv_F,
                          const double* A_uphi, const int* ipiv_uphi, const double* LAPpsi, const int* ipiv_lap) {
  if (!h || !h->b || h->b->groups.size() != 1) return fail(FALCON_EINVAL, "null or invalid handle");
  Group* g = h->b->groups[0].get();
  if ((!AT) != (!ipiv_T) || (!AF) != (!ipiv_F) || (!A_uphi) != (!ipiv_uphi) || (!LAPpsi) != (!ipiv_lap))
    return fail(FALCON_EINVAL, "falcon_upload_factors: each factor array needs its pivots");
  if (g->sch.type == FALCON_IMEXRK && g->sch.diag_diff)
    return fail(FALCON_EINVAL, "falcon_upload_factors: this scheme solves each stage with its own operators "
                               "(stage-dependent implicit diagonal); one set of factors cannot serve them");
  if (g->sch.type == FALCON_RK && (AT || AF || A_uphi))
    return fail(FALCON_EINVAL, "falcon_upload_factors: explicit RK has no implicit AT, AF or A_uphi operators");
  const OpKey k = g->ops->key;
  if (LAPpsi && !k.needs_lap)
    return fail(FALCON_EINVAL, "falcon_upload_factors: this scheme does not solve the psi Poisson operator LAPpsi");
  const int R = g->R, M = g->M;
  auto pivots_ok = [](const int* piv, int n, int nb) {
    for (size_t i = 0; i < (size_t)n * nb; ++i)
      if (piv[i] < 1 || piv[i] > n) return false;
    return true;
  };
  if ((ipiv_T && !pivots_ok(ipiv_T, R, M)) || (ipiv_F && !pivots_ok(ipiv_F + 2 * R, 2 * R, M - 1)) ||
      (ipiv_uphi && !pivots_ok(ipiv_uphi, R, 1)) || (ipiv_lap && !pivots_ok(ipiv_lap + R, R, M - 1)))
    return fail(FALCON_EINVAL, "falcon_upload_factors: a pivot lies outside [1, n]");
  HostFactors hf;
  hf.AT = AT; hf.pT = ipiv_T; hf.AF = AF; hf.pF = ipiv_F;
  hf.Au = A_uphi; hf.pu = ipiv_uphi; hf.LAP = LAPpsi; hf.pL = ipiv_lap;
  std::shared_ptr<OpSet> fresh;
  int rc = build_opset(k, &fresh, &hf);
  if (rc) return rc;
  g->ops = fresh;
  g->drop_graphs();  // captured steps hold the previous operators
  return 0;
}

int falcon_step(falcon_handle* h, int nsteps) {
  if (!h) return fail(FALCON_EINVAL, "null handle");
  return falcon_batch_step(h->b, nsteps);
}

int falcon_diagnostics(falcon_handle* h, falcon_diag* out) {
  if (!h) return fail(FALCON_EINVAL, "null handle");
  return falcon_batch_diagnostics(h->b, out);
}

int falcon_batch_spectra(falcon_batch* b, int i, double* kespec, double* tspec) {
  if (!b || i < 0 || i >= (int)b->params.size() || !kespec || !tspec)
    return fail(FALCON_EINVAL, "falcon_batch_spectra: invalid arguments");
  Group* g = b->groups[b->where[i].first].get();
  int rc = group_spectra(g);
  if (rc) return rc;
  const int slot = b->where[i].second, M = g->M;
  const double* ke = g->spec_host.data() + (size_t)slot * M;
  const double* ts = g->spec_host.data() + (size_t)g->B * M + (size_t)slot * M;
  std::copy(ke, ke + M, kespec);
  std::copy(ts, ts + M, tspec);
  return check_device_waits();
}

int falcon_batch_upbalance(falcon_batch* b, int i, double* out) {
  if (!b || i < 0 || i >= (int)b->params.size() || !out) return fail(FALCON_EINVAL, "falcon_batch_upbalance: invalid arguments");
  Group* g = b->groups[b->where[i].first].get();
  int rc = group_upbalance(g);
  if (rc) return rc;
  const int slot = b->where[i].second, R = g->R;
  const Cheb c = make_cheb(R, g->p.eta);
  for (int r = 0; r < R; ++r) {
    const double* v = g->ubal_host.data() + ((size_t)slot * R + r) * 3;
    out[4 * r + 0] = c.radius[r];
    out[4 * r + 1] = v[0];
    out[4 * r + 2] = v[1];
    out[4 * r + 3] = v[2];
  }
  return check_device_waits();
}

int falcon_time(falcon_handle* h, double* tot_time, double* dt, int* n_step) {
  if (!h || !h->b || h->b->groups.empty()) return fail(FALCON_EINVAL, "null handle");
  const Group* g = h->b->groups[0].get();
  if (tot_time) *tot_time = g->tot_time;
  if (dt) *dt = g->cur_dt();
  if (n_step) *n_step = g->n_step;
  return 0;
}

int falcon_spectra(falcon_handle* h, double* kespec, double* tspec) {
  if (!h) return fail(FALCON_EINVAL, "null handle");
  return falcon_batch_spectra(h->b, 0, kespec, tspec);
}

int falcon_upbalance(falcon_handle* h, double* out) {
  if (!h) return fail(FALCON_EINVAL, "null handle");
  return falcon_batch_upbalance(h->b, 0, out);
}

int falcon_batch_store_checkpoint(falcon_batch* b, int i, const char* path) {
  if (!b || !path || i < 0 || i >= (int)b->params.size()) return fail(FALCON_EINVAL, "invalid checkpoint arguments");
  int rc = b->sync();
  if (rc) return rc;
  return group_store_checkpoint(b->groups[b->where[i].first].get(), b->where[i].second, path);
}

int falcon_batch_load_checkpoint(falcon_batch* b, int i, const char* path) {
  if (!b || !path || i < 0 || i >= (int)b->params.size()) return fail(FALCON_EINVAL, "invalid checkpoint arguments");
  int rc = b->sync();
  if (rc) return rc;
  return group_load_checkpoint(b->groups[b->where[i].first].get(), b->where[i].second, path);
}

int falcon_batch_store_snapshot(falcon_batch* b, int i, const char* path) {
  if (!b || !path || i < 0 || i >= (int)b->params.size()) return fail(FALCON_EINVAL, "invalid snapshot arguments");
  int rc = b->sync();
  if (rc) return rc;
  return group_store_snapshot(b->groups[b->where[i].first].get(), b->where[i].second, path);
}

int falcon_batch_restart(falcon_batch* b, const char* const* dirs) {
  if (!b) return fail(FALCON_EINVAL, "null batch");
  int rc = b->sync();
  if (rc) return rc;
  for (auto& g : b->groups) {
    std::vector<std::string> d;
    std::vector<const falcon_params*> mp;
    for (int i : g->members) {
      d.push_back((dirs && dirs[i]) ? std::string(dirs[i]) : std::string("."));
      mp.push_back(&b->params[i]);
    }
    if ((rc = group_restart(g.get(), d, mp))) return rc;
  }
  b->restart_pending = false;
  return b->sync();
}

int falcon_restart(falcon_handle* h, const char* dir) {
  if (!h) return fail(FALCON_EINVAL, "null handle");
  const char* d[1] = {dir};
  return falcon_batch_restart(h->b, d);
}

int falcon_store_checkpoint(falcon_handle* h, const char* path) {
  if (!h) return fail(FALCON_EINVAL, "null handle");
  return falcon_batch_store_checkpoint(h->b, 0, path);
}

int falcon_load_checkpoint(falcon_handle* h, const char* path) {
  if (!h) return fail(FALCON_EINVAL, "null handle");
  return falcon_batch_load_checkpoint(h->b, 0, path);
}

int falcon_store_snapshot(falcon_handle* h, const char* path) {
  if (!h) return fail(FALCON_EINVAL, "null handle");
  return falcon_batch_store_snapshot(h->b, 0, path);
}

// ---- kernel-level entry points ----
int falcon_nonlin_dev(int nr, int nm, int nb, const double* t_dev, const double* omg_dev, const double* up_dev,
                      const double* ur_dev, double* uphi_t_dev, double* ur_t_dev, double* uphi_omg_dev,
                      double* ur_omg_dev, void* stream) {
  if (nr < 1 || nm < 1 || nb < 1) return fail(FALCON_EINVAL, "invalid sizes");
  CK(init_dft_tables());
  std::unique_ptr<FftTables> f;
  int rc = make_fft(3 * nm, &f);
  if (rc) return rc;
  NonlinArgs a{};
  a.R = nr; a.M = nm + 1; a.B = nb; a.Nm = nm;
  a.plan = f->plan; a.tw = f->tw; a.pos = f->pos;
  a.t = reinterpret_cast<const double2*>(t_dev); a.w = reinterpret_cast<const double2*>(omg_dev);
  a.up = reinterpret_cast<const double2*>(up_dev); a.ur = reinterpret_cast<const double2*>(ur_dev);
  a.ntp = reinterpret_cast<double2*>(uphi_t_dev); a.ntr = reinterpret_cast<double2*>(ur_t_dev);
  a.nwp = reinterpret_cast<double2*>(uphi_omg_dev); a.nwr = reinterpret_cast<double2*>(ur_omg_dev);
  CK(launch_nonlin(a, (cudaStream_t)stream));
  CK(cudaStreamSynchronize((cudaStream_t)stream));
  return 0;
}

int falcon_nonlin(int nr, int nm, const double* tFR, const double* omgFR, const double* upFR, const double* urFR,
                  double* o1, double* o2, double* o3, double* o4) {
  if (!tFR || !omgFR || !upFR || !urFR || !o1 || !o2 || !o3 || !o4) return fail(FALCON_EINVAL, "null argument");
  const size_t nb = sizeof(double2) * (size_t)(nm + 1) * nr;
  double* d = nullptr;
  CK(cudaMalloc(&d, nb * 8));
  const double* in[4] = {tFR, omgFR, upFR, urFR};
  for (int f = 0; f < 4; ++f) CK(cudaMemcpy((char*)d + f * nb, in[f], nb, cudaMemcpyHostToDevice));
  double* q[8];
  for (int f = 0; f < 8; ++f) q[f] = (double*)((char*)d + f * nb);
  int rc = falcon_nonlin_dev(nr, nm, 1, q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], nullptr);
  if (rc) { cudaFree(d); return rc; }
  double* out[4] = {o1, o2, o3, o4};
  for (int f = 0; f < 4; ++f) CK(cudaMemcpy(out[f], q[4 + f], nb, cudaMemcpyDeviceToHost));
  cudaFree(d);
  return 0;
}

int falcon_getrs_batched_dev(int n, int nsys, int nrhs, const double* lu_dev, const int* ipiv_dev, double* b_dev,
                             void* stream) {
  if (n < 1 || nsys < 1 || nrhs < 1) return fail(FALCON_EINVAL, "invalid sizes");
  CK(launch_getrs_batched(n, nsys, nrhs, lu_dev, ipiv_dev, b_dev, (cudaStream_t)stream));
  return 0;
}

double falcon_fp64_peak_gflops(void) { return measure_fp64_peak(); }
double falcon_fp64_mma_peak_gflops(void) { return measure_fp64_mma_peak(); }

}  // extern "C"

// ---------------------------------------------------------------------------
// Chebyshev transforms as dense operators (chebtransform / chebinvtran /
// chebinvtranD1 / chebinvtranD2 of src/chebyshev_fftw.F90:124-352).  Their
// matrices, row-major n x n: inv = C t H, d1 = C D H, d2 = C D2 H,
// fwd = t^T diag(c') / ((n-1) C) (C = sqrt(2/(n-1))).
// ---------------------------------------------------------------------------
namespace {
struct ChebMats {
  int n = 0;
  double *fwd = nullptr, *inv = nullptr, *d1 = nullptr, *d2 = nullptr;
};
std::mutex g_cheb_mu;
std::map<int, ChebMats> g_cheb;

int cheb_mats(int n, ChebMats** out) {
  std::lock_guard<std::mutex> lk(g_cheb_mu);
  auto it = g_cheb.find(n);
  if (it != g_cheb.end()) { *out = &it->second; return 0; }
  Cheb c = make_cheb(n, 0.35);
  const double C = std::sqrt(2.0 / (double)(n - 1));
  std::vector<double> fwd((size_t)n * n), inv((size_t)n * n), d1((size_t)n * n), d2((size_t)n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      const double h = (j == 0 || j == n - 1) ? 0.5 : 1.0;
      inv[(size_t)i * n + j] = C * c.t[i + (size_t)n * j] * h;
      d1[(size_t)i * n + j] = C * c.D[i + (size_t)n * j] * h;
      d2[(size_t)i * n + j] = C * c.D2[i + (size_t)n * j] * h;
      const double cp = (j == 0 || j == n - 1) ? 1.0 : 2.0;  // row i = coefficient, column j = point
      fwd[(size_t)i * n + j] = c.t[j + (size_t)n * i] * cp / ((double)(n - 1) * C);
    }
  ChebMats m;
  m.n = n;
  int rc;
  if ((rc = upload(&m.fwd, fwd, nullptr)) || (rc = upload(&m.inv, inv, nullptr)) ||
      (rc = upload(&m.d1, d1, nullptr)) || (rc = upload(&m.d2, d2, nullptr)))
    return rc;
  auto res = g_cheb.emplace(n, m);
  *out = &res.first->second;
  return 0;
}

int cheb_apply(int which, int nr, int ncol, const double* in, double* out, void* stream) {
  if (nr < 3 || ncol < 1 || !in || !out) return fail(FALCON_EINVAL, "invalid Chebyshev transform arguments");
  ChebMats* m = nullptr;
  int rc = cheb_mats(nr, &m);
  if (rc) return rc;
  const double* A = which == 0 ? m->fwd : which == 1 ? m->inv : which == 2 ? m->d1 : m->d2;
  CK(launch_apply_cols(nr, ncol, A, reinterpret_cast<const double2*>(in), reinterpret_cast<double2*>(out),
                       (cudaStream_t)stream));
  return 0;
}
}  // namespace

// ---------------------------------------------------------------------------
// Serving loop: requests admitted by device-memory footprint into groups
// that share operators, stepped together one step per iteration, retired at
// their horizon.  Groups are repacked when members join or leave.
// ---------------------------------------------------------------------------
struct ServerRequest {
  int64_t id = 0;
  falcon_params p{};
  uint64_t seed = 0;
  int horizon = 0;
  int steps = 0;
  int state = 0;  // 0 queued, 1 active, 2 done (horizon reached or retired)
  int status = 0; // FALCON_OK, or FALCON_EBLOWUP / FALCON_ENONFINITE when retired early
  size_t foot = 0;
  falcon_diag diag{};
  std::vector<double> tfr, omg, upf, urf;  // final fields (Fortran layout)
  std::vector<double> init_t, init_w, init_up, init_ur;  // caller's initial state (empty: seeded noise)
  OpKey key{};   // its group: grid, dt, scheme (any Pr)
  OpKey fkey{};  // its operator set (Pr included)
};

struct ServerGroup {
  std::unique_ptr<Group> g;
  std::vector<int64_t> ids;  // request id per slot
  std::vector<int64_t> pending;
  falcon_params rep{};       // parameters of the operator key
};

struct falcon_server {
  size_t budget = 0;
  int max_active = 0;
  size_t used = 0;
  int64_t next_id = 1;
  std::deque<int64_t> queue;
  std::map<int64_t, ServerRequest> reqs;
  std::map<OpKey, ServerGroup> groups;
  std::map<OpKey, int> per_opset;  // active requests per operator set (Pr included)
  // Operator sets of past requests, kept after their last request left
  // (a set costs its assembly, LU factorisation and slicing to rebuild when
  // a request of its key arrives again), least recently used out first
  // beyond half the device budget.
  std::map<OpKey, std::pair<std::shared_ptr<OpSet>, long long>> keep;
  long long keep_clock = 0;
  // groups are spread over a pool of streams so that their steps overlap
  std::vector<cudaStream_t> streams;
  int next_stream = 0;
  int active = 0;
  ~falcon_server() {
    for (cudaStream_t q : streams) cudaStreamSynchronize(q);
    groups.clear();
    for (cudaStream_t q : streams) cudaStreamDestroy(q);
  }
  int sync() {
    for (cudaStream_t q : streams) CK(cudaStreamSynchronize(q));
    return 0;
  }
};

constexpr int kServerStreams = 16;

namespace {

// Device bytes of one resident instance (state, histories, stage stores,
// products and scratch), from the same allocation list as group_init.
size_t instance_bytes(const falcon_params& p) {
  Scheme s;
  scheme_weights(p.scheme_type, p.scheme_imp, p.scheme_exp, &s);
  const size_t R = p.nr_max, M = p.nm_max + 1, f = 16 * R * M;
  size_t n = 0;
  if (p.scheme_type == FALCON_IMEX) n += (2 * s.n_imp + 2 * s.n_exp) * f + (s.n_imp + s.n_exp) * 8 * R;
  else if (p.scheme_type == FALCON_RK) n += (2 + 2 * s.n_exp) * f + 16 * R;
  else n += (2 + 5 * s.n_exp) * f + 8 * R;
  n += 13 * f + 16 * R + 32 * R + 8;
  return n;
}

size_t opset_bytes(const falcon_params& p) {
  const size_t R = p.nr_max, M = p.nm_max + 1;
  return 8 * (2 * R * R + M * R * R + M * 3 * R * R + 2 * R * R + 2 * R);
}

// Request r's initial state into slot j of its group: the caller's fields,
// or the conductive profile plus seeded noise of amplitude 1e-3.
int server_set_initial(Group* g, int j, const ServerRequest& r) {
  if (!r.init_t.empty())
    return group_set_instance(g, j, r.init_t.data(), r.init_w.empty() ? nullptr : r.init_w.data(),
                              r.init_up.empty() ? nullptr : r.init_up.data(),
                              r.init_ur.empty() ? nullptr : r.init_ur.data());
  std::vector<double> t;
  initial_temperature(r.p, 1, 1e-3, r.seed, t);
  return group_set_instance(g, j, t.data(), nullptr, nullptr, nullptr);
}

// The operator sets a group holds, into the server's kept sets; the least
// recently used kept sets that no group holds are released while the kept
// bytes exceed half the budget.
void server_keep(falcon_server* s, const Group* g) {
  auto add = [&](const std::shared_ptr<OpSet>& o) {
    if (o) s->keep[o->key] = {o, ++s->keep_clock};
  };
  add(g->ops);
  for (const auto& so : g->stage_ops) add(so);
  for (size_t k = 1; k < g->subs.size(); ++k) {
    add(g->subs[k].ops);
    for (const auto& so : g->subs[k].stage_ops) add(so);
  }
  for (;;) {
    size_t total = 0;
    auto oldest = s->keep.end();
    for (auto it = s->keep.begin(); it != s->keep.end(); ++it) {
      total += it->second.first->bytes;
      if (it->second.first.use_count() == 1 && (oldest == s->keep.end() || it->second.second < oldest->second.second))
        oldest = it;
    }
    if (total <= s->budget / 2 || oldest == s->keep.end()) break;
    s->keep.erase(oldest);
  }
}

int server_admit_group(falcon_server* s, const OpKey& key, ServerGroup& sg) {
  // repack: keep current ids (minus retired), append pending, ordered by Pr
  // (equal Pr in contiguous columns: one temperature solve per Pr)
  std::vector<std::pair<int64_t, int>> slots;
  for (size_t j = 0; j < sg.ids.size(); ++j) {
    auto it = s->reqs.find(sg.ids[j]);
    if (it != s->reqs.end() && it->second.state == 1) slots.push_back({sg.ids[j], (int)j});
  }
  for (int64_t id : sg.pending) slots.push_back({id, -1});
  std::stable_sort(slots.begin(), slots.end(), [&](const std::pair<int64_t, int>& a, const std::pair<int64_t, int>& b) {
    return s->reqs[a.first].p.pr < s->reqs[b.first].p.pr;
  });
  std::vector<int64_t> new_ids;
  std::vector<int> map;
  for (auto& sl : slots) { new_ids.push_back(sl.first); map.push_back(sl.second); }
  sg.pending.clear();
  if (new_ids.empty()) { sg.g.reset(); sg.ids.clear(); return 0; }
  int rc;
  if (!sg.g) {
    std::vector<falcon_params> ps;
    std::vector<int> mem;
    for (size_t j = 0; j < new_ids.size(); ++j) { ps.push_back(s->reqs[new_ids[j]].p); mem.push_back((int)j); }
    sg.g = std::make_unique<Group>();
    sg.g->stream = s->streams[s->next_stream++ % s->streams.size()];
    if ((rc = group_init(sg.g.get(), ps, mem))) return rc;
    server_keep(s, sg.g.get());
    sg.ids = new_ids;
    for (size_t j = 0; j < new_ids.size(); ++j)
      if ((rc = server_set_initial(sg.g.get(), (int)j, s->reqs[new_ids[j]]))) return rc;
    return group_reset(sg.g.get());
  }
  if ((rc = group_resize(sg.g.get(), map))) return rc;
  sg.ids = new_ids;
  for (size_t j = 0; j < new_ids.size(); ++j) {
    sg.g->ra_pr_h[j] = s->reqs[new_ids[j]].p.ra / s->reqs[new_ids[j]].p.pr;
    sg.g->pr_h[j] = s->reqs[new_ids[j]].p.pr;
  }
  if ((rc = upload_instance_params(sg.g.get())) || (rc = group_refresh_subs(sg.g.get()))) return rc;
  server_keep(s, sg.g.get());
  for (size_t j = 0; j < new_ids.size(); ++j) {
    if (map[j] >= 0) continue;
    if ((rc = server_set_initial(sg.g.get(), (int)j, s->reqs[new_ids[j]]))) return rc;
    if ((rc = group_reset_instance(sg.g.get(), (int)j))) return rc;
  }
  (void)key;
  return 0;
}

}  // namespace

extern "C" {

int falcon_cheb_fwd_dev(int nr, int ncol, const double* in_dev, double* out_dev, void* stream) {
  return cheb_apply(0, nr, ncol, in_dev, out_dev, stream);
}
int falcon_cheb_inv_dev(int nr, int ncol, const double* in_dev, double* out_dev, void* stream) {
  return cheb_apply(1, nr, ncol, in_dev, out_dev, stream);
}
int falcon_cheb_d1_dev(int nr, int ncol, const double* in_dev, double* out_dev, void* stream) {
  return cheb_apply(2, nr, ncol, in_dev, out_dev, stream);
}
int falcon_cheb_d2_dev(int nr, int ncol, const double* in_dev, double* out_dev, void* stream) {
  return cheb_apply(3, nr, ncol, in_dev, out_dev, stream);
}

int falcon_cheb_d1d2_dev(int nr, int ncol, const double* in_dev, double* d1_dev, double* d2_dev, void* stream) {
  if (!d1_dev || !d2_dev || d1_dev == d2_dev || d1_dev == in_dev || d2_dev == in_dev)
    return fail(FALCON_EINVAL, "falcon_cheb_d1d2_dev: outputs must be two arrays apart from the input");
  const int rc = cheb_apply(2, nr, ncol, in_dev, d1_dev, stream);
  return rc ? rc : cheb_apply(3, nr, ncol, in_dev, d2_dev, stream);
}

int falcon_server_create(size_t hbm_budget_bytes, int max_active, falcon_server** out) {
  if (!out || hbm_budget_bytes == 0) return fail(FALCON_EINVAL, "invalid server arguments");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(FALCON_ECUDA, "no CUDA device: the GB300 library has no CPU fallback");
  CK(init_dft_tables());
  auto* s = new falcon_server();
  s->budget = hbm_budget_bytes;
  s->max_active = max_active > 0 ? max_active : (1 << 30);
  for (int i = 0; i < kServerStreams; ++i) {
    cudaStream_t q = nullptr;
    if (cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking) != cudaSuccess) {
      delete s;
      return fail(FALCON_ECUDA, "stream creation failed");
    }
    s->streams.push_back(q);
  }
  *out = s;
  return 0;
}

void falcon_server_destroy(falcon_server* s) {
  if (!s) return;
  s->sync();
  delete s;
}

int falcon_server_submit_state(falcon_server* s, const falcon_params* p, const double* tFR, const double* omgFR,
                               const double* upFR, const double* urFR, int horizon, int64_t* id) {
  if (!tFR) return fail(FALCON_EINVAL, "falcon_server_submit_state: tFR is required");
  int64_t rid = 0;
  int rc = falcon_server_submit(s, p, 0, horizon, &rid);
  if (rc) return rc;
  ServerRequest& r = s->reqs[rid];
  const size_t n = (size_t)2 * (p->nm_max + 1) * p->nr_max;
  r.init_t.assign(tFR, tFR + n);
  if (omgFR) r.init_w.assign(omgFR, omgFR + n);
  if (upFR) r.init_up.assign(upFR, upFR + n);
  if (urFR) r.init_ur.assign(urFR, urFR + n);
  if (id) *id = rid;
  return 0;
}

int falcon_server_submit(falcon_server* s, const falcon_params* p, uint64_t seed, int horizon, int64_t* id) {
  if (!s || !p || horizon <= 0) return fail(FALCON_EINVAL, "invalid request");
  int rc = validate(*p);
  if (rc) return rc;
  ServerRequest r;
  r.id = s->next_id++;
  r.p = *p;
  r.seed = seed;
  r.horizon = horizon;
  r.foot = instance_bytes(*p);
  Scheme sc;
  scheme_weights(p->scheme_type, p->scheme_imp, p->scheme_exp, &sc);
  r.key = key_of(*p, sc);
  if (p->l_vartimestep) r.key.tag = r.id;
  r.fkey = r.key;
  r.key.pr = 0.0;
  if (r.foot + opset_bytes(*p) > s->budget) return fail(FALCON_EBUSY, "request larger than the device budget");
  s->reqs[r.id] = r;
  s->queue.push_back(r.id);
  if (id) *id = r.id;
  return 0;
}

int falcon_server_iterate(falcon_server* s, int* n_active, int* n_queued) {
  if (!s) return fail(FALCON_EINVAL, "null server");
  // 1. admission, first come first served, by device footprint
  std::map<OpKey, bool> touched;
  while (!s->queue.empty() && s->active < s->max_active) {
    ServerRequest& r = s->reqs[s->queue.front()];
    const bool resident = s->per_opset[r.fkey] > 0;  // its operator set is on the device
    const size_t need = r.foot + (resident ? 0 : opset_bytes(r.p));
    if (s->used + need > s->budget) break;
    s->used += need;
    s->per_opset[r.fkey]++;
    r.state = 1;
    s->groups[r.key].pending.push_back(r.id);
    s->groups[r.key].rep = r.p;
    touched[r.key] = true;
    s->active++;
    s->queue.pop_front();
  }
  // 2. repack groups whose membership changed
  for (auto& kv : s->groups) {
    if (!touched.count(kv.first)) continue;
    int rc = server_admit_group(s, kv.first, kv.second);
    if (rc) return rc;
  }
  // 3. one step of every active group, queued on the group streams without
  // waiting: the host goes on while the device works, and synchronises
  // (in 4.) only the groups it reads this iteration
  for (auto& kv : s->groups) {
    if (!kv.second.g) continue;
    int rc = group_step(kv.second.g.get());
    if (rc) return rc;
  }
  // 4. retire finished requests: at the horizon, or early at a check of
  // the request's n_KE cadence (the reference's writeKE_spectral cadence)
  // that finds a non-finite state or KE > 1e10 (src/output.F90:321-323);
  // the rest of the group keeps running
  for (auto& kv : s->groups) {
    ServerGroup& sg = kv.second;
    if (!sg.g) continue;
    bool changed = false, have_diag = false;
    for (size_t j = 0; j < sg.ids.size(); ++j) {
      ServerRequest& r = s->reqs[sg.ids[j]];
      if (r.state != 1) continue;
      r.steps++;
      const int every = r.p.n_KE > 0 ? r.p.n_KE : 1;
      const bool at_horizon = r.steps >= r.horizon;
      if (!at_horizon && r.steps % every != 0) continue;
      int rc;
      if (!have_diag) {  // synchronises this group's stream only
        if ((rc = group_diagnostics(sg.g.get()))) return rc;
        have_diag = true;
      }
      falcon_diag d;
      fill_diag(sg.g.get(), (int)j, r.steps * r.p.dt, &d);
      int status = FALCON_OK;
      if (!std::isfinite(d.ke) || !std::isfinite(d.nu_top) || !std::isfinite(d.nu_bot)) status = FALCON_ENONFINITE;
      else if (d.ke > 1e10) status = FALCON_EBLOWUP;
      if (!at_horizon && status == FALCON_OK) continue;
      const size_t n = (size_t)2 * (r.p.nm_max + 1) * r.p.nr_max;
      r.tfr.resize(n); r.omg.resize(n); r.upf.resize(n); r.urf.resize(n);
      if ((rc = group_get_instance(sg.g.get(), (int)j, r.tfr.data(), r.omg.data(), r.upf.data(), r.urf.data(),
                                   nullptr)))
        return rc;
      r.diag = d;
      r.status = status;
      r.state = 2;
      s->active--;
      s->used -= r.foot;
      if (--s->per_opset[r.fkey] == 0) s->used -= std::min(s->used, opset_bytes(r.p));
      changed = true;
    }
    if (changed) {
      int rc = server_admit_group(s, kv.first, sg);
      if (rc) return rc;
    }
  }
  if (n_active) *n_active = s->active;
  if (n_queued) *n_queued = (int)s->queue.size();
  return 0;
}

int falcon_server_poll(falcon_server* s, int64_t id, int* done, falcon_diag* out, double* tFR) {
  if (!s || !done) return fail(FALCON_EINVAL, "null argument");
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return fail(FALCON_EINVAL, "unknown request id");
  *done = it->second.state == 2;
  if (*done) {
    if (out) *out = it->second.diag;
    if (tFR) std::memcpy(tFR, it->second.tfr.data(), sizeof(double) * it->second.tfr.size());
  }
  return 0;
}

int falcon_server_result(falcon_server* s, int64_t id, int* done, int* status, falcon_diag* out, double* tFR,
                         double* omgFR, double* upFR, double* urFR) {
  if (!s || !done) return fail(FALCON_EINVAL, "null argument");
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return fail(FALCON_EINVAL, "unknown request id");
  const ServerRequest& r = it->second;
  *done = r.state == 2;
  if (status) *status = r.status;
  if (!*done) return 0;
  if (out) *out = r.diag;
  const size_t bytes = sizeof(double) * r.tfr.size();
  if (tFR) std::memcpy(tFR, r.tfr.data(), bytes);
  if (omgFR) std::memcpy(omgFR, r.omg.data(), bytes);
  if (upFR) std::memcpy(upFR, r.upf.data(), bytes);
  if (urFR) std::memcpy(urFR, r.urf.data(), bytes);
  return 0;
}

int falcon_server_steps(falcon_server* s, int64_t id, int* steps) {
  if (!s || !steps) return fail(FALCON_EINVAL, "null argument");
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return fail(FALCON_EINVAL, "unknown request id");
  *steps = it->second.steps;
  return 0;
}

}  // extern "C"

extern "C" {

long long falcon_launch_count(void) { return g_launches.load(); }

int falcon_set_step_graphs(int enable) { return g_graphs.exchange(enable ? 1 : 0); }
int falcon_set_gemm_mode(int mode) { return g_gemm_mode.exchange(mode < 0 || mode > 4 ? 4 : mode); }

int falcon_set_tune_cache(const char* path) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_env_checked = true;
  g_tune_path = path ? path : "";
  return g_tune_path.empty() ? 0 : tune_load_locked(g_tune_path);
}

int falcon_tune_clear(void) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  const int n = (int)g_tune.size();
  g_tune.clear();
  return n;
}

int falcon_tune_entries(long long* measured) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (measured) *measured = g_tune_measured.load();
  return (int)g_tune.size();
}

int falcon_tune_lookup(const char* device, int rows, int K, int N, int batch, int w, int per_mode, int reuse,
                       float* us) {
  if (!device) return fail(FALCON_EINVAL, "null device");
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(TuneKey{device, rows, K, N, batch, w, per_mode, reuse});
  if (it == g_tune.end()) return -1;
  if (us)
    for (int p = 0; p < PATH_COUNT; ++p) us[p] = it->second.us[p];
  return it->second.path;
}

const char* falcon_device_tag(void) { return device_tag().c_str(); }

int falcon_batch_profile(falcon_batch* b, int nsteps, falcon_kernel_stat* stats, int max_stats, int* nstats) {
  if (!b || nsteps <= 0 || !stats || !nstats) return fail(FALCON_EINVAL, "invalid profile arguments");
  Prof prof;
  for (auto& g : b->groups) g->prof = &prof;
  int rc = 0;
  // groups one after another: launches of concurrent groups would overlap
  // and every launch's events would time the other groups' kernels too
  for (int k = 0; k < nsteps && !rc; ++k)
    for (auto& g : b->groups) {
      rc = group_step(g.get());
      if (rc) break;
      if (cudaStreamSynchronize(g->stream) != cudaSuccess) { rc = fail(FALCON_ECUDA, "profile step failed"); break; }
    }
  for (auto& g : b->groups) g->prof = nullptr;
  b->sync();
  double ms[KC_COUNT] = {0}, fl[KC_COUNT] = {0};
  int nl[KC_COUNT] = {0};
  for (auto& r : prof.recs) {
    float t = 0.f;
    cudaEventElapsedTime(&t, r.a, r.b);
    ms[r.cls] += t;
    fl[r.cls] += r.flops;
    nl[r.cls] += 1;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  if (rc) return rc;
  int n = 0;
  for (int c = 0; c < KC_COUNT && n < max_stats; ++c) {
    if (!nl[c]) continue;
    std::snprintf(stats[n].name, sizeof(stats[n].name), "%s", kClassNames[c]);
    stats[n].launches = nl[c];
    stats[n].ms = ms[c];
    stats[n].flops = fl[c];
    ++n;
  }
  *nstats = n;
  return 0;
}

}  // extern "C"
