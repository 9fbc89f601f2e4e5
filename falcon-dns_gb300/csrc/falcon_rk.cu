// Explicit Runge-Kutta time stepping (RK2, RK4) of src/steptime_rk.F90,
// src/fourierloop_rk.F90 and src/rhs_create_rk.F90: the elementwise stage
// combination (Get_stage_var / Assembly_stage), the explicit right-hand
// sides, and the uphi_bar advection as a sum over modes.  The psi solves
// are the LAPpsi GEMMs of the host step; the radial derivatives are the
// physical-space GEMMs.
#include "falcon_internal.h"

namespace falcon {

static int rk_blocks(size_t n) {
  size_t g = (n + 255) / 256;
  if (g > 152 * 32) g = 152 * 32;
  return (int)(g ? g : 1);
}

// Y = Y_0 + dt sum_i c_i F_i  (src/fourierloop_rk.F90:100-112, :293-305)
__global__ void rk_combine_kernel(RkCombineArgs a) {
  const size_t total = (size_t)a.R * a.M * a.B;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(e % a.B);
    const size_t rm = e / a.B;
    const int m = (int)(rm % a.M);
    const int r = (int)(rm / a.M);
    double2 f = make_double2(0.0, 0.0);
    for (int i = 0; i < a.nf; ++i) {
      const double2 q = a.ft[i][e];
      f.x = f.x + a.c[i] * q.x;
      f.y = f.y + a.c[i] * q.y;
    }
    double2 t = a.t0[e];
    t.x = t.x + a.dt * f.x;
    t.y = t.y + a.dt * f.y;
    if (r == 0) t = make_double2(m == 0 ? 1.0 : 0.0, 0.0);
    if (r == a.R - 1) t = make_double2(0.0, 0.0);
    a.t_out[e] = t;
    double2 g = make_double2(0.0, 0.0);
    for (int i = 0; i < a.nf; ++i) {
      const double2 q = a.fw[i][e];
      g.x = g.x + a.c[i] * q.x;
      g.y = g.y + a.c[i] * q.y;
    }
    if (m == 0) {
      const size_t rb = (size_t)r * a.B + b;
      double u = a.u0[rb] + a.dt * g.x;
      if (r == 0 || r == a.R - 1) u = 0.0;
      a.u_out[rb] = u;
      a.rhs_w[e] = make_double2(0.0, 0.0);
    } else {
      double2 w = a.w0[e];
      w.x = w.x + a.dt * g.x;
      w.y = w.y + a.dt * g.y;
      a.w_out[e] = w;
      a.rhs_w[e] = (r == 0 || r == a.R - 1) ? make_double2(0.0, 0.0) : make_double2(-1.0 * w.x, -1.0 * w.y);
    }
  }
}

// F_T = Pr^-1 L_m T - (i m r^-1 (u_phi T) + d(u_r T)/dr + r^-1 (u_r T))
// F_w = L_m w - (i m r^-1 (u_phi w) + d(u_r w)/dr + r^-1 (u_r w)) - Ra/Pr i m r^-1 T
// with L_m f = (d2/dr2 + r^-1 d/dr) f - m^2 r^-2 f  (src/rhs_create_rk.F90:46-58, :103-111)
__global__ void rk_rhs_kernel(RkRhsArgs a) {
  const size_t total = (size_t)a.R * a.M * a.B;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(e % a.B);
    const size_t rm = e / a.B;
    const int m = (int)(rm % a.M);
    const int r = (int)(rm / a.M);
    const double rr = a.inv_r[r], rr2 = a.inv_r2[r];
    const double mm = (double)m * (double)m, mr = (double)m * rr;
    const double2 T = a.t[e], LT = a.lt[e];
    const double2 p = a.ntp[e], q = a.ntr[e], dq = a.dntr[e];
    const double lx = LT.x - mm * rr2 * T.x, ly = LT.y - mm * rr2 * T.y;
    const double ox = -((-mr * p.y) + dq.x + rr * q.x), oy = -((mr * p.x) + dq.y + rr * q.y);
    const double ip = a.inv_pr[b];
    a.ft[e] = make_double2(ip * lx + ox, ip * ly + oy);
    if (m == 0) continue;
    const double2 W = a.w[e], LW = a.lw[e];
    const double2 pw = a.nwp[e], qw = a.nwr[e], dqw = a.dnwr[e];
    const double wx = LW.x - mm * rr2 * W.x, wy = LW.y - mm * rr2 * W.y;
    const double vx = -((-mr * pw.y) + dqw.x + rr * qw.x), vy = -((mr * pw.x) + dqw.y + rr * qw.y);
    const double rp = a.ra_pr[b];
    a.fw[e] = make_double2((wx + vx) - rp * (-mr * T.y), (wy + vy) - rp * (mr * T.x));
  }
}

// uphi_bar right-hand side (src/rhs_create_rk.F90:135-224): diffusion
// d2u/dr2 - u/r^2 + r^-1 du/dr minus the Fourier-space means
// sum_m Re(u_r conj(d u_phi/dr)) + r^-1 Re(u_r conj(u_phi)) (both signs of m).
// One warp per (r, b); the result goes to fw[(r, 0, b)].
__global__ void rk_ubar_kernel(RkRhsArgs a) {
  const int lane = threadIdx.x & 31;
  const size_t wid = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
  if (wid >= (size_t)a.R * a.B) return;
  const int r = (int)(wid / a.B), b = (int)(wid % a.B);
  const size_t base = (size_t)r * a.M * a.B + b;
  double uu = 0.0, ud = 0.0;
  for (int m = lane; m < a.M; m += 32) {
    const size_t e = base + (size_t)m * a.B;
    const double2 ur = a.ur[e], up = a.up[e], du = a.dup[e];
    if (m == 0) {
      uu += ur.x * up.x - ur.y * up.y;
      ud += ur.x * du.x - ur.y * du.y;
    } else {
      uu += 2.0 * (ur.x * up.x + ur.y * up.y);
      ud += 2.0 * (ur.x * du.x + ur.y * du.y);
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    uu += __shfl_xor_sync(0xffffffffu, uu, off);
    ud += __shfl_xor_sync(0xffffffffu, ud, off);
  }
  if (lane == 0) {
    const double u = a.up[base].x;
    const double lu = a.lub[(size_t)r * a.B + b].x;
    const double diff = lu - a.inv_r2[r] * u;
    a.fw[base] = make_double2(diff - (ud + a.inv_r[r] * uu), 0.0);
  }
}

cudaError_t launch_rk_combine(const RkCombineArgs& a, cudaStream_t s) {
  rk_combine_kernel<<<rk_blocks((size_t)a.R * a.M * a.B), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_rk_rhs(const RkRhsArgs& a, cudaStream_t s) {
  rk_rhs_kernel<<<rk_blocks((size_t)a.R * a.M * a.B), 256, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_rk_ubar(const RkRhsArgs& a, cudaStream_t s) {
  const size_t warps = (size_t)a.R * a.B;
  const int blocks = (int)((warps * 32 + 255) / 256);
  rk_ubar_kernel<<<blocks ? blocks : 1, 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace falcon
