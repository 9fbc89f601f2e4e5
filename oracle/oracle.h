/*
 * CPU oracle for the FAlCon-DNS per-time-step hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of the
 * reference algorithm (Fortran sources of FAlCon-DNS, cited per function in
 * oracle_core.c).  It is the checker for the CUDA library and the timed CPU
 * baseline; nothing in the product links, loads or calls it.
 *
 * Arrays follow the reference's Fortran layout: a complex field X(M,R) is
 * stored mode-fastest, element (m, r) at X[m + M*r], each complex as two
 * doubles (re, im).  A real (R,R) matrix A(i,j) is column-major A[i + R*j].
 *
 * Parity status (tests/golden/make_golden.py writes the fixtures from the
 * reference tree; tests/test_oracle_golden.py checks them):
 *  - transforms against the reference's own Python restatements
 *    (python/annulus/cheblib.py: chebtransform, chebinvtran, D1, D2);
 *  - azimuthal transforms against the explicit sums of src/fourier_GG.F90;
 *  - LU against LAPACK dgetrf/dgetrs (SciPy), identical pivots;
 *  - operator assembly (orc_mat_assemble: AT, AF in both boundary-row
 *    orders, A_uphi, LAPpsi, no-slip and stress-free) against an
 *    independent numpy restatement of src/mat_assembly.F90;
 *  - restart resampling against the reference's cheblib padding;
 *  - the namelist reader against the reference's own src/input.txt;
 *  - time stepping by analytic known answers (conductive steady state,
 *    linear decay, schemes consistent in dt, scheme orders).
 * FFTW and LAPACK are not vendored by the reference and no Fortran compiler
 * exists here, so bitwise equality with the reference binary is not
 * claimed: agreement is to rounding.
 */
#ifndef FALCON_ORACLE_H
#define FALCON_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Scheme identifiers (time_scheme_imp / time_scheme_exp of the namelist). */
enum {
  ORC_TYPE_IMEX = 0, ORC_TYPE_IMEXRK = 1, ORC_TYPE_RK = 2
};
enum {
  ORC_IMP_CN = 0, ORC_IMP_BDF2 = 1, ORC_IMP_BDF3 = 2, ORC_IMP_BDF4 = 3,
  ORC_IMP_ARS443 = 10, ORC_IMP_ARS343 = 11, ORC_IMP_BPR353 = 12,
  ORC_IMP_ARS222 = 13, ORC_IMP_ARS232 = 14, ORC_IMP_ARS233 = 15,
  ORC_IMP_NONE = 20
};
enum {
  ORC_EXP_AB2 = 0, ORC_EXP_AB3 = 1, ORC_EXP_AB4 = 2,
  ORC_EXP_ARS443 = 10, ORC_EXP_ARS343 = 11, ORC_EXP_BPR353 = 12,
  ORC_EXP_ARS222 = 13, ORC_EXP_ARS232 = 14, ORC_EXP_ARS233 = 15,
  ORC_EXP_RK2 = 20, ORC_EXP_RK4 = 21
};

typedef struct orc_params {
  int nr_max;            /* &grid Nr_max */
  int nm_max;            /* &grid Nm_max; Np_max = 3*Nm_max */
  double eta, ra, pr;    /* &physics */
  int mbc;               /* 0 = "NS" (no-slip), 1 = "SF" (stress-free) */
  int lagpts;            /* lagpts (Johnston BC interpolation points) */
  int buo_imp;           /* buo_tscheme: 1 = "IMP", 0 = "EXP" */
  double dt;             /* &timecontrol dt */
  int scheme_type;       /* ORC_TYPE_* */
  int scheme_imp;        /* ORC_IMP_* */
  int scheme_exp;        /* ORC_EXP_* */
  int l_imexrk_started;  /* l_imexrk_started */
  int l_vartimestep;     /* &timecontrol l_vartimestep: dt from the CFL condition */
  int l_optimizedt;      /* l_optimizedt: change dt only when needed */
  double cfl, dt_coef, dt_max;  /* CFL, dt_coef, dt_max */
} orc_params;

/* ---- transforms (reference: src/fourier_fftw.F90, src/chebyshev_fftw.F90) ---- */
void orc_fft(int n, const double* in, double* out, int sign);
void orc_forfft(int nm, int np, const double* ff, double* f);
void orc_invfft(int nm, int np, const double* f, double* ff);
void orc_dcheb(int nr, double* xp, double* t, double* d, double* d2);
void orc_chebtransform(int nr, const double* f, double* ft);
void orc_chebinvtran(int nr, const double* ft, double* ff);
void orc_chebinvtranD1(int nr, const double* ft, double* df);
void orc_chebinvtranD2(int nr, const double* ft, double* d2f);
void orc_chebinvtranD1D2(int nr, const double* ft, double* df, double* d2f);

/* ---- dense LU (reference: src/algebra_lapack.F90) ---- */
int orc_dgetrf(int n, double* a, int* ipiv);
void orc_dgetrs(int n, const double* a, const int* ipiv, double* b);

/* ---- nonlinear pass (reference: src/nonlin.F90:35-91), one instance ---- */
void orc_nonlin(int nm, int nr, const double* tFR, const double* omgFR,
                const double* upFR, const double* urFR, double* uphi_temp,
                double* ur_temp, double* uphi_omg, double* ur_omg);

/* ---- simulation handle ---- */
typedef struct orc_sim orc_sim;
orc_sim* orc_sim_create(const orc_params* p);
void orc_sim_destroy(orc_sim* s);
/* Initial states.  kind 0: reference perturbation (n_init, ampT as in
 * src/init.F90:277-399); kind 1: conductive profile + seeded complex Gaussian
 * noise of amplitude amp on modes 1..Nm at interior radii. */
int orc_sim_init(orc_sim* s, int kind, int n_init, double amp, uint64_t seed);
int orc_sim_set_state(orc_sim* s, const double* tFR, const double* omgFR,
                      const double* upFR, const double* urFR);
int orc_sim_get_state(const orc_sim* s, double* tFR, double* omgFR, double* upFR,
                      double* urFR, double* psi);
int orc_sim_step(orc_sim* s, int nsteps);
/* writeKE_spectral quantities at the current state:
 * out[0]=KE_tot out[1]=KE_r out[2]=KE_phi out[3]=KE_upbar out[4]=Nu_top
 * out[5]=Nu_bot out[6]=viscous dissipation out[7]=buoyancy power out[8]=time */
int orc_sim_diagnostics(orc_sim* s, double* out);
/* calculate_spectra (src/output.F90:327-355): kespec, tspec of Nm_max+1
 * modes (already x 4 pi). */
int orc_sim_spectra(orc_sim* s, double* kespec, double* tspec);
/* The u_phi balance written to upbalance_<tag> by writeKE_spectral
 * (src/output.F90:145-228): out[4 r + 0..3] = radius, d(up_0)/dt from
 * upFR_prev, advection, diffusion. */
int orc_sim_upbalance(orc_sim* s, double* out);
int orc_sim_nstep(const orc_sim* s);
/* Current time step (dt_new; changes with l_vartimestep). */
double orc_sim_dt(const orc_sim* s);
/* Host seeded-noise generator shared by the kind-1 initial state. */
void orc_noise_pair(uint64_t seed, int m, int i, double* a, double* b);
/* IMEXRK table of scheme number `scheme` (see imexrk_tables.h): out = n,
 * aD (n x n, row-major), bD, aA, bA, check_D, check_A, diag_index. */
int orc_imexrk_table(int scheme, double* out);
/* store_checkpoint / store_snapshot files (src/output.F90:359-516). */
int orc_sim_store_checkpoint(const orc_sim* s, const char* path);
int orc_sim_store_snapshot(const orc_sim* s, const char* path);
/* l_restart: restore from "<dir>/checkpoint_%05d" files (get_checkpoint_data,
 * src/init.F90:447-935, and the multistep bootstrap of src/steptime.F90:87-193
 * when l_imexrk_started is set for CN/BDF2/BDF3/BDF4).  Returns 0, -2 (file
 * missing or malformed), -3 (smaller grid), -4 (grid change with multistep
 * histories), -5 (no usable multistep histories in the file). */
int orc_sim_restart(orc_sim* s, const char* dir, int npoint, int add_pert, double ampT);
/* The operator matrices of mode n before factorisation (column-major), on
 * the grid and walls of p: kind 0 AT (R x R), 1 AF (2R x 2R), 2 A_uphi
 * (R x R), 3 LAPpsi (R x R); irk = 1 gives mat_build_IRK's boundary-row
 * order of AF (src/mat_assembly.F90:68-240 against :242-413; LAPpsi is
 * mat_build_rk, :415-462).  dt and wt multiply the diffusion operator as in
 * the reference (wt = wt_lhs_tscheme_imp).  Returns 0, or -1. */
int orc_mat_assemble(const orc_params* p, int kind, int n, double dt, double wt, int irk, double* out);
/* Number of OpenMP threads the oracle uses (0 = runtime default). */
void orc_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
