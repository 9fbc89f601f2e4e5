/*
 * falcon_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the
 * FAlCon-DNS per-time-step hot path.
 *
 * The reference (FAlCon-DNS, Fortran) advances one annulus instance with
 * `timeloop_imex` / `timeloop_imexrk` (src/steptime.F90:52,
 * src/steptime_imexrk.F90:50), whose per-step body is the nonlinear pass
 * `Nr_maxLOOP` (src/nonlin.F90:35) followed by the per-mode implicit solves
 * (`Nm_maxLOOP`, src/fourierloop.F90:156; `Get_stage_var`,
 * src/fourierloop_imexrk.F90:75).  This header is the drop-in boundary a
 * Fortran host binds through ISO_C_BINDING, and that the C++ driver
 * `falcon_run` and the Python harness bind directly.
 *
 * Conventions
 *  - Every call returns 0 on success or a negative FALCON_E* code; the text
 *    of the last error of the calling thread is in falcon_last_error().
 *  - Complex fields use the reference's Fortran layout X(Nm_max+1, Nr_max):
 *    mode fastest, element (m, r) at index m + (Nm_max+1)*r, each complex
 *    value two doubles (re, im) -- i.e. `complex(c_double_complex)` arrays.
 *  - Host pointers unless a name ends in _dev; _dev entry points take device
 *    pointers and a cudaStream_t passed as void*.
 *  - All arithmetic is IEEE FP64.  Ownership: the caller owns every array it
 *    passes; a handle owns all device memory it allocates.
 */
#ifndef FALCON_GPU_H
#define FALCON_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes ---- */
#define FALCON_OK 0
#define FALCON_EINVAL (-1)     /* bad argument / size / unsupported option */
#define FALCON_ECUDA (-2)      /* CUDA runtime error */
#define FALCON_ENOMEM (-3)     /* device or host allocation failed */
#define FALCON_ESINGULAR (-4)  /* dgetrf reported INFO != 0 on an operator */
#define FALCON_ENONFINITE (-5) /* non-finite value found in the state */
#define FALCON_EBLOWUP (-6)    /* kinetic energy above 1e10 (src/output.F90:321) */
#define FALCON_EIO (-7)        /* namelist file missing or unreadable */
#define FALCON_EBUSY (-8)      /* server queue full / admission refused */

/* ---- scheme identifiers (namelist strings, src/timeschemes.F90:42-962) ---- */
enum falcon_scheme_type { FALCON_IMEX = 0, FALCON_IMEXRK = 1, FALCON_RK = 2 };
/* IMEXRK pairs use the same number for "XXX" (implicit) and "expXXX"
 * (explicit); all 31 pairs of the reference are built, up to 8 stages
 * (KC885).  The schemes whose implicit diagonal changes by stage (diag_diff:
 * SMR333, CB3e, CB3f, CB4, LZ3L1, LZ3A4a, LZ4A1) solve each stage with the
 * operators of its own weight (src/fourierloop_imexrk.F90:134-160).
 * LZ3A4a is rejected at creation: its stages 2 and 4 have a zero implicit
 * weight, for which the reference's coupled omega-psi operator is singular
 * (its runs diverge in the first step). */
enum falcon_scheme_imp {
  FALCON_IMP_CN = 0, FALCON_IMP_BDF2 = 1, FALCON_IMP_BDF3 = 2, FALCON_IMP_BDF4 = 3,
  FALCON_IMP_ARS443 = 10, FALCON_IMP_ARS343 = 11, FALCON_IMP_BPR353 = 12,
  FALCON_IMP_ARS222 = 13, FALCON_IMP_ARS232 = 14, FALCON_IMP_ARS233 = 15, FALCON_IMP_NONE = 20,
  FALCON_IMP_EUL111 = 30, FALCON_IMP_MARS343 = 31, FALCON_IMP_IJ3 = 32, FALCON_IMP_PC2 = 33,
  FALCON_IMP_SSP332 = 34, FALCON_IMP_SSP543 = 35, FALCON_IMP_PR433 = 36, FALCON_IMP_DBM453 = 37,
  FALCON_IMP_KC343 = 38, FALCON_IMP_KC564 = 39, FALCON_IMP_FW53 = 40, FALCON_IMP_CK222 = 41,
  FALCON_IMP_BPR442 = 42, FALCON_IMP_CFN343 = 43, FALCON_IMP_BHR553 = 44, FALCON_IMP_CFN564 = 45,
  FALCON_IMP_KC774 = 46, FALCON_IMP_KC885 = 47, FALCON_IMP_SMR333 = 48, FALCON_IMP_CB3E = 49,
  FALCON_IMP_CB3F = 50, FALCON_IMP_CB4 = 51, FALCON_IMP_LZ3L1 = 52, FALCON_IMP_LZ3A4A = 53,
  FALCON_IMP_LZ4A1 = 54
};
enum falcon_scheme_exp {
  FALCON_EXP_AB2 = 0, FALCON_EXP_AB3 = 1, FALCON_EXP_AB4 = 2,
  FALCON_EXP_ARS443 = 10, FALCON_EXP_ARS343 = 11, FALCON_EXP_BPR353 = 12,
  FALCON_EXP_ARS222 = 13, FALCON_EXP_ARS232 = 14, FALCON_EXP_ARS233 = 15,
  FALCON_EXP_RK2 = 20, FALCON_EXP_RK4 = 21,
  FALCON_EXP_EUL111 = 30, FALCON_EXP_MARS343 = 31, FALCON_EXP_IJ3 = 32, FALCON_EXP_PC2 = 33,
  FALCON_EXP_SSP332 = 34, FALCON_EXP_SSP543 = 35, FALCON_EXP_PR433 = 36, FALCON_EXP_DBM453 = 37,
  FALCON_EXP_KC343 = 38, FALCON_EXP_KC564 = 39, FALCON_EXP_FW53 = 40, FALCON_EXP_CK222 = 41,
  FALCON_EXP_BPR442 = 42, FALCON_EXP_CFN343 = 43, FALCON_EXP_BHR553 = 44, FALCON_EXP_CFN564 = 45,
  FALCON_EXP_KC774 = 46, FALCON_EXP_KC885 = 47, FALCON_EXP_SMR333 = 48, FALCON_EXP_CB3E = 49,
  FALCON_EXP_CB3F = 50, FALCON_EXP_CB4 = 51, FALCON_EXP_LZ3L1 = 52, FALCON_EXP_LZ3A4A = 53,
  FALCON_EXP_LZ4A1 = 54
};

/* Namelist scalars of src/namelists.F90:52-58 (&grid, &physics,
 * &timecontrol, &output).  Np_max = 3*Nm_max, rmin = eta/(1-eta) and
 * rmax = 1/(1-eta) are derived (src/namelists.F90:105-107). */
typedef struct falcon_params {
  int nr_max, nm_max;                 /* &grid */
  double eta, ra, pr;                 /* &physics */
  int mbc;                            /* 0 = "NS", 1 = "SF" */
  double ampT;
  int l_add_pert, lagpts, n_init;
  int buo_imp;                        /* buo_tscheme: 1 = "IMP", 0 = "EXP" */
  int n_time_steps;                   /* &timecontrol */
  double dt, totaltime;
  int l_vartimestep, l_optimizedt;
  int scheme_type, scheme_imp, scheme_exp;
  int l_imexrk_started;
  double dt_coef, dt_max, cfl;
  int l_restart, n_restart, n_restart_point, n_snapshot_point;
  char tag[100];                      /* &output */
  int n_checkpoint, n_snapshot, n_KE, n_KEspec;
} falcon_params;

/* writeKE_spectral quantities (src/output.F90:122-324) of one instance. */
typedef struct falcon_diag {
  double time, dt;
  double ke, ke_r, ke_phi, ke_upbar;  /* KE_<tag> columns 3-6 */
  double nu_top, nu_bot;              /* Nusselt_<tag> */
  double vis, buo;                    /* power_<tag> */
} falcon_diag;

typedef struct falcon_handle falcon_handle;
typedef struct falcon_batch falcon_batch;
typedef struct falcon_server falcon_server;

/* ---- parameters ---- */
/* defaultNamelists, src/namelists.F90:112-146 */
int falcon_params_default(falcon_params* p);
/* readNamelists, src/namelists.F90:49-110: reads &grid, &physics,
 * &timecontrol and &output from a namelist file into *p (defaults first). */
int falcon_params_read_namelist(const char* path, falcon_params* p);
/* Maps the namelist strings time_scheme_type/_imp/_exp onto the enums. */
int falcon_params_set_scheme(falcon_params* p, const char* type, const char* imp, const char* exp);

/* ---- one instance (a batch of one) ---- */
/* solver_init, src/solver.F90:38-66: grid, operators (mat_build* +
 * dgetrf, src/mat_assembly.F90), device state. */
int falcon_create(const falcon_params* p, falcon_handle** out);
void falcon_destroy(falcon_handle* h);
/* Initial state.  kind 0: reference perturbation (init_perturbation,
 * src/init.F90:277-399, n_init and ampT of the params).  kind 1: conductive
 * profile tcon (src/init.F90:209) plus complex Gaussian noise of amplitude
 * `amp` on modes 1..Nm_max at interior radii, seeded by `seed`. */
int falcon_init_state(falcon_handle* h, int kind, double amp, uint64_t seed);
/* Fortran-layout host arrays (M,R) complex; any of them may be NULL in
 * get_state.  set_state restarts the step counter (fresh start). */
int falcon_set_state(falcon_handle* h, const double* tFR, const double* omgFR,
                     const double* upFR, const double* urFR);
int falcon_get_state(falcon_handle* h, double* tFR, double* omgFR, double* upFR,
                     double* urFR, double* psi);
/* The implicit operators from the caller's own LU factors: the output of
 * its mat_build / mat_build_IRK / mat_build_uphibar / mat_build_rk + dgetrf
 * (src/mat_assembly.F90:68-462, factorize at src/algebra_lapack.F90:14-24),
 * in the reference's arrays: AT = AT_all (Nr,Nr,Nm+1) with ipiv_T = IPIV1
 * (Nr,Nm+1); AF = AF_all (2Nr,2Nr,Nm+1) with ipiv_F = IPIV2 (2Nr,Nm+1; mode
 * 0 unused); A_uphi = A_uphi_all(:,:,1) (Nr,Nr) with ipiv_uphi (Nr);
 * LAPpsi = LAPpsi_all (Nr,Nr,Nm+1) with ipiv_lap (Nr,Nm+1; mode 0 unused),
 * for the schemes that solve it (IMEXRK not stiffly accurate, RK).  Column-
 * major factors, 1-based pivots, as LAPACK dgetrf returns them.  Replaces
 * the solves of matsolve / matsolve_real (src/algebra_lapack.F90:26-53):
 * the library applies dgetrs to unit right-hand sides on the device with
 * these factors and folds the solutions into its per-mode operators.  A
 * NULL array (with its pivots) keeps the library's own factors of that
 * operator.  Built for the handle's current dt and scheme weight (IMEX
 * wt_lhs, IMEXRK butcher_aD(diag,diag)); a later operator rebuild (a dt
 * change of a variable-dt run) uses the library's own assembly again.
 * Schemes with stage-dependent implicit diagonals are refused. */
int falcon_upload_factors(falcon_handle* h, const double* AT, const int* ipiv_T, const double* AF,
                          const int* ipiv_F, const double* A_uphi, const int* ipiv_uphi,
                          const double* LAPpsi, const int* ipiv_lap);
/* Advances nsteps time steps (the loop bodies of src/steptime.F90:196-251 /
 * src/steptime_imexrk.F90:96-190). */
int falcon_step(falcon_handle* h, int nsteps);
int falcon_diagnostics(falcon_handle* h, falcon_diag* out);
/* The run's clock after the last step: tot_time (accumulated as the
 * reference does, tot_time = tot_time + dt_new), the dt_new of that step and
 * the step count n_step.  Host bookkeeping, no device work; any pointer may
 * be NULL. */
int falcon_time(falcon_handle* h, double* tot_time, double* dt, int* n_step);
/* calculate_spectra (src/output.F90:327-355) of the current state:
 * kespec[m] = 4 pi radInt(|ur_m ur_m + up_m up_m|) and tspec[m] =
 * 4 pi radInt(|T_m|) for m = 0..Nm_max (the KEspec_<tag> and
 * Temp_spec_<tag> columns). */
int falcon_spectra(falcon_handle* h, double* kespec, double* tspec);
/* The u_phi force balance that writeKE_spectral appends to upbalance_<tag>
 * (src/output.F90:145-228): out[4 r + 0..3] for r = 0..Nr_max-1 = radius,
 * real(up_0 - upFR_prev_0)/dt, the advection -(ur d(up)/dr + ur up / r)
 * over all modes and the diffusion d2 up_0/dr2 - up_0/r^2 + (d up_0/dr)/r.
 * upFR_prev is u_phi at the start of a run and, in the IMEX multistep
 * loop, after each step's nonlinear pass (src/init.F90:253,
 * src/steptime.F90:212). */
int falcon_upbalance(falcon_handle* h, double* out);
/* Checkpoint file in the layout of store_checkpoint (src/output.F90:359-447,
 * Fortran unformatted sequential records): dt_new, tot_time, Nm_max, Nr_max
 * and the time-scheme orders; dt_array; tFR, omgFR, urFR, upFR; the history
 * arrays rhs_imp_* / rhs_exp_* of the multistep schemes (the oldest implicit
 * level, which the next step shifts out unused, is written as zero; the
 * Runge-Kutta loops write zero arrays).  Replaces the call at
 * src/steptime.F90:269-277 (and its IMEXRK and RK twins). */
int falcon_store_checkpoint(falcon_handle* h, const char* path);
/* Restores a checkpoint written by falcon_store_checkpoint (same grid and
 * scheme): state, time, dt history and the multistep histories; a
 * constant-dt run continues bit for bit.  Counterpart of read_checkpoint
 * (src/init.F90:865-935), which reads the state and dt only. */
int falcon_load_checkpoint(falcon_handle* h, const char* path);
/* l_restart = .TRUE.: restores the instance from the checkpoint files
 * "<dir>/checkpoint_%05d" (dir NULL: the working directory) the way the
 * reference starts a restarted run, replacing init_fields' restart branch
 * (src/init.F90:183-204) with get_checkpoint_data / read_checkpoint
 * (:447-935) and the restart block of timeloop_imex (src/steptime.F90:87-193):
 *  - n_restart_point names the file; a multistep scheme (CN, BDF2, BDF3,
 *    BDF4) with l_imexrk_started reads the last n_imp checkpoints (e.g. of
 *    an IMEXRK run) and builds its histories from those states
 *    (rhs_*_from_restart, src/rhs_create.F90:387-573);
 *  - another multistep restart takes the histories stored in the file, with
 *    the reference's rules for a change of order (src/init.F90:593-716);
 *  - IMEXRK and RK may restart on a larger grid (Chebyshev resampling,
 *    src/init.F90:726-861);
 *  - dt_array follows src/init.F90:566-580; l_add_pert adds ampT to tFR.
 * The first step after it follows the reference's restart step (nonlinear
 * pass first, restart rules of compute_new_dt).  With l_restart set,
 * falcon_step fails until this (or falcon_set_state / falcon_init_state)
 * has given the state. */
int falcon_restart(falcon_handle* h, const char* dir);
/* Snapshot file in the layout of store_snapshot (src/output.F90:487-516):
 * Ra, Pr, eta; dt, time; Nm_max, Nr_max; radius; tFR, omgFR, urFR, upFR. */
int falcon_store_snapshot(falcon_handle* h, const char* path);

/* ---- batches of independent instances ---- */
/* Instances are grouped by operator key (Nr, Nm, mBC, scheme, dt, Pr);
 * each group shares its implicit operators. */
int falcon_batch_create(const falcon_params* params, int n, falcon_batch** out);
/* Batches created after the call split the instances of one operator key
 * into balanced groups of at most n instances (default 128; 0: one group
 * per key).  The groups share the operators and step on separate streams,
 * so one group's nonlinear pass (FP64 pipe) can run beside another's
 * operator contractions (tensor cores).  Results do not change.  Returns
 * the previous value.  No reference counterpart (the reference steps one
 * run). */
int falcon_set_max_group_size(int n);
void falcon_batch_destroy(falcon_batch* b);
int falcon_batch_size(const falcon_batch* b);
int falcon_batch_ngroups(const falcon_batch* b);
int falcon_batch_init_state(falcon_batch* b, int kind, double amp, const uint64_t* seeds);
int falcon_batch_set_state(falcon_batch* b, int i, const double* tFR, const double* omgFR,
                           const double* upFR, const double* urFR);
/* Bulk form of falcon_batch_set_state for every instance at once (no
 * reference counterpart: the reference loads one run's state at a time).
 * Each array holds the n instances' Fortran-layout fields back to back,
 * instance i at offset sum_{j<i} 2 Nr_j (Nm_j + 1) doubles; omgFR, upFR,
 * urFR may be null (zeros).  Same result as n falcon_batch_set_state
 * calls, with one host-to-device copy per field and group and one
 * synchronisation; the arrays may be reused when the call returns. */
int falcon_batch_set_states(falcon_batch* b, const double* tFR, const double* omgFR,
                            const double* upFR, const double* urFR);
int falcon_batch_get_state(falcon_batch* b, int i, double* tFR, double* omgFR, double* upFR,
                           double* urFR, double* psi);
int falcon_batch_step(falcon_batch* b, int nsteps);
int falcon_batch_diagnostics(falcon_batch* b, falcon_diag* out /* n entries */);
/* falcon_spectra / falcon_upbalance of instance i. */
int falcon_batch_spectra(falcon_batch* b, int i, double* kespec, double* tspec);
int falcon_batch_upbalance(falcon_batch* b, int i, double* out);
/* Checkpoint / snapshot of instance i (as the falcon_handle forms).  A load
 * sets the time and step count of instance i's group: load every instance
 * of a group from checkpoints of the same run time. */
int falcon_batch_store_checkpoint(falcon_batch* b, int i, const char* path);
int falcon_batch_load_checkpoint(falcon_batch* b, int i, const char* path);
int falcon_batch_store_snapshot(falcon_batch* b, int i, const char* path);
/* falcon_restart for every instance, instance i from directory dirs[i]
 * (dirs or dirs[i] NULL: the working directory) with its own
 * n_restart_point.  Instances of one operator group step together, so
 * they must restart to the same time and dt history. */
int falcon_batch_restart(falcon_batch* b, const char* const* dirs);
/* Optional: run every step of the batch on this stream (cudaStream_t). */
int falcon_batch_set_stream(falcon_batch* b, void* stream);
/* Device bytes held by the batch (state, history, operators, scratch). */
size_t falcon_batch_device_bytes(const falcon_batch* b);

/* ---- kernel-level entry points (device pointers) ---- */
/* Nr_maxLOOP (src/nonlin.F90:35-91) for `nb` instances that share
 * (Nr, Nm).  Device layout X[r][m][b] (instance fastest), double2 per
 * element, for the four inputs and the four products. */
int falcon_nonlin_dev(int nr, int nm, int nb, const double* t_dev, const double* omg_dev,
                      const double* up_dev, const double* ur_dev, double* uphi_t_dev,
                      double* ur_t_dev, double* uphi_omg_dev, double* ur_omg_dev, void* stream);
/* Allocation-free form of falcon_nonlin_dev (no counterpart in the
 * reference): same arguments, layout and bits, but the library allocates no
 * device memory -- its FFT tables are built on the host and copied into a
 * fixed 80 KiB static device array -- for hosts that own all device memory
 * through their own budgeted pool, or that step in loops where
 * cudaMalloc/cudaFree would synchronise the device.  Limit: 3*nm <= 4096,
 * else FALCON_EINVAL.  Unlike falcon_nonlin_dev it is asynchronous on
 * `stream`: it returns once the table copies and the kernel are queued, so
 * synchronise the stream before reading the outputs (a kernel fault shows
 * there, not in the return code).  The first call on a device resolves the
 * array's device address (make it before any stream capture); every call
 * overwrites the table region it uses; calls whose kernels overlap on the
 * GPU share the array and race, so serialise them. */
int falcon_nonlin_noalloc_dev(int nr, int nm, int nb, const double* t_dev, const double* omg_dev,
                              const double* up_dev, const double* ur_dev, double* uphi_t_dev,
                              double* ur_t_dev, double* uphi_omg_dev, double* ur_omg_dev, void* stream);
/* Host-array form of falcon_nonlin_dev for one instance, Fortran layout;
 * copies in and out inside the call. */
int falcon_nonlin(int nr, int nm, const double* tFR, const double* omgFR, const double* upFR,
                  const double* urFR, double* uphi_temp_FR, double* ur_temp_FR,
                  double* uphi_omg_FR, double* ur_omg_FR);
/* matsolve (src/algebra_lapack.F90:26-38): for each of `nsys` systems,
 * solves A x = b with the LU factors and pivots of dgetrf (column-major
 * n x n, 1-based pivots), `nrhs` real right-hand sides per system.
 * lu: nsys*n*n, ipiv: nsys*n, b: nsys*nrhs*n (solved in place). */
int falcon_getrs_batched_dev(int n, int nsys, int nrhs, const double* lu_dev,
                             const int* ipiv_dev, double* b_dev, void* stream);
/* chebtransform / chebinvtran / chebinvtranD1 / chebinvtranD2
 * (src/chebyshev_fftw.F90:124-352) applied to `ncol` complex columns of
 * length nr stored contiguously (column-major, nr x ncol). */
int falcon_cheb_fwd_dev(int nr, int ncol, const double* in_dev, double* out_dev, void* stream);
int falcon_cheb_inv_dev(int nr, int ncol, const double* in_dev, double* out_dev, void* stream);
int falcon_cheb_d1_dev(int nr, int ncol, const double* in_dev, double* out_dev, void* stream);
int falcon_cheb_d2_dev(int nr, int ncol, const double* in_dev, double* out_dev, void* stream);
/* chebinvtranD1D2 (src/chebyshev_fftw.F90:369-427): first and second radial
 * derivatives of the same coefficient columns in one call. */
int falcon_cheb_d1d2_dev(int nr, int ncol, const double* in_dev, double* d1_dev, double* d2_dev, void* stream);

/* ---- serving ---- */
/* A request loop that admits simulation requests by device-memory
 * footprint, keeps their state resident, steps every admitted request
 * together each iteration, and retires each one at its horizon. */
int falcon_server_create(size_t hbm_budget_bytes, int max_active, falcon_server** out);
void falcon_server_destroy(falcon_server* s);
/* Queues a request; *id receives its identifier. */
int falcon_server_submit(falcon_server* s, const falcon_params* p, uint64_t seed, int horizon,
                         int64_t* id);
/* One serving iteration: admit what fits, queue one step of every active
 * group on its stream, retire finished requests (synchronising only the
 * groups read this iteration).  *n_active / *n_queued report the sizes. */
int falcon_server_iterate(falcon_server* s, int* n_active, int* n_queued);
/* Queues a request whose initial state is given (Fortran-layout host
 * arrays, copied; omgFR, upFR, urFR may be NULL for zeros) instead of the
 * seeded conductive-plus-noise state. */
int falcon_server_submit_state(falcon_server* s, const falcon_params* p, const double* tFR, const double* omgFR,
                               const double* upFR, const double* urFR, int horizon, int64_t* id);
/* 1 when request `id` has finished; its final diagnostics in *out and, if
 * tFR is not NULL, its final temperature field (Fortran layout). */
int falcon_server_poll(falcon_server* s, int64_t id, int* done, falcon_diag* out, double* tFR);
/* A finished request's status and fields: *status is FALCON_OK when it
 * reached its horizon, FALCON_EBLOWUP (kinetic energy above 1e10, the
 * reference's stop at src/output.F90:321-323) or FALCON_ENONFINITE when a
 * check at its n_KE cadence retired it early (the other requests of its
 * group keep running); the fields are its state at that step (any pointer
 * may be NULL).  *done = 0 while it runs. */
int falcon_server_result(falcon_server* s, int64_t id, int* done, int* status, falcon_diag* out, double* tFR,
                         double* omgFR, double* upFR, double* urFR);
/* Steps request `id` has taken so far. */
int falcon_server_steps(falcon_server* s, int64_t id, int* steps);

/* ---- measurement hooks ---- */
/* Per-kernel-class statistics of `nsteps` steps of a batch, timed with CUDA
 * events around every launch on its group's stream, the groups of a step
 * one after another (the steps advance the state like falcon_batch_step).  flops is the algorithmic FP64 operation
 * count of the launches: 2*rows*K*N per GEMM, 5 P log2 P per complex FFT of
 * length P (four per radial line) plus the grid products. */
typedef struct falcon_kernel_stat {
  char name[32];
  int launches;
  double ms;
  double flops;
} falcon_kernel_stat;
int falcon_batch_profile(falcon_batch* b, int nsteps, falcon_kernel_stat* stats, int max_stats, int* nstats);
/* Number of kernels this library has launched in the calling process
 * (kernels inside a replayed step graph count once per replay). */
long long falcon_launch_count(void);
/* Steady-state steps (from the second step of a run on) are captured once
 * per history phase into CUDA graphs and replayed; 0 turns this off for the
 * whole process (every kernel launched directly), 1 turns it back on.
 * Returns the previous setting.  Results are identical either way.
 * No reference counterpart (launch mechanics of the GPU step). */
int falcon_set_step_graphs(int enable);
/* Operator contractions (the radial derivative / Laplacian and per-mode
 * solve products) run on one of three paths: FP64 FMA tiles; the bf16
 * tensor cores by exact integer slicing of the FP64 operands on warp-level
 * mma.sync; the same slices on the 5th-generation tcgen05 MMA with
 * accumulators in tensor memory.  The two sliced paths give the same bits;
 * all give FP64-accurate results (the slices: error of the order of
 * K 2^-56 max|A_row| max|X_col|), and the sliced ones are several times
 * faster on GB300, whose FP64 pipe is ~500x slower than its bf16 tensor
 * cores.  Modes:
 *   4 (default) autotuned: the first time a contraction shape runs outside
 *     graph capture, every available path is timed on it (the device
 *     otherwise idle, L2 flushed before each timed run, as a step's
 *     operators come from HBM) and the fastest is kept for that shape (the
 *     path of mode 2's rules unless another is at least 10 % faster; see
 *     falcon_set_tune_cache; the library holds a 256 MiB device buffer
 *     for the flush from the first measurement on);
 *   3 tcgen05 for every contraction with a slice view of its operator
 *     (mma.sync where that view has no tensor map): the same bits as 1;
 *   2 fixed rules: tcgen05 for contractions of at least two 128 x 24 tiles
 *     per SM, mma.sync for the other ones of at least 16 columns per batch
 *     entry, FMA for narrower ones;
 *   1 mma.sync for every contraction with a slice view;
 *   0 FMA only.
 * Applies to launches after the call (step graphs already captured keep
 * their paths).  Returns the previous mode; an unknown mode selects 4.
 * No counterpart in the reference, which uses LAPACK dgetrs
 * (src/algebra_lapack.F90). */
int falcon_set_gemm_mode(int mode);
/* Contraction tuning cache of mode 4: decisions are read from `path` (if it
 * exists) and every new decision is appended to it, so that later processes
 * take the same paths without measuring.  Text format: the header line
 * "falcon-contraction-tuning 2", then one line per decision
 *   <device> <rows> <K> <N> <batch> <w> <per_mode> <reuse> <path> <us_0> <us_1> <us_2> <us_3> <us_4> <us_5>
 * device = CUDA device name with blanks as '_' plus "_sm<SM count>"
 * (falcon_device_tag); rows, K, N, batch = the contraction's shape (rows x K
 * operator, N columns per batch entry); w = slice format in bits (6 or 7);
 * per_mode = 1 when every batch entry has its own columns (2 + n: n row
 * blocks of one operator narrower than 16 columns, merged into one tcgen05
 * launch, path 2, or run one after another, path 0); reuse = 1 when
 * the X slice planes were made by the contraction before; path 0 FMA
 * tiles of the cost model's shape, 1 mma.sync, 2 tcgen05, 3 / 4 / 5 FMA
 * tiles of the best shape 16 / 32 / 64 columns wide (the same bits as 0);
 * us_p = measured microseconds per contraction on path p (-1: not
 * measured).  NULL or "" detaches the file (decisions stay in
 * memory).  The environment variable FALCON_TUNE_CACHE names a file when
 * this is not called.  Returns FALCON_EINVAL for a file with another
 * header or a malformed line. */
int falcon_set_tune_cache(const char* path);
/* Decisions held (and, in *measured, how many this process measured). */
int falcon_tune_entries(long long* measured);
/* Forget every decision held in memory (the file is kept); returns their number. */
int falcon_tune_clear(void);
/* The decision for one shape (path 0-5, -1 if none), with the measured times
 * (6 floats, may be NULL). */
int falcon_tune_lookup(const char* device, int rows, int K, int N, int batch, int w, int per_mode, int reuse,
                       float* us);
/* The device key of the tuning cache for the current device. */
const char* falcon_device_tag(void);

/* ---- misc ---- */
const char* falcon_last_error(void);
const char* falcon_version(void);
/* Measured FP64 FMA throughput of the current device in GFLOP/s (a short
 * self-timed kernel), used as the roofline denominator. */
double falcon_fp64_peak_gflops(void);
/* Same for the FP64 tensor-core path (mma.sync f64), for comparison. */
double falcon_fp64_mma_peak_gflops(void);

#ifdef __cplusplus
}
#endif
#endif /* FALCON_GPU_H */
