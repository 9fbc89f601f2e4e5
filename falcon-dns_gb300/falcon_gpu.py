"""Python binding of libfalcon_gpu (the C ABI declared in include/falcon_gpu.h).

Mirrors the reference's driver interface for the time-step path:
``solver_init`` (src/solver.F90:38-66) -> :class:`Instance` / :class:`Batch`
construction, ``timeloop_*`` step bodies -> :meth:`step`, and
``writeKE_spectral`` (src/output.F90:122-324) -> :meth:`diagnostics`.  Fields
are numpy complex128 arrays of shape (Nr_max, Nm_max+1), i.e. the Fortran
(Nm_max+1, Nr_max) layout, mode fastest.

There is no CPU fallback: importing works anywhere, but creating an instance
raises if the CUDA library or a GPU is missing.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libfalcon_gpu.so")

FALCON_IMEX, FALCON_IMEXRK, FALCON_RK = 0, 1, 2
IMP = {"CN": 0, "BDF2": 1, "BDF3": 2, "BDF4": 3, "ARS443": 10, "ARS343": 11, "BPR353": 12,
       "ARS222": 13, "NONE": 20}
EXP = {"AB2": 0, "AB3": 1, "AB4": 2, "expARS443": 10, "expARS343": 11, "expBPR353": 12,
       "expARS222": 13, "RK2": 20, "RK4": 21}
TYPE = {"IMEX": 0, "IMEXRK": 1, "RK": 2}
SCHEMES = {
    "CNAB2": ("IMEX", "CN", "AB2"),
    "CNAB3": ("IMEX", "CN", "AB3"),
    "SBDF2": ("IMEX", "BDF2", "AB2"),
    "SBDF3": ("IMEX", "BDF3", "AB3"),
    "SBDF4": ("IMEX", "BDF4", "AB4"),
    "ARS443": ("IMEXRK", "ARS443", "expARS443"),
    "ARS343": ("IMEXRK", "ARS343", "expARS343"),
    "BPR353": ("IMEXRK", "BPR353", "expBPR353"),
    "ARS222": ("IMEXRK", "ARS222", "expARS222"),
    "RK2": ("RK", "NONE", "RK2"),
    "RK4": ("RK", "NONE", "RK4"),
}
# IMEXRK pairs "XXX" / "expXXX" (same number for both halves)
IMEXRK_IDS = {"ARS232": 14, "ARS233": 15, "EUL111": 30, "MARS343": 31, "IJ3": 32, "PC2": 33, "SSP332": 34,
              "SSP543": 35, "PR433": 36, "DBM453": 37, "KC343": 38, "KC564": 39, "FW53": 40, "CK222": 41,
              "BPR442": 42, "CFN343": 43, "BHR553": 44, "CFN564": 45, "KC774": 46, "KC885": 47,
              "SMR333": 48, "CB3e": 49, "CB3f": 50, "CB4": 51, "LZ3L1": 52, "LZ3A4a": 53, "LZ4A1": 54}
for _n, _i in IMEXRK_IDS.items():
    IMP[_n] = _i
    EXP["exp" + _n] = _i
    SCHEMES[_n] = ("IMEXRK", _n, "exp" + _n)


class FalconParams(ctypes.Structure):
    _fields_ = [
        ("nr_max", ctypes.c_int), ("nm_max", ctypes.c_int),
        ("eta", ctypes.c_double), ("ra", ctypes.c_double), ("pr", ctypes.c_double),
        ("mbc", ctypes.c_int), ("ampT", ctypes.c_double),
        ("l_add_pert", ctypes.c_int), ("lagpts", ctypes.c_int), ("n_init", ctypes.c_int),
        ("buo_imp", ctypes.c_int), ("n_time_steps", ctypes.c_int),
        ("dt", ctypes.c_double), ("totaltime", ctypes.c_double),
        ("l_vartimestep", ctypes.c_int), ("l_optimizedt", ctypes.c_int),
        ("scheme_type", ctypes.c_int), ("scheme_imp", ctypes.c_int), ("scheme_exp", ctypes.c_int),
        ("l_imexrk_started", ctypes.c_int),
        ("dt_coef", ctypes.c_double), ("dt_max", ctypes.c_double), ("cfl", ctypes.c_double),
        ("l_restart", ctypes.c_int), ("n_restart", ctypes.c_int), ("n_restart_point", ctypes.c_int),
        ("n_snapshot_point", ctypes.c_int), ("tag", ctypes.c_char * 100),
        ("n_checkpoint", ctypes.c_int), ("n_snapshot", ctypes.c_int), ("n_KE", ctypes.c_int),
        ("n_KEspec", ctypes.c_int),
    ]


class FalconDiag(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("time", "dt", "ke", "ke_r", "ke_phi", "ke_upbar", "nu_top", "nu_bot", "vis", "buo")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


DIAG_DTYPE = np.dtype([(n, np.float64) for n, _ in FalconDiag._fields_])


class KernelStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_int), ("ms", ctypes.c_double),
                ("flops", ctypes.c_double)]


class FalconError(RuntimeError):
    pass


_lib = None
EXPORTS = (
    "falcon_params_default", "falcon_params_read_namelist", "falcon_params_set_scheme",
    "falcon_create", "falcon_destroy", "falcon_init_state", "falcon_set_state", "falcon_get_state",
    "falcon_step", "falcon_diagnostics", "falcon_batch_create", "falcon_batch_destroy",
    "falcon_batch_size", "falcon_batch_ngroups", "falcon_batch_init_state", "falcon_batch_set_state",
    "falcon_batch_set_states", "falcon_set_max_group_size",
    "falcon_batch_get_state", "falcon_batch_step", "falcon_batch_diagnostics", "falcon_batch_set_stream",
    "falcon_batch_device_bytes", "falcon_nonlin_dev", "falcon_nonlin", "falcon_getrs_batched_dev",
    "falcon_cheb_fwd_dev", "falcon_cheb_inv_dev", "falcon_cheb_d1_dev", "falcon_cheb_d2_dev",
    "falcon_server_create", "falcon_server_destroy", "falcon_server_submit", "falcon_server_iterate",
    "falcon_server_poll", "falcon_last_error", "falcon_version", "falcon_fp64_peak_gflops",
    "falcon_batch_profile", "falcon_launch_count", "falcon_fp64_mma_peak_gflops",
    "falcon_nonlin_noalloc_dev", "falcon_set_step_graphs", "falcon_store_checkpoint", "falcon_load_checkpoint",
    "falcon_store_snapshot", "falcon_batch_store_checkpoint", "falcon_batch_load_checkpoint",
    "falcon_batch_store_snapshot", "falcon_restart", "falcon_batch_restart", "falcon_set_gemm_mode",
    "falcon_upload_factors", "falcon_cheb_d1d2_dev", "falcon_spectra", "falcon_upbalance",
    "falcon_batch_spectra", "falcon_batch_upbalance", "falcon_time", "falcon_server_submit_state",
    "falcon_server_result", "falcon_server_steps", "falcon_set_tune_cache", "falcon_tune_entries",
    "falcon_tune_clear", "falcon_tune_lookup", "falcon_device_tag",
)


def lib():
    """Load libfalcon_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FalconError("libfalcon_gpu.so is not built: run falcon-dns_gb300/build.py")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    dp, vp, ip = P(ctypes.c_double), ctypes.c_void_p, ctypes.c_int
    pp = P(FalconParams)
    L.falcon_last_error.restype = ctypes.c_char_p
    L.falcon_version.restype = ctypes.c_char_p
    L.falcon_params_default.argtypes = [pp]
    L.falcon_params_read_namelist.argtypes = [ctypes.c_char_p, pp]
    L.falcon_params_set_scheme.argtypes = [pp, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
    L.falcon_create.argtypes = [pp, P(vp)]
    L.falcon_destroy.argtypes = [vp]
    L.falcon_destroy.restype = None
    L.falcon_init_state.argtypes = [vp, ip, ctypes.c_double, ctypes.c_uint64]
    L.falcon_set_state.argtypes = [vp, dp, dp, dp, dp]
    L.falcon_get_state.argtypes = [vp, dp, dp, dp, dp, dp]
    L.falcon_step.argtypes = [vp, ip]
    L.falcon_diagnostics.argtypes = [vp, P(FalconDiag)]
    L.falcon_batch_create.argtypes = [pp, ip, P(vp)]
    L.falcon_batch_destroy.argtypes = [vp]
    L.falcon_batch_destroy.restype = None
    L.falcon_batch_size.argtypes = [vp]
    L.falcon_batch_ngroups.argtypes = [vp]
    L.falcon_batch_init_state.argtypes = [vp, ip, ctypes.c_double, P(ctypes.c_uint64)]
    L.falcon_batch_set_state.argtypes = [vp, ip, dp, dp, dp, dp]
    L.falcon_batch_set_states.argtypes = [vp, dp, dp, dp, dp]
    L.falcon_set_max_group_size.argtypes = [ip]
    L.falcon_batch_get_state.argtypes = [vp, ip, dp, dp, dp, dp, dp]
    L.falcon_batch_step.argtypes = [vp, ip]
    L.falcon_batch_diagnostics.argtypes = [vp, P(FalconDiag)]
    L.falcon_batch_set_stream.argtypes = [vp, vp]
    L.falcon_batch_device_bytes.argtypes = [vp]
    L.falcon_batch_device_bytes.restype = ctypes.c_size_t
    L.falcon_nonlin_dev.argtypes = [ip, ip, ip] + [ctypes.c_void_p] * 8 + [vp]
    L.falcon_nonlin.argtypes = [ip, ip] + [dp] * 8
    L.falcon_nonlin_noalloc_dev.argtypes = [ip, ip, ip] + [ctypes.c_void_p] * 8 + [vp]
    L.falcon_getrs_batched_dev.argtypes = [ip, ip, ip, vp, vp, vp, vp]
    for f in ("falcon_cheb_fwd_dev", "falcon_cheb_inv_dev", "falcon_cheb_d1_dev", "falcon_cheb_d2_dev"):
        getattr(L, f).argtypes = [ip, ip, vp, vp, vp]
    L.falcon_server_create.argtypes = [ctypes.c_size_t, ip, P(vp)]
    L.falcon_server_destroy.argtypes = [vp]
    L.falcon_server_destroy.restype = None
    L.falcon_server_submit.argtypes = [vp, pp, ctypes.c_uint64, ip, P(ctypes.c_int64)]
    L.falcon_server_iterate.argtypes = [vp, P(ctypes.c_int), P(ctypes.c_int)]
    L.falcon_server_poll.argtypes = [vp, ctypes.c_int64, P(ctypes.c_int), P(FalconDiag), dp]
    L.falcon_server_submit_state.argtypes = [vp, pp, dp, dp, dp, dp, ip, P(ctypes.c_int64)]
    L.falcon_server_result.argtypes = [vp, ctypes.c_int64, P(ctypes.c_int), P(ctypes.c_int), P(FalconDiag), dp, dp,
                                       dp, dp]
    L.falcon_server_steps.argtypes = [vp, ctypes.c_int64, P(ctypes.c_int)]
    L.falcon_fp64_peak_gflops.restype = ctypes.c_double
    L.falcon_fp64_mma_peak_gflops.restype = ctypes.c_double
    L.falcon_batch_profile.argtypes = [vp, ip, P(KernelStat), ip, P(ctypes.c_int)]
    L.falcon_launch_count.restype = ctypes.c_longlong
    L.falcon_set_step_graphs.argtypes = [ip]
    for f in ("falcon_store_checkpoint", "falcon_load_checkpoint", "falcon_store_snapshot"):
        getattr(L, f).argtypes = [vp, ctypes.c_char_p]
    for f in ("falcon_batch_store_checkpoint", "falcon_batch_load_checkpoint", "falcon_batch_store_snapshot"):
        getattr(L, f).argtypes = [vp, ip, ctypes.c_char_p]
    L.falcon_restart.argtypes = [vp, ctypes.c_char_p]
    L.falcon_upload_factors.argtypes = [vp, dp, P(ctypes.c_int), dp, P(ctypes.c_int), dp, P(ctypes.c_int), dp,
                                        P(ctypes.c_int)]
    L.falcon_cheb_d1d2_dev.argtypes = [ip, ip, vp, vp, vp, vp]
    L.falcon_spectra.argtypes = [vp, dp, dp]
    L.falcon_upbalance.argtypes = [vp, dp]
    L.falcon_batch_spectra.argtypes = [vp, ip, dp, dp]
    L.falcon_batch_upbalance.argtypes = [vp, ip, dp]
    L.falcon_batch_restart.argtypes = [vp, P(ctypes.c_char_p)]
    L.falcon_set_gemm_mode.argtypes = [ip]
    L.falcon_set_tune_cache.argtypes = [ctypes.c_char_p]
    L.falcon_tune_entries.argtypes = [P(ctypes.c_longlong)]
    L.falcon_tune_lookup.argtypes = [ctypes.c_char_p, ip, ip, ip, ip, ip, ip, ip, P(ctypes.c_float)]
    L.falcon_device_tag.restype = ctypes.c_char_p
    _lib = L
    return L


def check(rc):
    if rc != 0:
        msg = lib().falcon_last_error().decode()
        raise FalconError(f"falcon error {rc}: {msg}")
    return rc


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def default_params():
    p = FalconParams()
    check(lib().falcon_params_default(ctypes.byref(p)))
    return p


def read_namelist(path):
    """readNamelists (src/namelists.F90:49-110) through the C ABI."""
    p = FalconParams()
    check(lib().falcon_params_read_namelist(str(path).encode(), ctypes.byref(p)))
    return p


def make_params(nr, nm, scheme="CNAB2", eta=0.35, ra=1e5, pr=1.0, dt=1e-5, mbc="NS", lagpts=16,
                buo="IMP", vartimestep=False, optimizedt=False, cfl=0.9, dt_coef=2.0, dt_max=3e-5,
                imexrk_started=False, restart=False, restart_point=0, add_pert=False, ampT=None):
    p = default_params()
    p.nr_max, p.nm_max, p.eta, p.ra, p.pr, p.dt = nr, nm, eta, ra, pr, dt
    p.mbc = 0 if mbc == "NS" else 1
    p.lagpts = lagpts
    p.buo_imp = 1 if buo == "IMP" else 0
    p.l_vartimestep = 1 if vartimestep else 0
    p.l_optimizedt = 1 if optimizedt else 0
    p.cfl, p.dt_coef, p.dt_max = cfl, dt_coef, dt_max
    p.l_imexrk_started = 1 if imexrk_started else 0
    p.l_restart = 1 if restart else 0
    p.n_restart_point = restart_point
    p.l_add_pert = 1 if add_pert else 0
    if ampT is not None:
        p.ampT = ampT
    typ, imp, exp = SCHEMES[scheme]
    check(lib().falcon_params_set_scheme(ctypes.byref(p), typ.encode(), imp.encode(), exp.encode()))
    return p


def _field(shape):
    return np.empty(shape, np.complex128)


class Batch:
    """Independent annulus instances stepped together on the GPU."""

    def __init__(self, params):
        params = list(params)
        arr = (FalconParams * len(params))(*params)
        h = ctypes.c_void_p()
        check(lib().falcon_batch_create(arr, len(params), ctypes.byref(h)))
        self.h = h
        self.params = params
        self.n = len(params)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            lib().falcon_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ngroups(self):
        return lib().falcon_batch_ngroups(self.h)

    @property
    def device_bytes(self):
        return lib().falcon_batch_device_bytes(self.h)

    def init_noise(self, seeds, amp=1e-3):
        s = (ctypes.c_uint64 * self.n)(*[int(x) for x in seeds])
        check(lib().falcon_batch_init_state(self.h, 1, amp, s))

    def init_reference(self):
        check(lib().falcon_batch_init_state(self.h, 0, 0.0, None))

    def set_state(self, i, t, om=None, up=None, ur=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.complex128) for a in (t, om, up, ur)]
        check(lib().falcon_batch_set_state(self.h, i, *[_dp(a) for a in arrs]))

    def set_states(self, t, om=None, up=None, ur=None):
        """Every instance's state at once (falcon_batch_set_states).  Each
        field is either one contiguous complex128 array holding the
        instances' (Nr, Nm + 1) arrays back to back in instance order (used
        in place, e.g. a view of pinned memory) or a list of n such arrays
        (concatenated on the host first)."""
        total = sum(p.nr_max * (p.nm_max + 1) for p in self.params)

        def flat(a):
            if a is None:
                return None
            if isinstance(a, (list, tuple)):
                if len(a) != self.n:
                    raise ValueError("expected %d arrays" % self.n)
                a = np.concatenate([np.asarray(x, np.complex128).ravel() for x in a])
            a = np.ascontiguousarray(a, np.complex128)
            if a.size != total:
                raise ValueError("expected %d complex values, got %d" % (total, a.size))
            return a

        arrs = [flat(a) for a in (t, om, up, ur)]
        check(lib().falcon_batch_set_states(self.h, *[_dp(a) for a in arrs]))

    def get_state(self, i):
        p = self.params[i]
        shape = (p.nr_max, p.nm_max + 1)
        arrs = [_field(shape) for _ in range(5)]
        check(lib().falcon_batch_get_state(self.h, i, *[_dp(a) for a in arrs]))
        return dict(zip(("T", "omg", "up", "ur", "psi"), arrs))

    def step(self, n=1):
        check(lib().falcon_batch_step(self.h, n))

    def set_stream(self, stream_ptr):
        check(lib().falcon_batch_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def diagnostics(self):
        out = (FalconDiag * self.n)()
        check(lib().falcon_batch_diagnostics(self.h, out))
        return [d.as_dict() for d in out]

    def spectra(self, i):
        """calculate_spectra of instance i: (KEspec, Temp_spec), Nm_max + 1 modes."""
        M = self.params[i].nm_max + 1
        ke, ts = np.zeros(M), np.zeros(M)
        check(lib().falcon_batch_spectra(self.h, i, _dp(ke), _dp(ts)))
        return ke, ts

    def upbalance(self, i):
        """The u_phi balance of instance i: (Nr, 4) = radius, d(up_0)/dt, advection, diffusion."""
        out = np.zeros((self.params[i].nr_max, 4))
        check(lib().falcon_batch_upbalance(self.h, i, _dp(out)))
        return out

    def diagnostics_array(self):
        """The same values as diagnostics() in one numpy structured array
        (fields time, dt, ke, ...; one record per instance), without the
        per-instance Python objects."""
        out = np.zeros(self.n, DIAG_DTYPE)
        check(lib().falcon_batch_diagnostics(self.h, out.ctypes.data_as(ctypes.POINTER(FalconDiag))))
        return out

    def store_checkpoint(self, i, path):
        """store_checkpoint layout (Fortran unformatted records) of instance i."""
        check(lib().falcon_batch_store_checkpoint(self.h, i, os.fsencode(path)))

    def load_checkpoint(self, i, path):
        """Restore instance i (state, time, dt and multistep histories)."""
        check(lib().falcon_batch_load_checkpoint(self.h, i, os.fsencode(path)))

    def store_snapshot(self, i, path):
        """store_snapshot layout of instance i."""
        check(lib().falcon_batch_store_snapshot(self.h, i, os.fsencode(path)))

    def restart(self, dirs):
        """l_restart: every instance from "<dirs[i]>/checkpoint_%05d" (its n_restart_point)."""
        arr = (ctypes.c_char_p * self.n)(*[os.fsencode(str(d)) for d in dirs])
        check(lib().falcon_batch_restart(self.h, arr))

    def profile(self, nsteps):
        """Per-kernel-class CUDA-event times of `nsteps` steps (advances the state)."""
        stats = (KernelStat * 8)()
        n = ctypes.c_int()
        check(lib().falcon_batch_profile(self.h, nsteps, stats, 8, ctypes.byref(n)))
        return {stats[i].name.decode(): {"launches": stats[i].launches, "ms": stats[i].ms,
                                         "flops": stats[i].flops} for i in range(n.value)}


class Instance(Batch):
    """One annulus instance (a batch of one)."""

    def __init__(self, params):
        super().__init__([params])

    def init_noise(self, seed, amp=1e-3):
        super().init_noise([seed], amp)

    def get_state(self, i=0):
        return super().get_state(0)

    def set_state(self, t, om=None, up=None, ur=None):
        super().set_state(0, t, om, up, ur)

    def diagnostics(self):
        return super().diagnostics()[0]

    def spectra(self, i=0):
        return super().spectra(0)

    def upbalance(self, i=0):
        return super().upbalance(0)

    def store_checkpoint(self, path):
        super().store_checkpoint(0, path)

    def load_checkpoint(self, path):
        super().load_checkpoint(0, path)

    def restart(self, directory):
        super().restart([directory])

    def store_snapshot(self, path):
        super().store_snapshot(0, path)


class Server:
    """Continuous-batching request loop (falcon_server_*).

    submit() queues a simulation request (seeded noise initial state, a
    horizon in steps); iterate() admits queued requests by device footprint,
    steps every admitted request once and retires finished ones; poll()
    returns (done, diagnostics, final temperature spectrum)."""

    def __init__(self, hbm_budget_bytes, max_active=0):
        self.h = ctypes.c_void_p()
        check(lib().falcon_server_create(int(hbm_budget_bytes), int(max_active), ctypes.byref(self.h)))
        self.shape = {}

    def submit(self, params, seed, horizon):
        i = ctypes.c_int64()
        check(lib().falcon_server_submit(self.h, ctypes.byref(params), int(seed), int(horizon), ctypes.byref(i)))
        self.shape[i.value] = (params.nr_max, params.nm_max + 1)
        return i.value

    def submit_state(self, params, t, om=None, up=None, ur=None, horizon=1):
        """A request from a given initial state (Fortran-layout (Nr, Nm+1) complex arrays)."""
        arrs = [None if a is None else np.ascontiguousarray(a, np.complex128) for a in (t, om, up, ur)]
        i = ctypes.c_int64()
        check(lib().falcon_server_submit_state(self.h, ctypes.byref(params), *[_dp(a) for a in arrs], int(horizon),
                                               ctypes.byref(i)))
        self.shape[i.value] = (params.nr_max, params.nm_max + 1)
        return i.value

    def result(self, rid):
        """(done, status, diagnostics, fields dict) of a request; status 0 at
        its horizon, FALCON_EBLOWUP (-6) / FALCON_ENONFINITE (-5) when
        retired early."""
        done, status, diag = ctypes.c_int(), ctypes.c_int(), FalconDiag()
        f = [np.empty(self.shape[rid], np.complex128) for _ in range(4)]
        check(lib().falcon_server_result(self.h, rid, ctypes.byref(done), ctypes.byref(status), ctypes.byref(diag),
                                         *[_dp(a) for a in f]))
        if not done.value:
            return False, status.value, None, None
        return True, status.value, diag.as_dict(), dict(zip(("T", "omg", "up", "ur"), f))

    def steps(self, rid):
        n = ctypes.c_int()
        check(lib().falcon_server_steps(self.h, rid, ctypes.byref(n)))
        return n.value

    def iterate(self):
        na, nq = ctypes.c_int(), ctypes.c_int()
        check(lib().falcon_server_iterate(self.h, ctypes.byref(na), ctypes.byref(nq)))
        return na.value, nq.value

    def poll(self, rid, want_state=False):
        done = ctypes.c_int()
        diag = FalconDiag()
        t = None
        if want_state:
            t = np.empty(self.shape[rid], np.complex128)
        check(lib().falcon_server_poll(self.h, rid, ctypes.byref(done), ctypes.byref(diag),
                                       _dp(t) if t is not None else None))
        return bool(done.value), (diag.as_dict() if done.value else None), (t if done.value else None)

    def close(self):
        if self.h:
            lib().falcon_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def nonlin(nm, t, om, up, ur):
    """Nr_maxLOOP for one instance through the host-array C entry point."""
    ins = [np.ascontiguousarray(a, np.complex128) for a in (t, om, up, ur)]
    outs = [np.empty_like(ins[0]) for _ in range(4)]
    check(lib().falcon_nonlin(ins[0].shape[0], nm, *[_dp(a) for a in ins], *[_dp(o) for o in outs]))
    return outs


def fp64_peak_gflops():
    return lib().falcon_fp64_peak_gflops()


def fp64_mma_peak_gflops():
    return lib().falcon_fp64_mma_peak_gflops()


def launch_count():
    return lib().falcon_launch_count()


def set_max_group_size(n):
    """Largest group of batches created afterwards (default 128; 0: one group
    per operator key); groups of one key share operators and run on separate
    streams.  Returns the previous value."""
    return lib().falcon_set_max_group_size(int(n))


def set_gemm_mode(mode):
    """Operator contraction paths: 4 (default) the fastest measured per shape
    (autotuned, see set_tune_cache); 3 tcgen05 for every sliced contraction;
    2 fixed rules (tcgen05 where a contraction fills the GPU, mma.sync for
    other ones of >= 16 columns, FMA below); 1 mma.sync for every sliced
    contraction (the same bits as 3); 0 FP64 FMA tiles.  Returns the
    previous mode."""
    return lib().falcon_set_gemm_mode(int(mode))


PATHS = ("fma", "mma_sync", "tcgen05", "fma_ncol16", "fma_ncol32", "fma_ncol64")


def set_tune_cache(path):
    """Read the autotuner's decisions from `path` and append new ones to it
    (None detaches the file)."""
    check(lib().falcon_set_tune_cache(os.fsencode(str(path)) if path else None))


def tune_entries():
    """(decisions held, decisions this process measured)."""
    m = ctypes.c_longlong()
    n = lib().falcon_tune_entries(ctypes.byref(m))
    return n, m.value


def tune_clear():
    """Forget the decisions held in memory; returns their number."""
    return lib().falcon_tune_clear()


def tune_lookup(device, rows, K, N, batch, w, per_mode, reuse):
    """The decision for one contraction shape: (path name, {path: microseconds})
    or None."""
    us = (ctypes.c_float * len(PATHS))()
    p = lib().falcon_tune_lookup(device.encode(), rows, K, N, batch, w, per_mode, reuse, us)
    if p < 0:
        return None
    return PATHS[p], {PATHS[i]: float(us[i]) for i in range(len(PATHS)) if us[i] >= 0}


def device_tag():
    """Device key of the tuning cache for the current device."""
    return lib().falcon_device_tag().decode()


def set_step_graphs(enable):
    """Replay steady-state steps as CUDA graphs (default on); returns the previous setting."""
    return lib().falcon_set_step_graphs(1 if enable else 0)


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if a is not None else None


class Handle:
    """One instance through the single-run entry points a Fortran host binds
    (falcon_create, falcon_init_state, falcon_upload_factors, falcon_step,
    falcon_get_state, falcon_destroy)."""

    def __init__(self, params):
        self.params = params
        h = ctypes.c_void_p()
        check(lib().falcon_create(ctypes.byref(params), ctypes.byref(h)))
        self.h = h

    def init_noise(self, seed, amp=1e-3):
        check(lib().falcon_init_state(self.h, 1, amp, seed))

    def upload_factors(self, AT=None, ipiv_T=None, AF=None, ipiv_F=None, A_uphi=None, ipiv_uphi=None,
                       LAPpsi=None, ipiv_lap=None):
        """Factors (n, n, Nm+1) and 1-based pivots (n, Nm+1) in Fortran
        order, as numpy arrays indexed [i, j, m] and [i, m]."""
        f = [None if a is None else np.asfortranarray(a, np.float64) for a in (AT, AF, A_uphi, LAPpsi)]
        q = [None if a is None else np.asfortranarray(a, np.int32) for a in (ipiv_T, ipiv_F, ipiv_uphi, ipiv_lap)]
        check(lib().falcon_upload_factors(self.h, _dp(f[0]), _ip(q[0]), _dp(f[1]), _ip(q[1]), _dp(f[2]), _ip(q[2]),
                                          _dp(f[3]), _ip(q[3])))

    def step(self, n=1):
        check(lib().falcon_step(self.h, n))

    def get_state(self):
        shape = (self.params.nr_max, self.params.nm_max + 1)
        arrs = [_field(shape) for _ in range(5)]
        check(lib().falcon_get_state(self.h, *[_dp(a) for a in arrs]))
        return dict(zip(("T", "omg", "up", "ur", "psi"), arrs))

    def close(self):
        if self.h:
            lib().falcon_destroy(self.h)
            self.h = None
