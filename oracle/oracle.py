"""ctypes front-end of the CPU oracle (test infrastructure only).

Used by tests/, ``__graft_entry__.smoke()`` and the cpu_baseline leg of
``bench.py`` as the checker.  The product never imports this module.
Complex arrays are numpy complex128 in the reference's Fortran (M, R) layout,
i.e. numpy arrays of shape (R, M) in C order (mode fastest).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

TYPE = {"IMEX": 0, "IMEXRK": 1, "RK": 2}
IMP = {"CN": 0, "BDF2": 1, "BDF3": 2, "BDF4": 3, "ARS443": 10, "ARS343": 11,
       "BPR353": 12, "ARS222": 13, "ARS232": 14, "ARS233": 15, "NONE": 20}
EXP = {"AB2": 0, "AB3": 1, "AB4": 2, "expARS443": 10, "expARS343": 11,
       "expBPR353": 12, "expARS222": 13, "expARS232": 14, "expARS233": 15,
       "RK2": 20, "RK4": 21}
# Scheme shorthands used by the workload definitions.
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


class OrcParams(ctypes.Structure):
    _fields_ = [("nr_max", ctypes.c_int), ("nm_max", ctypes.c_int),
                ("eta", ctypes.c_double), ("ra", ctypes.c_double), ("pr", ctypes.c_double),
                ("mbc", ctypes.c_int), ("lagpts", ctypes.c_int), ("buo_imp", ctypes.c_int),
                ("dt", ctypes.c_double), ("scheme_type", ctypes.c_int),
                ("scheme_imp", ctypes.c_int), ("scheme_exp", ctypes.c_int),
                ("l_imexrk_started", ctypes.c_int), ("l_vartimestep", ctypes.c_int),
                ("l_optimizedt", ctypes.c_int), ("cfl", ctypes.c_double), ("dt_coef", ctypes.c_double),
                ("dt_max", ctypes.c_double)]


def build():
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_fft.argtypes = [ctypes.c_int, dp, dp, ctypes.c_int]
        for f in ("orc_forfft", "orc_invfft"):
            getattr(L, f).argtypes = [ctypes.c_int, ctypes.c_int, dp, dp]
        for f in ("orc_chebtransform", "orc_chebinvtran", "orc_chebinvtranD1", "orc_chebinvtranD2"):
            getattr(L, f).argtypes = [ctypes.c_int, dp, dp]
        L.orc_chebinvtranD1D2.argtypes = [ctypes.c_int, dp, dp, dp]
        L.orc_dcheb.argtypes = [ctypes.c_int, dp, dp, dp, dp]
        L.orc_dgetrf.argtypes = [ctypes.c_int, dp, ip]
        L.orc_dgetrf.restype = ctypes.c_int
        L.orc_dgetrs.argtypes = [ctypes.c_int, dp, ip, dp]
        L.orc_nonlin.argtypes = [ctypes.c_int, ctypes.c_int] + [dp] * 8
        L.orc_sim_create.argtypes = [ctypes.POINTER(OrcParams)]
        L.orc_sim_create.restype = ctypes.c_void_p
        L.orc_sim_destroy.argtypes = [ctypes.c_void_p]
        L.orc_sim_init.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_uint64]
        L.orc_sim_set_state.argtypes = [ctypes.c_void_p, dp, dp, dp, dp]
        L.orc_sim_get_state.argtypes = [ctypes.c_void_p, dp, dp, dp, dp, dp]
        L.orc_sim_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_sim_diagnostics.argtypes = [ctypes.c_void_p, dp]
        L.orc_sim_nstep.argtypes = [ctypes.c_void_p]
        L.orc_sim_dt.argtypes = [ctypes.c_void_p]
        L.orc_sim_store_checkpoint.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.orc_sim_store_snapshot.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.orc_sim_restart.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_double]
        L.orc_sim_dt.restype = ctypes.c_double
        L.orc_noise_pair.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, dp, dp]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_sim_spectra.argtypes = [ctypes.c_void_p, dp, dp]
        L.orc_sim_upbalance.argtypes = [ctypes.c_void_p, dp]
        L.orc_mat_assemble.argtypes = [ctypes.POINTER(OrcParams), ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_int, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _c(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def fft(x, sign):
    x = _c(x)
    out = np.empty_like(x)
    lib().orc_fft(x.size, _dp(x), _dp(out), sign)
    return out


def forfft(nm, np_, ff):
    ff = np.ascontiguousarray(ff, dtype=np.float64)
    out = np.empty(nm + 1, np.complex128)
    lib().orc_forfft(nm, np_, _dp(ff), _dp(out))
    return out


def invfft(nm, np_, f):
    f = _c(f)
    out = np.empty(np_, np.float64)
    lib().orc_invfft(nm, np_, _dp(f), _dp(out))
    return out


def _cheb1(name, f):
    f = _c(f)
    out = np.empty_like(f)
    getattr(lib(), name)(f.size, _dp(f), _dp(out))
    return out


def chebtransform(f):
    return _cheb1("orc_chebtransform", f)


def chebinvtran(f):
    return _cheb1("orc_chebinvtran", f)


def chebinvtranD1(f):
    return _cheb1("orc_chebinvtranD1", f)


def chebinvtranD2(f):
    return _cheb1("orc_chebinvtranD2", f)


def dcheb(nr):
    xp = np.empty(nr)
    t = np.empty((nr, nr), order="F")
    d = np.empty((nr, nr), order="F")
    d2 = np.empty((nr, nr), order="F")
    lib().orc_dcheb(nr, _dp(xp), _dp(t), _dp(d), _dp(d2))
    return xp, t, d, d2


def dgetrf(a):
    a = np.asfortranarray(a, dtype=np.float64).copy(order="F")
    piv = np.zeros(a.shape[0], np.int32)
    info = lib().orc_dgetrf(a.shape[0], _dp(a), piv.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return a, piv, info


def dgetrs(lu, piv, b):
    b = np.ascontiguousarray(b, dtype=np.float64).copy()
    lu = np.asfortranarray(lu)
    piv = np.ascontiguousarray(piv, dtype=np.int32)
    lib().orc_dgetrs(lu.shape[0], _dp(lu), piv.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(b))
    return b


def nonlin(nm, t, om, up, ur):
    """Nr_maxLOOP for one instance; fields are (R, M) complex (mode fastest)."""
    t, om, up, ur = (_c(a) for a in (t, om, up, ur))
    nr = t.shape[0]
    outs = [np.empty_like(t) for _ in range(4)]
    lib().orc_nonlin(nm, nr, _dp(t), _dp(om), _dp(up), _dp(ur), *[_dp(o) for o in outs])
    return outs


MAT_KINDS = {"AT": 0, "AF": 1, "A_uphi": 2, "LAPpsi": 3}


def mat_assemble(nr, kind, n, dt, wt, pr=1.0, mbc="NS", irk=False):
    """Operator matrix `kind` (AT, AF, A_uphi, LAPpsi) of mode n before its
    LU factorisation, as a numpy array indexed [i, j] (row, column)."""
    p = make_params(nr, 4, "CNAB2", pr=pr, dt=dt, mbc=mbc)
    size = 2 * nr if kind == "AF" else nr
    out = np.zeros(size * size)
    if lib().orc_mat_assemble(ctypes.byref(p), MAT_KINDS[kind], n, dt, wt, 1 if irk else 0, _dp(out)) != 0:
        raise RuntimeError("orc_mat_assemble failed")
    return out.reshape(size, size).T  # column-major -> [row, column]


def make_params(nr, nm, scheme="CNAB2", eta=0.35, ra=1e5, pr=1.0, dt=1e-5, mbc="NS",
                lagpts=16, buo="IMP", imexrk_started=False, vartimestep=False, optimizedt=False,
                cfl=0.9, dt_coef=2.0, dt_max=3e-5):
    typ, imp, exp = SCHEMES[scheme]
    return OrcParams(nr, nm, eta, ra, pr, 0 if mbc == "NS" else 1, lagpts,
                     1 if buo == "IMP" else 0, dt, TYPE[typ], IMP[imp], EXP[exp],
                     1 if imexrk_started else 0, 1 if vartimestep else 0, 1 if optimizedt else 0,
                     cfl, dt_coef, dt_max)


class Sim:
    """One annulus instance stepped by the oracle."""

    def __init__(self, params):
        self.p = params
        self.h = lib().orc_sim_create(ctypes.byref(params))
        if not self.h:
            raise ValueError("oracle: unsupported parameters")
        self.R = params.nr_max
        self.M = params.nm_max + 1

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_sim_destroy(self.h)
            self.h = None

    def init_noise(self, seed, amp=1e-3):
        lib().orc_sim_init(self.h, 1, 0, amp, seed)

    def init_reference(self, n_init=0, amp=1e-2):
        lib().orc_sim_init(self.h, 0, n_init, amp, 0)

    def set_state(self, t, om, up, ur):
        t, om, up, ur = (_c(a) for a in (t, om, up, ur))
        lib().orc_sim_set_state(self.h, _dp(t), _dp(om), _dp(up), _dp(ur))

    def get_state(self):
        arrs = [np.empty((self.R, self.M), np.complex128) for _ in range(5)]
        lib().orc_sim_get_state(self.h, *[_dp(a) for a in arrs])
        return dict(zip(("T", "omg", "up", "ur", "psi"), arrs))

    def store_checkpoint(self, path):
        if lib().orc_sim_store_checkpoint(self.h, os.fsencode(path)) != 0:
            raise RuntimeError("oracle: checkpoint write failed")

    def store_snapshot(self, path):
        if lib().orc_sim_store_snapshot(self.h, os.fsencode(path)) != 0:
            raise RuntimeError("oracle: snapshot write failed")

    def restart(self, directory, npoint, add_pert=False, ampT=0.0):
        """l_restart from "<directory>/checkpoint_%05d" files (see orc_sim_restart)."""
        rc = lib().orc_sim_restart(self.h, os.fsencode(str(directory)), npoint, 1 if add_pert else 0, ampT)
        if rc != 0:
            raise RuntimeError("oracle: restart failed (%d)" % rc)

    @property
    def dt(self):
        """Current time step (dt_new)."""
        return lib().orc_sim_dt(self.h)

    def step(self, n=1):
        rc = lib().orc_sim_step(self.h, n)
        if rc != 0:
            raise RuntimeError("oracle step failed")

    def spectra(self):
        """calculate_spectra: (KEspec, Temp_spec) of modes 0..Nm_max (x 4 pi)."""
        M = self.p.nm_max + 1
        ke = np.zeros(M)
        ts = np.zeros(M)
        lib().orc_sim_spectra(self.h, _dp(ke), _dp(ts))
        return ke, ts

    def upbalance(self):
        """The u_phi balance columns of upbalance_<tag>: (Nr, 4) = radius,
        d(up_0)/dt, advection, diffusion."""
        out = np.zeros((self.p.nr_max, 4))
        lib().orc_sim_upbalance(self.h, _dp(out))
        return out

    def diagnostics(self):
        out = np.empty(9)
        lib().orc_sim_diagnostics(self.h, _dp(out))
        keys = ("KE", "KE_r", "KE_phi", "KE_upbar", "Nu_top", "Nu_bot", "vis", "buo", "time")
        return dict(zip(keys, out))


def set_threads(n):
    lib().orc_set_threads(n)
