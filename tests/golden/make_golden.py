"""Generate the golden vectors that pin the CPU oracle to the reference.

Run where the FAlCon-DNS reference tree is available, with the environment
variable FALCON_REFERENCE naming its root (the directory holding src/ and
python/).  It imports the
reference's own Python restatement of the Chebyshev transforms
(python/annulus/cheblib.py: chebtransform, chebinvtran, chebinvtranD1,
chebinvtranD2, lines 467-585) and evaluates them on seeded inputs.  The
azimuthal transforms are pinned to the explicit sums of
src/fourier_GG.F90:14-71 (the reference's FFT-free build of forfft/invfft),
evaluated here in numpy.  Dense LU is pinned to LAPACK dgetrf/dgetrs through
SciPy on the reference's own operator matrices (src/mat_assembly.F90
mat_build, AT/AF blocks).  Output: tests/golden/golden.npz.
"""
import importlib.util
import os

import numpy as np
import scipy.linalg.lapack as lapack

REF = os.environ.get("FALCON_REFERENCE")
if not REF or not os.path.isdir(os.path.join(REF, "src")):
    raise SystemExit("set FALCON_REFERENCE to the root of the FAlCon-DNS source tree")
HERE = os.path.dirname(os.path.abspath(__file__))


def load_cheblib():
    path = os.path.join(REF, "python", "annulus", "cheblib.py")
    spec = importlib.util.spec_from_file_location("ref_cheblib", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def fourier_gg_forfft(nm, np_, ff):
    # src/fourier_GG.F90:14-38: f(m) = (1/Np) sum_j ff(j) exp(-2 pi i m (j-1)/Np)
    # the phase index m*(j-1) is reduced modulo Np exactly before the angle is
    # formed, so the sums carry no argument-rounding error
    j = np.arange(np_)
    m = np.arange(nm + 1)[:, None]
    k = (m * j[None, :]) % np_
    return (ff[None, :] * np.exp(-2j * np.pi * k / np_)).sum(axis=1) / np_


def fourier_gg_invfft(nm, np_, f):
    # src/fourier_GG.F90:40-71: ff(j) = 2*sum_m c_m Re(f(m) exp(2 pi i m (j-1)/Np)), c_0 = 1/2
    j = np.arange(np_)
    out = np.zeros(np_)
    for m in range(nm + 1):
        c = 0.5 if m == 0 else 1.0
        out += c * np.real(f[m] * np.exp(2j * np.pi * ((m * j) % np_) / np_))
    return 2.0 * out


def mat_build_blocks(nr, n, dt, wt, pr):
    """AT and AF of src/mat_assembly.F90:242-359 (mat_build, no-slip), numpy restatement."""
    xp = np.cos(np.pi * (nr - 1 - np.arange(nr)) / (nr - 1))
    t = np.zeros((nr, nr)); d = np.zeros((nr, nr)); d2 = np.zeros((nr, nr))
    for i in range(nr):
        T = [1.0, xp[i]]; dT = [0.0, 1.0]; d2T = [0.0, 0.0]
        for j in range(2, nr):
            T.append(2 * xp[i] * T[j - 1] - T[j - 2])
            dT.append(2 * T[j - 1] + 2 * xp[i] * dT[j - 1] - dT[j - 2])
            d2T.append(4 * dT[j - 1] + 2 * xp[i] * d2T[j - 1] - d2T[j - 2])
        t[i] = T; d[i] = 2 * np.array(dT); d2[i] = 4 * np.array(d2T)
    eta = 0.35
    rmin = eta / (1 - eta)
    rad = rmin + 0.5 * (1 + np.cos((nr - 1 - np.arange(nr)) * np.pi / (nr - 1)))
    rr = 1 / rad
    rr2 = rr * rr
    L = rr[:, None] * d + d2 - n * n * rr2[:, None] * t
    C = np.sqrt(2.0 / (nr - 1))
    AT = t - wt * dt / pr * L
    AT[0] = t[0]; AT[-1] = t[-1]
    AT[:, 0] *= 0.5; AT[:, -1] *= 0.5
    AT *= C
    AF = np.zeros((2 * nr, 2 * nr))
    AF[:nr, :nr] = L; AF[:nr, nr:] = t; AF[nr:, nr:] = t - wt * dt * L
    AF[0, :nr] = t[0]; AF[nr - 1, :nr] = t[-1]; AF[0, nr:] = 0; AF[nr - 1, nr:] = 0
    AF[nr, :nr] = d[0]; AF[2 * nr - 1, :nr] = d[-1]; AF[nr, nr:] = 0; AF[2 * nr - 1, nr:] = 0
    for c in (0, nr - 1, nr, 2 * nr - 1):
        AF[:, c] *= 0.5
    AF *= C
    return AT, AF


def main():
    cl = load_cheblib()
    rng = np.random.default_rng(20240607)
    out = {}
    for nr in (9, 17, 33, 65, 97, 129):
        f = rng.standard_normal(nr) + 1j * rng.standard_normal(nr)
        c = rng.standard_normal(nr) + 1j * rng.standard_normal(nr)
        c *= np.exp(-0.15 * np.arange(nr))  # decaying spectrum, like a smooth field
        out[f"cheb_{nr}_f"] = f
        out[f"cheb_{nr}_c"] = c
        out[f"cheb_{nr}_fwd"] = cl.chebtransform(nr, f.copy())
        out[f"cheb_{nr}_inv"] = cl.chebinvtran(nr, c.copy())
        out[f"cheb_{nr}_d1"] = cl.chebinvtranD1(nr, c.copy())
        out[f"cheb_{nr}_d2"] = cl.chebinvtranD2(nr, c.copy())
    for nm in (4, 42, 85, 170, 341, 512):
        np_ = 3 * nm
        ff = rng.standard_normal(np_)
        f = (rng.standard_normal(nm + 1) + 1j * rng.standard_normal(nm + 1)) * np.exp(-0.02 * np.arange(nm + 1))
        out[f"four_{nm}_ff"] = ff
        out[f"four_{nm}_f"] = f
        out[f"four_{nm}_fwd"] = fourier_gg_forfft(nm, np_, ff)
        out[f"four_{nm}_inv"] = fourier_gg_invfft(nm, np_, f)
    for nr, n in ((9, 3), (33, 7), (65, 40)):
        AT, AF = mat_build_blocks(nr, n, 1e-5, 0.5, 1.0)
        for name, A in (("AT", AT), ("AF", AF)):
            lu, piv, info = lapack.dgetrf(A)
            b = rng.standard_normal(A.shape[0])
            x, info2 = lapack.dgetrs(lu, piv, b)
            out[f"lu_{name}_{nr}_{n}_A"] = A
            out[f"lu_{name}_{nr}_{n}_lu"] = lu
            out[f"lu_{name}_{nr}_{n}_piv"] = piv + 1  # 1-based like Fortran
            out[f"lu_{name}_{nr}_{n}_b"] = b
            out[f"lu_{name}_{nr}_{n}_x"] = x
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
