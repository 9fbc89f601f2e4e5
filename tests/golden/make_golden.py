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
mat_build, AT/AF blocks).  The operator matrices themselves (AT, AF in
both boundary-row orders, A_uphi and LAPpsi, no-slip and stress-free) are
written by an independent numpy restatement of src/mat_assembly.F90:68-462.
Grid changes at restart are pinned to the reference's own Python resampling
(cheblib.chebforward, padding and chebinverse, python/annulus/cheblib.py:
184-234), and the reference's error norm calc_rel_L2norm (:251-271) is
evaluated on seeded fields.  The reference's own namelist src/input.txt is
copied verbatim to tests/golden/input_reference.txt.
Output: tests/golden/golden.npz.
"""
import importlib.util
import os
import shutil

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


def cheb_grid_ops(nr, eta=0.35):
    """Gauss-Lobatto points, T_j(x_i) and its first two r-derivatives (d/dr =
    2 d/dx on the unit-width annulus), radius, 1/r and 1/r^2 (dcheb,
    src/chebyshev_fftw.F90:88-121, and init_grid, src/init.F90:128-131)."""
    xp = np.cos(np.pi * (nr - 1 - np.arange(nr)) / (nr - 1))
    t = np.zeros((nr, nr)); d = np.zeros((nr, nr)); d2 = np.zeros((nr, nr))
    for i in range(nr):
        T = [1.0, xp[i]]; dT = [0.0, 1.0]; d2T = [0.0, 0.0]
        for j in range(2, nr):
            T.append(2 * xp[i] * T[j - 1] - T[j - 2])
            dT.append(2 * T[j - 1] + 2 * xp[i] * dT[j - 1] - dT[j - 2])
            d2T.append(4 * dT[j - 1] + 2 * xp[i] * d2T[j - 1] - d2T[j - 2])
        t[i] = T; d[i] = 2 * np.array(dT); d2[i] = 4 * np.array(d2T)
    rmin = eta / (1 - eta)
    rad = rmin + 0.5 * (1 + xp)
    return t, d, d2, 1 / rad, 1 / rad ** 2


def operator_matrix(kind, nr, n, dt, wt, pr, mbc, irk):
    """AT, AF, A_uphi or LAPpsi of mode n before dgetrf, [row, column]:
    mat_build (src/mat_assembly.F90:242-359), mat_build_IRK (:68-187, psi
    boundary rows in the other order), mat_build_uphibar(_IRK) (:189-240,
    :361-413) and mat_build_rk (:415-462)."""
    t, d, d2, rr, rr2 = cheb_grid_ops(nr)
    C = np.sqrt(2.0 / (nr - 1))
    lap = rr[:, None] * d + d2 - n * n * rr2[:, None] * t
    if mbc == "NS":
        bc2 = (d[0], d[-1])
        bcu = (t[0], t[-1])
    else:
        bc2 = (d2[0] - rr[0] * d[0], d2[-1] - rr[-1] * d[-1])
        bcu = (d[0] - rr[0] * t[0], d[-1] - rr[-1] * t[-1])
    if kind == "AT":
        A = t - wt * dt * (1.0 / pr) * lap
        A[0], A[-1] = t[0], t[-1]
    elif kind == "A_uphi":
        A = t - wt * dt * (rr[:, None] * d + d2 - rr2[:, None] * t)
        A[0], A[-1] = bcu
    elif kind == "LAPpsi":
        A = lap.copy()
        A[0], A[-1] = t[0], t[-1]
    else:
        A = np.zeros((2 * nr, 2 * nr))
        A[:nr, :nr] = lap
        A[:nr, nr:] = t
        A[nr:, nr:] = t - wt * dt * lap
        first, second = (bc2, (t[0], t[-1])) if irk else (((t[0], t[-1])), bc2)
        A[0, :nr], A[nr - 1, :nr] = first
        A[nr, :nr], A[2 * nr - 1, :nr] = second
        A[0, nr:] = A[nr - 1, nr:] = A[nr, nr:] = A[2 * nr - 1, nr:] = 0.0
        for c in (0, nr - 1, nr, 2 * nr - 1):
            A[:, c] *= 0.5
        return C * A
    A[:, 0] *= 0.5
    A[:, -1] *= 0.5
    return C * A


MAT_CASES = [(nr, n, mbc, irk) for nr, n in ((9, 0), (9, 3), (9, 4), (33, 0), (33, 3), (33, 16), (65, 32))
             for mbc in ("NS", "SF") for irk in (0, 1)]
MAT_DT, MAT_WT, MAT_PR = 2e-5, 0.4358665215, 0.7
RESAMPLE_CASES = ((17, 8, 17, 12), (17, 8, 33, 8), (17, 8, 33, 12))
NORM_GRID = (33, 16)


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
    # operator matrices (independent restatement of src/mat_assembly.F90)
    for nr, n, mbc, irk in MAT_CASES:
        for kind in ("AT", "AF", "A_uphi", "LAPpsi"):
            if kind != "AF" and irk:
                continue  # the IRK forms differ from mat_build only in AF's rows
            out[f"mat_{kind}_{nr}_{n}_{mbc}_{irk}"] = operator_matrix(kind, nr, n, MAT_DT, MAT_WT, MAT_PR, mbc, irk)
    # grid change at restart through the reference's own resampling
    for nr0, nm0, nr1, nm1 in RESAMPLE_CASES:
        key = f"resample_{nr0}_{nm0}_{nr1}_{nm1}"
        fields = []
        for _ in range(4):
            f = (rng.standard_normal((nm0 + 1, nr0)) + 1j * rng.standard_normal((nm0 + 1, nr0)))
            fields.append(f * np.exp(-0.1 * np.arange(nm0 + 1))[:, None])
        for name, f in zip(("T", "omg", "ur", "up"), fields):
            fc = cl.chebforward(f, nm0, nr0)
            padded = cl.padding(fc, nm1, nr1, nm0, nr0)
            out[f"{key}_{name}_old"] = f.T.copy()  # stored (R, M): mode fastest, like the state arrays
            out[f"{key}_{name}_new"] = cl.chebinverse(padded, nm1, nr1, nr0).T.copy()
    # the reference's relative L2 error norm on seeded fields
    nr, nm = NORM_GRID
    eta = 0.35
    rmin, rmax = eta / (1 - eta), 1 / (1 - eta)
    for k in range(3):
        ref = (rng.standard_normal((nm + 1, nr)) + 1j * rng.standard_normal((nm + 1, nr)))
        comp = ref + (10.0 ** (-3 * k - 3)) * (rng.standard_normal((nm + 1, nr)) + 1j * rng.standard_normal((nm + 1, nr)))
        out[f"norm_{k}_ref"] = ref.T.copy()
        out[f"norm_{k}_comp"] = comp.T.copy()
        out[f"norm_{k}_rel_l2"] = np.array(cl.calc_rel_L2norm(comp, ref, nm, nr, rmin, rmax))
    shutil.copyfile(os.path.join(REF, "src", "input.txt"), os.path.join(HERE, "input_reference.txt"))
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
