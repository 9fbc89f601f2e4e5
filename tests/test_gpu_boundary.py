"""The remaining drop-in entry points of the C ABI:

- falcon_upload_factors: the implicit operators from the caller's own
  dgetrf factors (the output of mat_build* + factorize,
  src/mat_assembly.F90:68-462).  The matrices are assembled by the oracle,
  factorised by LAPACK (SciPy), uploaded through the single-run handle
  entry points a Fortran host binds, and the run must step to the same
  state as one whose factors the library builds itself (1e-12 after 20
  steps) and as the oracle (1e-10);
- falcon_cheb_d1d2_dev: chebinvtranD1D2 (src/chebyshev_fftw.F90:369-427)
  against the reference's own cheblib derivatives.
"""
import json
import os

import numpy as np
import pytest

from conftest import ROOT, rel

pytestmark = pytest.mark.gpu


def lapack_factors(orc, kind, R, M, dt, wt, pr, mbc, irk, first=0):
    from scipy.linalg import lapack
    n = 2 * R if kind == "AF" else R
    F = np.zeros((n, n, M), order="F")
    P = np.ones((n, M), np.int32, order="F")
    for m in range(first, M):
        A = orc.mat_assemble(R, kind, m, dt, wt, pr=pr, mbc=mbc, irk=irk)
        lu, piv, info = lapack.dgetrf(A)
        assert info == 0
        F[:, :, m] = lu
        P[:, m] = piv + 1
    return F, P


def run(fg, params, seed, nsteps, factors=None):
    h = fg.Handle(params)
    h.init_noise(seed)
    if factors is not None:
        h.upload_factors(**factors)
    h.step(nsteps)
    st = h.get_state()
    h.close()
    return st


@pytest.mark.parametrize("scheme,mbc", [("CNAB2", "NS"), ("SBDF3", "SF"), ("ARS343", "NS")])
def test_uploaded_lapack_factors_step_like_device_factors(fg, orc, scheme, mbc):
    R, Nm, dt, ra, pr = 17, 8, 1e-4, 1e4, 0.7
    M = Nm + 1
    if scheme == "CNAB2":
        wt, irk = 0.5, False                  # CN: wt_lhs = 1/2
    elif scheme == "SBDF3":
        wt, irk = 6.0 / 11.0, False           # BDF3 at constant dt
    else:
        tab = json.load(open(os.path.join(ROOT, "tests", "golden", "imexrk_tables.json")))["ARS343"]
        d = tab["diag_index"] - 1
        wt, irk = tab["aD"][d][d], True       # butcher_aD(diag_index, diag_index)
    AT, pT = lapack_factors(orc, "AT", R, M, dt, wt, pr, mbc, irk)
    AF, pF = lapack_factors(orc, "AF", R, M, dt, wt, pr, mbc, irk, first=1)
    Au, pu = lapack_factors(orc, "A_uphi", R, 1, dt, wt, pr, mbc, irk)
    f = dict(AT=AT, ipiv_T=pT, AF=AF, ipiv_F=pF, A_uphi=Au[:, :, 0], ipiv_uphi=pu[:, 0])
    if scheme == "ARS343":  # not stiffly accurate: the psi Poisson operator too
        f["LAPpsi"], f["ipiv_lap"] = lapack_factors(orc, "LAPpsi", R, M, dt, 0.0, pr, mbc, False, first=1)
    params = fg.make_params(R, Nm, scheme, ra=ra, dt=dt, pr=pr, mbc=mbc)
    got = run(fg, params, 5, 20, f)
    own = run(fg, params, 5, 20)
    for k in ("T", "omg", "up", "ur", "psi"):
        assert rel(got[k], own[k]) < 1e-12, k
    o = orc.Sim(orc.make_params(R, Nm, scheme, ra=ra, dt=dt, pr=pr, mbc=mbc))
    o.init_noise(5)
    o.step(20)
    os_ = o.get_state()
    for k in ("T", "omg", "up", "ur"):
        assert rel(got[k], os_[k]) < 1e-10, k


def test_upload_factors_refusals(fg, orc):
    R, Nm = 9, 4
    M = Nm + 1
    AT, pT = lapack_factors(orc, "AT", R, M, 1e-4, 0.5, 1.0, "NS", False)
    h = fg.Handle(fg.make_params(R, Nm, "CNAB2", dt=1e-4))
    bad = pT.copy()
    bad[2, 1] = R + 1
    with pytest.raises(fg.FalconError, match="pivot"):
        h.upload_factors(AT=AT, ipiv_T=bad)
    with pytest.raises(fg.FalconError, match="pivots"):
        h.upload_factors(AT=AT)
    h.upload_factors(AT=AT, ipiv_T=pT)   # AT alone: AF and A_uphi stay the library's own
    h.close()
    h = fg.Handle(fg.make_params(R, Nm, "SMR333", dt=1e-4))   # stage-dependent implicit diagonal
    with pytest.raises(fg.FalconError, match="stage"):
        h.upload_factors(AT=AT, ipiv_T=pT)
    h.close()


@pytest.mark.parametrize("nr", [9, 33, 97, 129])
def test_cheb_d1d2_entry_point_matches_reference_cheblib(fg, golden, nr):
    import torch
    c = golden[f"cheb_{nr}_c"]
    xin = torch.from_numpy(np.ascontiguousarray(c).view(np.float64)).cuda()
    d1 = torch.empty_like(xin)
    d2 = torch.empty_like(xin)
    fg.check(fg.lib().falcon_cheb_d1d2_dev(nr, 1, xin.data_ptr(), d1.data_ptr(), d2.data_ptr(), None))
    torch.cuda.synchronize()
    assert rel(d1.cpu().numpy().view(np.complex128), golden[f"cheb_{nr}_d1"]) < 1e-12
    assert rel(d2.cpu().numpy().view(np.complex128), golden[f"cheb_{nr}_d2"]) < 1e-12
    with pytest.raises(fg.FalconError):
        fg.check(fg.lib().falcon_cheb_d1d2_dev(nr, 1, xin.data_ptr(), d1.data_ptr(), d1.data_ptr(), None))
