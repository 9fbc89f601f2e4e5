"""The CPU oracle pinned against the reference: golden vectors produced by the
reference's own Python transforms (python/annulus/cheblib.py), the explicit
DFT sums of src/fourier_GG.F90, and LAPACK dgetrf/dgetrs on the reference's
operator matrices (tests/golden/make_golden.py), plus analytic known answers.
"""
import numpy as np
import pytest

from conftest import rel

NRS = (9, 17, 33, 65, 97, 129)
NMS = (4, 42, 85, 170, 341, 512)


@pytest.mark.parametrize("nr", NRS)
def test_chebyshev_transforms_match_reference_cheblib(orc, golden, nr):
    f = golden[f"cheb_{nr}_f"]
    c = golden[f"cheb_{nr}_c"]
    assert rel(orc.chebtransform(f), golden[f"cheb_{nr}_fwd"]) < 1e-14
    assert rel(orc.chebinvtran(c), golden[f"cheb_{nr}_inv"]) < 1e-14
    assert rel(orc.chebinvtranD1(c), golden[f"cheb_{nr}_d1"]) < 1e-14
    assert rel(orc.chebinvtranD2(c), golden[f"cheb_{nr}_d2"]) < 1e-14


@pytest.mark.parametrize("nm", NMS)
def test_azimuthal_transforms_match_direct_sums(orc, golden, nm):
    np_ = 3 * nm
    assert rel(orc.forfft(nm, np_, golden[f"four_{nm}_ff"]), golden[f"four_{nm}_fwd"]) < 1e-13
    assert rel(orc.invfft(nm, np_, golden[f"four_{nm}_f"]), golden[f"four_{nm}_inv"]) < 1e-13


@pytest.mark.parametrize("case", ["AT_9_3", "AF_9_3", "AT_33_7", "AF_33_7", "AT_65_40", "AF_65_40"])
def test_lu_matches_lapack(orc, golden, case):
    k = "lu_" + case
    lu, piv, info = orc.dgetrf(golden[k + "_A"])
    assert info == 0
    assert np.array_equal(piv, golden[k + "_piv"])
    assert rel(lu, golden[k + "_lu"]) < 1e-13
    x = orc.dgetrs(lu, piv, golden[k + "_b"])
    assert rel(x, golden[k + "_x"]) < 1e-11


def test_chebyshev_round_trip_and_polynomial_derivative(orc):
    nr = 33
    xp, t, d, d2 = orc.dcheb(nr)
    # r = rmin + (1 + x)/2 so d/dr = 2 d/dx; f(x) = x^3 -> df/dr = 6 x^2, d2f/dr2 = 24 x
    f = xp ** 3 + 0j
    c = orc.chebtransform(f)
    assert rel(orc.chebinvtran(c), f) < 1e-14
    assert np.abs(orc.chebinvtranD1(c) - 6 * xp ** 2).max() < 1e-11
    assert np.abs(orc.chebinvtranD2(c) - 24 * xp).max() < 1e-9


def test_conductive_state_is_stationary(orc):
    p = orc.make_params(33, 42, "CNAB2", ra=1e5, dt=1e-4)
    s = orc.Sim(p)
    s.init_noise(1, 0.0)
    t0 = s.get_state()["T"]
    s.step(20)
    st = s.get_state()
    assert np.abs(st["T"] - t0).max() < 1e-13
    assert np.abs(st["omg"]).max() == 0.0
    d = s.diagnostics()
    assert abs(d["Nu_top"] - 1.0) < 1e-12 and abs(d["Nu_bot"] - 1.0) < 1e-12
    assert d["KE"] == 0.0


def test_pure_diffusion_is_linear_and_decaying(orc):
    # Ra = 0 and u = 0: the step is the linear diffusion operator on each
    # temperature mode, so doubling the perturbation doubles the result and
    # every mode decays monotonically.
    def run(amp, n):
        s = orc.Sim(orc.make_params(17, 4, "CNAB2", ra=0.0, dt=1e-3))
        s.init_noise(7, amp)
        out = []
        for _ in range(n):
            s.step(1)
            out.append(s.get_state()["T"][:, 1:].copy())
        return out
    a = run(1e-3, 4)
    b = run(2e-3, 4)
    for x, y in zip(a, b):
        assert rel(y, 2.0 * x) < 1e-13
    norms = [np.linalg.norm(x) for x in a]
    assert all(n2 < n1 for n1, n2 in zip(norms, norms[1:]))


@pytest.mark.parametrize("scheme", ["CNAB2", "ARS343", "BPR353"])
def test_schemes_agree_at_small_dt(orc, scheme):
    # Consistent schemes converge to the same solution; CNAB2 is the baseline.
    ref = orc.Sim(orc.make_params(17, 8, "CNAB2", ra=1e4, dt=1e-6))
    ref.init_noise(3)
    ref.step(20)
    s = orc.Sim(orc.make_params(17, 8, scheme, ra=1e4, dt=1e-6))
    s.init_noise(3)
    s.step(20)
    assert rel(s.get_state()["T"], ref.get_state()["T"]) < 1e-6
