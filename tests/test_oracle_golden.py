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


MAT_CASES = [(nr, n) for nr, n in ((9, 0), (9, 3), (9, 4), (33, 0), (33, 3), (33, 16), (65, 32))]
MAT_DT, MAT_WT, MAT_PR = 2e-5, 0.4358665215, 0.7


@pytest.mark.parametrize("nr,n", MAT_CASES)
@pytest.mark.parametrize("mbc", ["NS", "SF"])
def test_operator_matrices_match_independent_restatement(orc, golden, nr, n, mbc):
    # AT, A_uphi, LAPpsi and AF in both boundary-row orders (mat_build and
    # mat_build_IRK, src/mat_assembly.F90:143-150 vs :316-323) against the
    # numpy restatement of tests/golden/make_golden.py
    for kind, irk in (("AT", 0), ("A_uphi", 0), ("LAPpsi", 0), ("AF", 0), ("AF", 1)):
        want = golden[f"mat_{kind}_{nr}_{n}_{mbc}_{irk}"]
        got = orc.mat_assemble(nr, kind, n, MAT_DT, MAT_WT, pr=MAT_PR, mbc=mbc, irk=bool(irk))
        assert got.shape == want.shape
        assert rel(got, want) < 1e-13, (kind, irk)
    # the two AF orders are different matrices with the same rows
    a0 = orc.mat_assemble(nr, "AF", n, MAT_DT, MAT_WT, pr=MAT_PR, mbc=mbc, irk=False)
    a1 = orc.mat_assemble(nr, "AF", n, MAT_DT, MAT_WT, pr=MAT_PR, mbc=mbc, irk=True)
    assert not np.array_equal(a0, a1)
    assert np.array_equal(np.sort(a0, axis=0), np.sort(a1, axis=0))


@pytest.mark.parametrize("case", [(17, 8, 17, 12), (17, 8, 33, 8), (17, 8, 33, 12)])
def test_restart_resampling_matches_reference_padding(orc, golden, tmp_path, case):
    # get_checkpoint_data's grid change (src/init.F90:726-861) against the
    # reference's Python resampling: chebforward, padding, chebinverse
    nr0, nm0, nr1, nm1 = case
    key = "resample_%d_%d_%d_%d" % case
    old = {f: golden[f"{key}_{f}_old"] for f in ("T", "omg", "ur", "up")}
    o = orc.Sim(orc.make_params(nr0, nm0, "ARS443"))
    o.set_state(old["T"], old["omg"], old["up"], old["ur"])
    o.store_checkpoint(str(tmp_path / "checkpoint_00003"))
    n = orc.Sim(orc.make_params(nr1, nm1, "ARS443"))
    n.restart(tmp_path, 3)
    st = n.get_state()
    for f in ("T", "omg", "ur", "up"):
        assert rel(st[f], golden[f"{key}_{f}_new"]) < 1e-13, f


@pytest.mark.parametrize("k", [0, 1, 2])
def test_error_norm_restatement_matches_reference(golden, k):
    from conftest import rel_l2_reference
    got = rel_l2_reference(golden[f"norm_{k}_comp"], golden[f"norm_{k}_ref"])
    want = float(golden[f"norm_{k}_rel_l2"])
    assert abs(got - want) <= 1e-12 * want
