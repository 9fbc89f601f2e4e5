"""Every built IMEXRK scheme (src/timeschemes.F90 tables) on the GPU against
the oracle: stiffly accurate ones through Assembly_stage_SA, the others
through Assembly_stage (psi Poisson solve, Johnston wall vorticity); the
7- and 8-stage KC774 / KC885; and the schemes whose implicit diagonal
varies by stage (diag_diff), which solve each such stage with operators of
its own weight (src/fourierloop_imexrk.F90:134-160)."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-10
SCHEMES = ["ARS443", "ARS343", "BPR353", "ARS222", "ARS232", "ARS233", "EUL111", "MARS343", "IJ3", "PC2",
           "SSP332", "SSP543", "PR433", "DBM453", "KC343", "KC564", "FW53", "CK222", "BPR442", "CFN343",
           "BHR553", "CFN564", "KC774", "KC885", "SMR333", "CB3e", "CB3f", "CB4", "LZ3L1", "LZ4A1"]
DIAG_DIFF = ["SMR333", "CB3e", "CB3f", "CB4", "LZ3L1", "LZ4A1"]
FIELDS = ("T", "omg", "up", "ur", "psi")


def run(orc, fg, scheme, R, Nm, ra, dt, nsteps, mbc="NS"):
    g = fg.Instance(fg.make_params(R, Nm, scheme, ra=ra, dt=dt, mbc=mbc))
    o = orc.Sim(orc.make_params(R, Nm, scheme, ra=ra, dt=dt, mbc=mbc))
    g.init_noise(3)
    o.init_noise(3)
    g.step(nsteps)
    o.step(nsteps)
    gs, os_ = g.get_state(), o.get_state()
    return {k: rel(gs[k], os_[k]) for k in ("T", "omg", "up", "ur", "psi")}


@pytest.mark.parametrize("scheme", SCHEMES)
def test_imexrk_scheme_parity(orc, fg, scheme):
    errs = run(orc, fg, scheme, 17, 8, 1e4, 1e-5, 30)
    assert max(errs.values()) < STEP_TOL, errs


def test_bhr553_reference_input_scheme_100_steps(orc, fg):
    # the scheme of the reference's own input.txt, at the plain run's grid
    errs = run(orc, fg, "BHR553", 33, 42, 1e5, 1e-5, 100)
    assert max(errs.values()) < STEP_TOL, errs


def test_kc564_stress_free(orc, fg):
    errs = run(orc, fg, "KC564", 17, 8, 1e4, 1e-5, 30, mbc="SF")
    assert max(errs.values()) < STEP_TOL, errs


@pytest.mark.parametrize("scheme", ["CB4", "KC885", "LZ4A1"])
def test_many_stage_schemes_100_steps(orc, fg, scheme):
    errs = run(orc, fg, scheme, 33, 42, 1e5, 1e-5, 100)
    assert max(errs.values()) < STEP_TOL, errs


@pytest.mark.parametrize("scheme", ["SMR333", "CB3f"])
def test_diag_diff_stress_free(orc, fg, scheme):
    errs = run(orc, fg, scheme, 17, 8, 1e4, 1e-5, 30, mbc="SF")
    assert max(errs.values()) < STEP_TOL, errs


def test_diag_diff_group_shares_stage_operators_bitwise(fg, fixed_paths):
    # two SMR333 instances (different Ra) form one group with one set of
    # stage operators; each equals its own run alone
    ps = [fg.make_params(17, 10, "SMR333", ra=1e4, dt=1e-5), fg.make_params(17, 10, "SMR333", ra=3e4, dt=1e-5),
          fg.make_params(17, 10, "CB4", ra=1e4, dt=1e-5)]
    b = fg.Batch(ps)
    assert b.ngroups == 2
    b.init_noise([4, 5, 6])
    b.step(12)
    for i in range(3):
        alone = fg.Instance(ps[i])
        alone.init_noise(4 + i)
        alone.step(12)
        sb, sa = b.get_state(i), alone.get_state()
        for f in FIELDS:
            assert np.array_equal(sb[f], sa[f]), (i, f)


def test_lz3a4a_is_refused(fg):
    import ctypes
    p = fg.make_params(17, 8, "LZ3A4a")
    h = ctypes.c_void_p()
    assert fg.lib().falcon_create(ctypes.byref(p), ctypes.byref(h)) == -1
    assert b"singular" in fg.lib().falcon_last_error()
