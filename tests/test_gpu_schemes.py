"""Every built IMEXRK scheme (src/timeschemes.F90 tables) on the GPU against
the oracle: stiffly accurate ones through Assembly_stage_SA, the others
through Assembly_stage (psi Poisson solve, Johnston wall vorticity)."""
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-10
SCHEMES = ["ARS443", "ARS343", "BPR353", "ARS222", "ARS232", "ARS233", "EUL111", "MARS343", "IJ3", "PC2",
           "SSP332", "SSP543", "PR433", "DBM453", "KC343", "KC564", "FW53", "CK222", "BPR442", "CFN343",
           "BHR553", "CFN564"]


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
