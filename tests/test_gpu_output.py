"""The reference's remaining output diagnostics on the device against the
oracle: calculate_spectra (src/output.F90:327-355, the KEspec_<tag> and
Temp_spec_<tag> columns) and the u_phi force balance of writeKE_spectral
(src/output.F90:145-228, upbalance_<tag>), for an IMEX, an IMEXRK and an
RK run and for an instance inside a batch.  The balance's time derivative
uses upFR_prev, which the IMEX loop renews after each nonlinear pass and
the IMEXRK / RK loops keep from the start of the run."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def compare(g, o, label):
    kg, tg = g
    ko, to = o
    assert rel(kg, ko) < 1e-9, (label, "KEspec")
    assert rel(tg, to) < 1e-9, (label, "Temp_spec")


def compare_balance(ug, uo, label):
    assert np.array_equal(ug[:, 0], uo[:, 0]) or rel(ug[:, 0], uo[:, 0]) < 1e-15
    for c in (1, 2, 3):
        scale = max(np.abs(uo[:, c]).max(), 1e-300)
        assert np.abs(ug[:, c] - uo[:, c]).max() <= 1e-8 * scale, (label, c)


@pytest.mark.parametrize("scheme,dt", [("CNAB2", 1e-4), ("ARS443", 1e-5), ("RK4", 1e-6)])
def test_spectra_and_upbalance_match_oracle(fg, orc, scheme, dt):
    R, Nm, steps = 17, 8, 20
    g = fg.Instance(fg.make_params(R, Nm, scheme, ra=1e5, dt=dt))
    g.init_noise(4)
    o = orc.Sim(orc.make_params(R, Nm, scheme, ra=1e5, dt=dt))
    o.init_noise(4)
    for k in (1, steps - 1):
        g.step(k)
        o.step(k)
        compare(g.spectra(), o.spectra(), scheme)
        compare_balance(g.upbalance(), o.upbalance(), scheme)
    g.close()


def test_instance_inside_a_batch(fg, orc):
    ps = [fg.make_params(17, 8, "SBDF3", ra=ra, dt=1e-4) for ra in (1e4, 3e4, 1e5)]
    b = fg.Batch(ps)
    b.init_noise([7, 8, 9])
    b.step(15)
    o = orc.Sim(orc.make_params(17, 8, "SBDF3", ra=3e4, dt=1e-4))
    o.init_noise(8)
    o.step(15)
    compare(b.spectra(1), o.spectra(), "batch")
    compare_balance(b.upbalance(1), o.upbalance(), "batch")
    b.close()
