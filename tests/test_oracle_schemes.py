"""The oracle's IMEXRK schemes with a stage-dependent implicit diagonal
(diag_diff, src/fourierloop_imexrk.F90:134-160) and with 7-8 stages: the
solution converges in time at the order of the scheme's tables, which fails
if a stage solves with the operators of another stage's weight.  LZ3A4a's
zero-weight stages make the reference's coupled omega-psi operator singular:
the reference algorithm diverges in its first steps, and the library refuses
the scheme."""
import ctypes

import numpy as np
import pytest


def run(orc, name, dt, n):
    o = orc.Sim(orc.make_params(17, 8, name, ra=1e4, dt=dt))
    o.init_noise(2)
    o.step(n)
    return o.get_state()


@pytest.mark.parametrize("name,order", [("SMR333", 2), ("CB3f", 3), ("CB4", 4), ("LZ3L1", 3), ("KC774", 4),
                                        ("KC885", 5)])
def test_temporal_convergence_order(orc, name, order):
    T = 4e-3
    s = [run(orc, name, T / n, n) for n in (20, 40, 80)]
    d = [max(np.abs(s[k + 1][f] - s[k][f]).max() for f in ("T", "omg")) for k in range(2)]
    observed = np.log2(d[0] / d[1])
    assert observed > order - 0.35, (name, d, observed)


def test_lz3a4a_reference_algorithm_diverges_and_library_refuses(orc, fg):
    o = orc.Sim(orc.make_params(17, 8, "LZ3A4a", ra=1e4, dt=1e-5))
    o.init_noise(1)
    o.step(2)
    om = o.get_state()["omg"]
    assert not np.all(np.isfinite(om)) or np.abs(om).max() > 1e30
    p = fg.make_params(17, 8, "LZ3A4a")
    h = ctypes.c_void_p()
    assert fg.lib().falcon_create(ctypes.byref(p), ctypes.byref(h)) == -1
    assert b"singular" in fg.lib().falcon_last_error()
