"""The oracle's restart (l_restart): get_checkpoint_data and the multistep
bootstrap of timeloop_imex (src/init.F90:447-935, src/steptime.F90:87-193).

A multistep run restarted from its own checkpoints, with or without
l_imexrk_started, continues the uninterrupted run: the bootstrap rebuilds
from the stored states the same histories the run held.  The reference's
first step after a restart takes the Chebyshev coefficients afresh from the
values (src/fourierloop.F90:78-84), so the agreement is to rounding, not bit
for bit.  A restart on a larger grid reproduces a polynomial state exactly
at the new points."""
import numpy as np
import pytest

FIELDS = ("T", "omg", "up", "ur")


def run_with_checkpoints(orc, d, scheme, steps, store, R=17, Nm=8, **kw):
    o = orc.Sim(orc.make_params(R, Nm, scheme, ra=1e5, dt=1e-5, **kw))
    o.init_noise(3)
    for k in range(1, steps + 1):
        o.step(1)
        if k in store:
            o.store_checkpoint(str(d / ("checkpoint_%05d" % store[k])))
    return o


def relerr(a, b):
    return max(np.abs(a[f] - b[f]).max() / max(np.abs(a[f]).max(), 1e-300) for f in FIELDS)


@pytest.mark.parametrize("scheme", ["SBDF2", "SBDF3", "SBDF4", "CNAB2"])
@pytest.mark.parametrize("started", [True, False])
def test_multistep_restart_continues_the_run(orc, tmp_path, scheme, started):
    a = run_with_checkpoints(orc, tmp_path, scheme, 10, {7: 1, 8: 2, 9: 3, 10: 4})
    a.step(6)
    b = orc.Sim(orc.make_params(17, 8, scheme, ra=1e5, dt=1e-5, imexrk_started=started))
    b.init_noise(99)
    b.restart(tmp_path, 4)
    b.step(6)
    assert relerr(a.get_state(), b.get_state()) < 1e-11
    assert abs(a.diagnostics()["time"] - b.diagnostics()["time"]) < 1e-15


def test_restart_on_a_larger_grid_keeps_a_polynomial(orc, tmp_path):
    R0, N0, R1, N1 = 13, 6, 21, 9
    o = orc.Sim(orc.make_params(R0, N0, "ARS443"))
    x0 = -np.cos(np.pi * np.arange(R0) / (R0 - 1))    # stored order, rmin to rmax

    def field(x, M, seed):
        rng = np.random.default_rng(seed)
        c = rng.standard_normal((M, 6)) + 1j * rng.standard_normal((M, 6))
        return np.array([[np.polyval(c[m], xi) for m in range(M)] for xi in x])   # (R, M)
    fs = [field(x0, N0 + 1, s) for s in range(4)]
    o.set_state(fs[0], fs[1], fs[2], fs[3])
    o.store_checkpoint(str(tmp_path / "checkpoint_00007"))
    n = orc.Sim(orc.make_params(R1, N1, "ARS443"))
    n.restart(tmp_path, 7)
    st = n.get_state()
    x1 = -np.cos(np.pi * np.arange(R1) / (R1 - 1))
    for f, k in zip(("T", "omg", "up", "ur"), range(4)):
        want = np.zeros((R1, N1 + 1), complex)
        want[:, :N0 + 1] = field(x1, N0 + 1, k)
        assert np.abs(st[f] - want).max() < 1e-12 * np.abs(want).max(), f


def test_add_pert_and_refusals(orc, tmp_path):
    o = orc.Sim(orc.make_params(17, 8, "SBDF3"))
    o.init_noise(4)
    o.step(3)
    o.store_checkpoint(str(tmp_path / "checkpoint_00002"))
    b = orc.Sim(orc.make_params(17, 8, "SBDF3"))
    b.restart(tmp_path, 2, add_pert=True, ampT=0.25)
    assert np.allclose(b.get_state()["T"] - o.get_state()["T"], 0.25, atol=1e-15, rtol=0)
    with pytest.raises(RuntimeError):   # multistep histories do not change grid
        orc.Sim(orc.make_params(21, 8, "SBDF3")).restart(tmp_path, 2)
    with pytest.raises(RuntimeError):   # a smaller grid is not restored
        orc.Sim(orc.make_params(13, 8, "ARS443")).restart(tmp_path, 2)
    with pytest.raises(RuntimeError):   # l_imexrk_started with BDF3 needs checkpoints 0..2
        orc.Sim(orc.make_params(17, 8, "SBDF3", imexrk_started=True)).restart(tmp_path, 2)
