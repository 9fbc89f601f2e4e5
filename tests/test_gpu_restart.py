"""Restart (l_restart) on the GPU against the oracle, both reading the same
checkpoint files (written by the oracle): the multistep bootstrap from an
IMEXRK run's checkpoints (l_imexrk_started, src/steptime.F90:87-193), a
multistep restart from its own histories (with a change of order), IMEXRK
and RK restarts on a larger grid (src/init.F90:726-861), the restart rules
of the variable time step, and batches.  Tolerance: 1e-10 relative."""
import ctypes

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

TOL = 1e-10
FIELDS = ("T", "omg", "up", "ur", "psi")


def write_checkpoints(orc, d, scheme, steps, store, R=17, Nm=8, ra=1e5, dt=1e-5, **kw):
    o = orc.Sim(orc.make_params(R, Nm, scheme, ra=ra, dt=dt, **kw))
    o.init_noise(5, 1e-2)
    for k in range(1, steps + 1):
        o.step(1)
        if k in store:
            o.store_checkpoint(str(d / ("checkpoint_%05d" % store[k])))
    return o


def pair(orc, fg, d, scheme, point, nsteps, R=17, Nm=8, ra=1e5, dt=1e-5, started=False, add_pert=False,
         ampT=0.0, **kw):
    g = fg.Instance(fg.make_params(R, Nm, scheme, ra=ra, dt=dt, imexrk_started=started, restart=True,
                                   restart_point=point, add_pert=add_pert, ampT=ampT, **kw))
    o = orc.Sim(orc.make_params(R, Nm, scheme, ra=ra, dt=dt, imexrk_started=started, **kw))
    g.restart(str(d))
    o.restart(d, point, add_pert=add_pert, ampT=ampT)
    dts = []
    for _ in range(nsteps):
        g.step(1)
        o.step(1)
        dts.append((g.diagnostics()["dt"], o.dt))
    gs, os_ = g.get_state(), o.get_state()
    errs = {f: rel(gs[f], os_[f]) for f in FIELDS}
    return errs, dts, g, o


@pytest.mark.parametrize("scheme", ["SBDF2", "SBDF3", "SBDF4", "CNAB2", "CNAB3"])
def test_bootstrap_from_imexrk_checkpoints(orc, fg, tmp_path, scheme):
    write_checkpoints(orc, tmp_path, "ARS443", 20, {17: 1, 18: 2, 19: 3, 20: 4})
    errs, _, g, o = pair(orc, fg, tmp_path, scheme, 4, 30, started=True)
    assert max(errs.values()) < TOL, errs
    assert abs(g.diagnostics()["time"] - o.diagnostics()["time"]) <= 1e-14


@pytest.mark.parametrize("written,scheme", [("SBDF3", "SBDF3"), ("CNAB2", "SBDF3"), ("SBDF4", "CNAB2")])
def test_multistep_restart_from_file_histories(orc, fg, tmp_path, written, scheme):
    write_checkpoints(orc, tmp_path, written, 12, {12: 2})
    errs, _, _, _ = pair(orc, fg, tmp_path, scheme, 2, 30, add_pert=True, ampT=1e-3)
    assert max(errs.values()) < TOL, errs


@pytest.mark.parametrize("scheme,dt", [("ARS443", 1e-5), ("CB4", 1e-5), ("RK4", 1e-6)])
def test_restart_on_a_larger_grid(orc, fg, tmp_path, scheme, dt):
    write_checkpoints(orc, tmp_path, scheme, 10, {10: 3}, dt=dt)
    errs, _, _, _ = pair(orc, fg, tmp_path, scheme, 3, 20, R=25, Nm=11, dt=dt)
    assert max(errs.values()) < TOL, errs


@pytest.mark.parametrize("scheme,started,optimize", [("SBDF3", False, False), ("SBDF3", True, True),
                                                     ("ARS443", False, False), ("KC564", False, True),
                                                     ("RK4", False, False)])
def test_variable_dt_restart(orc, fg, tmp_path, scheme, started, optimize):
    kw = dict(ra=1e6, vartimestep=True, optimizedt=optimize, cfl=0.05, dt_coef=1.5, dt_max=1e-4)
    dt = 1e-6 if scheme == "RK4" else 1e-5
    write_checkpoints(orc, tmp_path, "ARS443" if started else scheme, 14, {12: 1, 13: 2, 14: 3}, dt=dt, **kw)
    errs, dts, _, _ = pair(orc, fg, tmp_path, scheme, 3, 20, dt=dt, started=started, **kw)
    for k, (a, b) in enumerate(dts):
        assert abs(a - b) <= 1e-12 * b, (k, a, b)
    assert max(errs.values()) < TOL, errs


def test_batch_restart_from_two_directories(orc, fg, tmp_path, fixed_paths):
    d1, d2 = tmp_path / "a", tmp_path / "b"
    d1.mkdir()
    d2.mkdir()
    write_checkpoints(orc, d1, "SBDF3", 9, {9: 5}, ra=1e5)
    write_checkpoints(orc, d2, "SBDF3", 9, {9: 5}, ra=1e5)   # same run time
    ps = [fg.make_params(17, 8, "SBDF3", ra=1e5, restart=True, restart_point=5),
          fg.make_params(17, 8, "SBDF3", ra=3e5, restart=True, restart_point=5, add_pert=True, ampT=1e-3)]
    b = fg.Batch(ps)
    assert b.ngroups == 1
    b.restart([str(d1), str(d2)])
    b.step(10)
    for i, d in enumerate((d1, d2)):
        alone = fg.Instance(ps[i])
        alone.restart(str(d))
        alone.step(10)
        sb, sa = b.get_state(i), alone.get_state()
        for f in FIELDS:
            assert np.array_equal(sb[f], sa[f]), (i, f)


def test_step_before_restart_is_refused(fg, tmp_path):
    h = fg.Instance(fg.make_params(17, 8, "SBDF3", restart=True, restart_point=1))
    with pytest.raises(fg.FalconError, match="falcon_restart"):
        h.step(1)
    with pytest.raises(fg.FalconError, match="checkpoint not found"):
        h.restart(str(tmp_path))
