"""Variable time step (l_vartimestep, compute_new_dt of src/steptime.F90:313-370)
on the GPU against the oracle: the CFL time step from the velocity maxima of
each nonlinear pass (get_dtvals, src/nonlin.F90:93-106), the variable-dt
multistep weights, and the operators rebuilt whenever dt changes."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-10
FIELDS = ("T", "omg", "up", "ur", "psi")


@pytest.mark.parametrize("scheme,optimize", [("CNAB2", False), ("SBDF3", False), ("SBDF3", True),
                                             ("SBDF2", True), ("CNAB3", False), ("SBDF4", True)])
def test_variable_dt_matches_oracle(orc, fg, scheme, optimize):
    kw = dict(ra=1e5, dt=1e-5, cfl=0.5, dt_coef=2.0, dt_max=1e-4)
    g = fg.Instance(fg.make_params(17, 10, scheme, vartimestep=True, optimizedt=optimize, **kw))
    o = orc.Sim(orc.make_params(17, 10, scheme, vartimestep=True, optimizedt=optimize, **kw))
    g.init_noise(1, 1e-1)
    o.init_noise(1, 1e-1)
    dts = []
    for k in range(40):
        g.step(1)
        o.step(1)
        dg = g.diagnostics()
        assert abs(dg["dt"] - o.dt) <= 1e-12 * o.dt, (k, dg["dt"], o.dt)
        dts.append(o.dt)
    assert len(set(dts)) > 1  # dt did change
    gs, os_ = g.get_state(), o.get_state()
    errs = {f: rel(gs[f], os_[f]) for f in FIELDS}
    assert max(errs.values()) < STEP_TOL, errs
    assert abs(g.diagnostics()["time"] - o.diagnostics()["time"]) <= 1e-12 * o.diagnostics()["time"]


def test_variable_dt_instances_keep_their_own_step_in_a_batch(orc, fg):
    kw = dict(dt=1e-5, cfl=0.5, dt_coef=2.0, dt_max=1e-4, vartimestep=True)
    ps = [fg.make_params(17, 10, "SBDF3", ra=1e5, **kw), fg.make_params(17, 10, "SBDF3", ra=3e5, **kw),
          fg.make_params(17, 10, "SBDF3", ra=1e5, dt=1e-5)]
    b = fg.Batch(ps)
    assert b.ngroups == 3  # variable-dt instances are never grouped
    b.init_noise([1, 2, 3], 1e-1)
    b.step(25)
    d = b.diagnostics()
    assert d[2]["dt"] == 1e-5
    for i, ra in ((0, 1e5), (1, 3e5)):
        o = orc.Sim(orc.make_params(17, 10, "SBDF3", ra=ra, dt=1e-5, cfl=0.5, dt_coef=2.0, dt_max=1e-4,
                                    vartimestep=True))
        o.init_noise(i + 1, 1e-1)
        o.step(25)
        assert abs(d[i]["dt"] - o.dt) <= 1e-12 * o.dt
        gs, os_ = b.get_state(i), o.get_state()
        assert max(rel(gs[f], os_[f]) for f in FIELDS) < STEP_TOL


@pytest.mark.parametrize("scheme,optimize", [("ARS443", False), ("ARS343", False), ("BHR553", False),
                                             ("BPR353", True), ("PC2", False), ("SMR333", False),
                                             ("CB3f", False), ("LZ4A1", True), ("KC885", False)])
def test_variable_dt_imexrk_matches_oracle(orc, fg, scheme, optimize):
    # IMEXRK compute_new_dt (src/steptime_imexrk.F90:248-308), operators
    # rebuilt whenever dt changes
    kw = dict(ra=1e6, dt=1e-5, cfl=0.02, dt_coef=1.5, dt_max=1e-4)
    g = fg.Instance(fg.make_params(17, 10, scheme, vartimestep=True, optimizedt=optimize, **kw))
    o = orc.Sim(orc.make_params(17, 10, scheme, vartimestep=True, optimizedt=optimize, **kw))
    g.init_noise(1, 1e-1)
    o.init_noise(1, 1e-1)
    for k in range(25):
        g.step(1)
        o.step(1)
        dg = g.diagnostics()
        assert abs(dg["dt"] - o.dt) <= 1e-12 * o.dt, (k, dg["dt"], o.dt)
    gs, os_ = g.get_state(), o.get_state()
    errs = {f: rel(gs[f], os_[f]) for f in FIELDS}
    assert max(errs.values()) < STEP_TOL, errs


@pytest.mark.parametrize("scheme", ["RK2", "RK4"])
def test_variable_dt_rk_matches_oracle(orc, fg, scheme):
    # RK compute_new_dt (src/steptime_rk.F90:180-238): diffusive scales included
    kw = dict(ra=1e5, dt=1e-6, cfl=0.5, dt_coef=2.0, dt_max=1e-4)
    g = fg.Instance(fg.make_params(17, 10, scheme, vartimestep=True, **kw))
    o = orc.Sim(orc.make_params(17, 10, scheme, vartimestep=True, **kw))
    g.init_noise(1, 1e-1)
    o.init_noise(1, 1e-1)
    for k in range(25):
        g.step(1)
        o.step(1)
        assert abs(g.diagnostics()["dt"] - o.dt) <= 1e-12 * o.dt
    gs, os_ = g.get_state(), o.get_state()
    errs = {f: rel(gs[f], os_[f]) for f in FIELDS}
    assert max(errs.values()) < STEP_TOL, errs
