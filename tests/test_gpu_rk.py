"""Explicit RK2 / RK4 (timeloop_rk, src/steptime_rk.F90) on the GPU against the oracle.

The reference runs RK with the LAPpsi Poisson solve and Johnston's wall
vorticity (src/fourierloop_rk.F90); the GPU applies the same operators as
GEMMs.  Tolerance: 1e-10 relative spectral error after 100 steps.
"""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-10
FIELDS = ("T", "omg", "up", "ur", "psi")


def run_pair(orc, fg, scheme, R, Nm, ra, dt, nsteps, mbc="NS", pr=1.0, seed=1, state=None):
    g = fg.Instance(fg.make_params(R, Nm, scheme, ra=ra, dt=dt, mbc=mbc, pr=pr))
    o = orc.Sim(orc.make_params(R, Nm, scheme, ra=ra, dt=dt, mbc=mbc, pr=pr))
    if state is None:
        g.init_noise(seed)
        o.init_noise(seed)
    else:
        g.set_state(*state)
        o.set_state(*state)
    g.step(nsteps)
    o.step(nsteps)
    gs, os_ = g.get_state(), o.get_state()
    return {k: rel(gs[k], os_[k]) for k in FIELDS}, g, o


@pytest.mark.parametrize("scheme,R,Nm,ra,dt,mbc", [
    ("RK2", 17, 10, 1e4, 1e-6, "NS"),
    ("RK4", 33, 42, 1e5, 2e-7, "NS"),
    ("RK4", 17, 10, 1e4, 1e-6, "SF"),
    ("RK2", 33, 42, 1e5, 2e-7, "SF"),
])
def test_rk_parity_after_100_steps(orc, fg, scheme, R, Nm, ra, dt, mbc):
    errs, _, _ = run_pair(orc, fg, scheme, R, Nm, ra, dt, 100, mbc=mbc)
    assert max(errs.values()) < STEP_TOL, errs


def test_rk_first_stage_reads_initial_upfc(orc, fg):
    # a state with velocity: the first stage of the run takes upFC = upFR
    # (src/init.F90:252), later stages the Chebyshev transform of u_phi
    R, Nm = 17, 10
    rng = np.random.default_rng(9)
    M = Nm + 1
    d = np.exp(-0.3 * np.arange(M))[None, :]
    T = np.zeros((R, M), complex)
    T[:, 0] = np.linspace(1.0, 0.0, R)
    T[1:-1, 1:] = 1e-3 * (rng.standard_normal((R - 2, M - 1)) + 1j * rng.standard_normal((R - 2, M - 1)))
    up = 1e-2 * (rng.standard_normal((R, M)) + 1j * rng.standard_normal((R, M))) * d
    up[:, 0] = up[:, 0].real
    up[[0, -1], :] = 0.0
    om = np.zeros((R, M), complex)
    ur = np.zeros((R, M), complex)
    errs, _, _ = run_pair(orc, fg, "RK4", R, Nm, 1e4, 1e-6, 20, state=(T, om, up, ur))
    assert max(errs.values()) < STEP_TOL, errs


def test_rk_diagnostics_match_oracle(orc, fg):
    _, g, o = run_pair(orc, fg, "RK4", 17, 10, 1e4, 1e-6, 30)
    dg, do = g.diagnostics(), o.diagnostics()
    for kg, ko in (("ke", "KE"), ("nu_top", "Nu_top"), ("nu_bot", "Nu_bot"), ("vis", "vis"), ("buo", "buo")):
        assert abs(dg[kg] - do[ko]) <= 1e-9 * max(abs(do[ko]), 1e-300), (kg, dg[kg], do[ko])


def test_rk_in_mixed_batch_bitwise_alone(fg, fixed_paths):
    ps = [fg.make_params(17, 10, "RK4", ra=1e4, dt=1e-6), fg.make_params(17, 8, "SBDF3", ra=1e4, dt=1e-4),
          fg.make_params(17, 10, "RK4", ra=3e4, dt=1e-6)]
    b = fg.Batch(ps)
    assert b.ngroups == 2
    b.init_noise([5, 6, 7])
    b.step(15)
    alone = fg.Instance(ps[2])
    alone.init_noise(7)
    alone.step(15)
    sb, sa = b.get_state(2), alone.get_state()
    for f in FIELDS:
        assert np.array_equal(sb[f], sa[f]), f
