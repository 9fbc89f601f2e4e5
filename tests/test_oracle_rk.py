"""The oracle's explicit RK (src/steptime_rk.F90, src/fourierloop_rk.F90,
src/rhs_create_rk.F90) checked for consistency: no reference test or golden
vector covers RK, so the restatement is pinned by its convergence in dt
(RK4 fourth order, RK2 second order) and by its boundary values."""
import numpy as np


def run(orc, scheme, dt, n, R=17, Nm=10, seed=2, mbc="NS"):
    o = orc.Sim(orc.make_params(R, Nm, scheme, ra=1e4, dt=dt, mbc=mbc))
    o.init_noise(seed)
    o.step(n)
    return o.get_state()


def test_rk4_converges_in_dt(orc):
    a = run(orc, "RK4", 1e-7, 100)
    b = run(orc, "RK4", 5e-8, 200)
    for k in ("T", "omg", "up", "ur"):
        assert np.linalg.norm(a[k] - b[k]) / np.linalg.norm(b[k]) < 1e-12, k


def test_rk2_agrees_with_rk4_to_second_order(orc):
    ref = run(orc, "RK4", 5e-8, 200)
    e = []
    for dt, n in ((1e-7, 100), (5e-8, 200)):
        s = run(orc, "RK2", dt, n)
        e.append(np.linalg.norm(s["omg"] - ref["omg"]) / np.linalg.norm(ref["omg"]))
    assert e[1] < e[0] and 2.5 < e[0] / e[1] < 6.0, e  # halving dt divides the error by ~4


def test_rk_boundary_values(orc):
    for mbc in ("NS", "SF"):
        s = run(orc, "RK4", 1e-6, 20, mbc=mbc)
        assert abs(s["T"][0, 0] - 1.0) == 0.0 and np.all(s["T"][-1] == 0) and np.all(s["T"][0, 1:] == 0)
        assert np.all(s["psi"][[0, -1], 1:] == 0) or np.abs(s["psi"][[0, -1], 1:]).max() < 1e-14
        assert np.all(s["up"][[0, -1], 0] == 0)
