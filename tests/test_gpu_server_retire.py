"""The serving loop retires a request whose state goes bad, on its own and
with a status, while the other requests of its operator group keep
stepping: a non-finite state (a NaN planted in the caller's initial state)
retires with FALCON_ENONFINITE and a kinetic energy above 1e10 with
FALCON_EBLOWUP (the reference's stop, src/output.F90:321-323), both at
the first check of their n_KE cadence; the healthy request of the same
group reaches its horizon with the same result as when it is served alone,
and the server returns all its fields."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

FALCON_ENONFINITE, FALCON_EBLOWUP = -5, -6


def serve(fg, requests, budget=4 << 30):
    srv = fg.Server(budget)
    ids = []
    for kind, p, arg, horizon in requests:
        ids.append(srv.submit(p, arg, horizon) if kind == "seed" else srv.submit_state(p, *arg, horizon=horizon))
    for _ in range(200):
        srv.iterate()
        if all(srv.result(i)[0] for i in ids):
            break
    out = [srv.result(i) + (srv.steps(i),) for i in ids]
    srv.close()
    return out


def test_bad_requests_retire_alone(fg):
    R, Nm = 17, 8
    p = fg.make_params(R, Nm, "SBDF3", ra=1e5, dt=1e-4)
    p.n_KE = 5
    # initial states: the seeded one as the host builds it, one with a NaN,
    # one with a large u_phi (KE ~ 3e10 at the first check)
    g = fg.Instance(p)
    g.init_noise(3)
    s0 = g.get_state()
    g.close()
    t_nan = s0["T"].copy()
    t_nan[4, 2] = np.nan
    big_up = np.zeros_like(s0["T"])
    big_up[:, 0] = 1e5
    reqs = [("seed", p, 3, 30), ("state", p, (t_nan,), 30), ("state", p, (s0["T"], None, big_up, None), 30)]
    (ok, st_ok, d_ok, f_ok, n_ok), (done1, st1, _, _, n1), (done2, st2, _, _, n2) = serve(fg, reqs)
    assert ok and st_ok == 0 and n_ok == 30
    assert done1 and st1 == FALCON_ENONFINITE and n1 == 5
    assert done2 and st2 == FALCON_EBLOWUP and n2 == 5
    assert all(np.isfinite(f_ok[k]).all() for k in ("T", "omg", "up", "ur"))
    # the healthy request alone gives the same result
    (a_ok, a_st, a_d, a_f, _), = serve(fg, [("seed", p, 3, 30)])
    for k in ("T", "omg", "up", "ur"):
        assert rel(f_ok[k], a_f[k]) < 1e-12, k
    assert abs(d_ok["ke"] - a_d["ke"]) <= 1e-12 * a_d["ke"]
