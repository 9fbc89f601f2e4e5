"""The serving loop under churn: 36 requests of three grids and schemes,
each with Pr from {0.1, 1, 10}, arriving a few per iteration with horizons
of 3 to 30 steps, so that the groups are repacked (columns remapped, Pr
subs and their operator sets refreshed, graphs dropped and recaptured)
dozens of times while other groups keep stepping on their streams.  Every
request must reach its horizon with the state of the same request run
alone (to FP64 rounding: the contraction paths of the changing group sizes
may differ from the lone run's)."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

KEYS = [(17, 8, "SBDF3", 1e-4), (33, 20, "CNAB2", 1e-5), (17, 10, "ARS343", 1e-5)]
PRS = (0.1, 1.0, 10.0)


def test_churning_stream_matches_lone_runs(fg):
    rng = np.random.default_rng(123)
    reqs = []
    for k in range(36):
        R, Nm, scheme, dt = KEYS[k % 3]
        p = fg.make_params(R, Nm, scheme, ra=float(10 ** rng.uniform(4, 5)), dt=dt, pr=PRS[(k // 3) % 3])
        reqs.append((p, 400 + k, int(rng.integers(3, 31))))
    srv = fg.Server(2 << 30)
    ids, nxt = [], 0
    for it in range(200):
        for _ in range(int(rng.integers(0, 4))):   # 0-3 arrivals per iteration
            if nxt < len(reqs):
                p, seed, hor = reqs[nxt]
                ids.append(srv.submit(p, seed, hor))
                nxt += 1
        srv.iterate()
        if nxt == len(reqs) and all(srv.result(i)[0] for i in ids):
            break
    assert nxt == len(reqs)
    res = [srv.result(i) for i in ids]
    steps = [srv.steps(i) for i in ids]
    srv.close()
    for (p, seed, hor), (done, status, diag, fields), n in zip(reqs, res, steps):
        assert done and status == 0 and n == hor
        alone = fg.Instance(p)
        alone.init_noise(seed)
        alone.step(hor)
        st = alone.get_state()
        alone.close()
        for k in ("T", "omg", "up", "ur"):
            assert rel(fields[k], st[k]) < 1e-11, (seed, k, rel(fields[k], st[k]))
