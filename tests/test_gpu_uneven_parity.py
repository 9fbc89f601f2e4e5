"""Parity on the uneven batch's own path: a batch drawn like the bench's
uneven batch (schemes CNAB2, SBDF3, ARS343, BPR353; Pr from {0.1, 1, 10};
Ra log-uniform; dt = 0.2 x the t=0 CFL estimate), restricted to the grids
the oracle steps in seconds (Nr 33 and 65, Ntheta 128 and 256), stepped
100 times as groups of one grid, dt and scheme with mixed Pr on the default
autotuned contraction paths, every instance against the oracle (relative
spectral error <= 1e-10; omega of the not stiffly accurate ARS343 within
ten times the oracle's own sensitivity to a 1e-16 perturbation, as on the
Nr = 129 grid)."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, rel

pytestmark = pytest.mark.gpu


def test_uneven_mix_matches_oracle_after_100_steps(fg, orc):
    sys.path.insert(0, ROOT)
    import bench
    rng = np.random.default_rng(21)
    cases = []
    for k in range(32):
        key = k % 16                         # every grid and scheme twice, with two Pr
        nr = (33, 65)[key % 2]
        nm = (128, 256)[(key // 2) % 2] // 3
        scheme = bench.MIXED_SCHEMES[(key // 4) % 4]
        pr = bench.MIXED_PR[(k // 16 + key) % 3]
        ra = float(10 ** rng.uniform(5.0, 7.0))
        cases.append((nr, nm, scheme, ra, pr, bench.cfl_dt(nr, nm), 600 + k))
    b = fg.Batch([fg.make_params(nr, nm, s, ra=ra, dt=dt, pr=pr) for nr, nm, s, ra, pr, dt, _ in cases])
    # 16 keys of grid, dt and scheme, each holding two instances of two Pr
    assert b.ngroups == 16
    b.init_noise([c[-1] for c in cases])
    b.step(100)
    for i, (nr, nm, s, ra, pr, dt, seed) in enumerate(cases):
        o = orc.Sim(orc.make_params(nr, nm, s, ra=ra, dt=dt, pr=pr))
        o.init_noise(seed)
        o.step(100)
        got, want = b.get_state(i), o.get_state()
        tol = {k: 1e-10 for k in ("T", "omg", "up", "ur")}
        if s == "ARS343":
            # not stiffly accurate: the psi Poisson solve with Johnston's
            # wall vorticity amplifies rounding; omega is held to ten times
            # the oracle's own change under a 1e-16 perturbation of T
            q = orc.Sim(orc.make_params(nr, nm, s, ra=ra, dt=dt, pr=pr))
            q.init_noise(seed)
            st = q.get_state()
            pert = np.random.default_rng(1).standard_normal(st["T"].shape)
            q.set_state(st["T"] * (1.0 + 1e-16 * pert), st["omg"], st["up"], st["ur"])
            q.step(100)
            tol["omg"] = max(1e-10, 10.0 * rel(q.get_state()["omg"], want["omg"]))
        errs = {k: rel(got[k], want[k]) for k in tol}
        assert all(errs[k] < tol[k] for k in tol), (i, nr, nm, s, pr, errs, tol)
    b.close()
