"""Instances that differ only in Pr (and Ra) step as one group: Pr enters only
the temperature operator AT (src/mat_assembly.F90), so each run of equal Pr
has its own temperature solve while the nonlinear pass, the radial
contractions, the omega-psi solves and every elementwise kernel cover all
instances at once, with 1/Pr taken per instance in the right-hand sides
(CN explicit diffusion, IMEXRK stage derivatives, RK right-hand sides).
Every instance must agree with the oracle, and (under the fixed contraction
rules) step to the same bits as alone; its snapshot carries its own Pr."""
import numpy as np
import pytest

from conftest import rel
from test_checkpoint_format import parse_snapshot

pytestmark = pytest.mark.gpu

FIELDS = ("T", "omg", "up", "ur")
# scheme, R, Nm, dt, Pr of the instances (interleaved on purpose)
CASES = [("SBDF3", 33, 20, 1e-5, (10.0, 0.1, 1.0, 10.0, 0.1)),
         ("CNAB2", 17, 8, 1e-4, (0.7, 10.0, 0.7)),
         ("ARS343", 17, 10, 1e-5, (0.1, 10.0)),
         ("SMR333", 17, 10, 1e-5, (1.0, 10.0)),   # stage-dependent implicit diagonal: stage operators per Pr
         ("RK4", 17, 10, 1e-6, (0.1, 10.0))]


def params(fg, with_schemes=False):
    ps, seeds, schemes = [], [], []
    for scheme, R, Nm, dt, prs in CASES:
        for j, pr in enumerate(prs):
            ps.append(fg.make_params(R, Nm, scheme, ra=1e4 * (1 + j), dt=dt, pr=pr))
            seeds.append(70 + len(seeds))
            schemes.append(scheme)
    return (ps, seeds, schemes) if with_schemes else (ps, seeds)


def test_pr_mix_is_one_group_per_grid_and_scheme_and_matches_oracle(fg, orc):
    ps, seeds, schemes = params(fg, True)
    b = fg.Batch(ps)
    assert b.ngroups == len(CASES)
    b.init_noise(seeds)
    b.step(30)
    for i, p in enumerate(ps):
        o = orc.Sim(orc.make_params(p.nr_max, p.nm_max, schemes[i], ra=p.ra, dt=p.dt, pr=p.pr))
        o.init_noise(seeds[i])
        o.step(30)
        got, want = b.get_state(i), o.get_state()
        errs = {k: rel(got[k], want[k]) for k in FIELDS}
        assert max(errs.values()) < 1e-10, (i, p.pr, errs)
    b.close()


def test_pr_mix_instances_identical_alone(fg, fixed_paths):
    ps, seeds = params(fg)
    b = fg.Batch(ps)
    b.init_noise(seeds)
    b.step(12)
    for i in (0, 1, 2, 5, 6, 8, 9, 11, 13):
        alone = fg.Instance(ps[i])
        alone.init_noise(seeds[i])
        alone.step(12)
        sa, sb = alone.get_state(), b.get_state(i)
        alone.close()
        for k in FIELDS + ("psi",):
            assert np.array_equal(sa[k], sb[k]), (i, k)
    b.close()


def test_snapshot_of_a_mixed_group_carries_the_instance_pr(fg, tmp_path):
    ps, seeds = params(fg)
    b = fg.Batch(ps[:5])
    b.init_noise(seeds[:5])
    b.step(3)
    for i in range(5):
        path = str(tmp_path / f"snap{i}")
        b.store_snapshot(i, path)
        s = parse_snapshot(path, 33, 21)
        assert s["pr"] == ps[i].pr and s["ra"] == ps[i].ra, i
    b.close()


def test_served_pr_mix_shares_a_group_and_matches_alone(fg, fixed_paths):
    # requests of one grid, dt and scheme with Pr 10, 0.1 and 1 arriving at
    # different iterations and with different horizons: they step in one
    # server group (sorted by Pr, one temperature solve per Pr), columns
    # leave and join as requests finish and arrive, and each result equals
    # the request served alone
    p = [fg.make_params(17, 8, "SBDF3", ra=ra, dt=1e-4, pr=pr) for ra, pr in ((2e4, 10.0), (1e4, 0.1), (3e4, 1.0),
                                                                           (1.5e4, 0.1), (2.5e4, 10.0))]
    horizons = (9, 14, 6, 11, 8)
    seeds = (31, 32, 33, 34, 35)
    srv = fg.Server(1 << 30)
    ids = [srv.submit(p[i], seeds[i], horizons[i]) for i in range(3)]
    srv.iterate()
    srv.iterate()
    ids += [srv.submit(p[i], seeds[i], horizons[i]) for i in (3, 4)]   # arrive while the others run
    for _ in range(40):
        srv.iterate()
        if all(srv.result(i)[0] for i in ids):
            break
    res = [srv.result(i) for i in ids]
    srv.close()
    for i, (done, status, diag, fields) in enumerate(res):
        assert done and status == 0, i
        alone = fg.Instance(p[i])
        alone.init_noise(seeds[i])
        alone.step(horizons[i])
        st = alone.get_state()
        alone.close()
        for k in FIELDS:
            assert np.array_equal(fields[k], st[k]), (i, k)
