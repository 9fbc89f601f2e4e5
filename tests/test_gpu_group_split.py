"""Instances of one operator key split into several groups (each on its own
stream, operators shared) step to the same bits as one group: every
contraction is exact per column and the groups are independent."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run(fg, ps, seeds, gmax, nsteps):
    prev = fg.set_max_group_size(gmax)
    try:
        b = fg.Batch(ps)
    finally:
        fg.set_max_group_size(prev)
    b.init_noise(seeds)
    b.step(nsteps)
    out = [b.get_state(i) for i in range(len(ps))], b.ngroups, b.diagnostics_array()
    b.close()
    return out


def test_split_groups_step_to_the_same_bits(fg, fixed_paths):
    R, Nm, n = 65, 42, 20
    ps = [fg.make_params(R, Nm, "SBDF3", ra=1e5 * (1 + 0.1 * k), dt=1e-5) for k in range(n)]
    seeds = list(range(300, 300 + n))
    one, g1, d1 = run(fg, ps, seeds, 0, 12)
    two, g2, d2 = run(fg, ps, seeds, 10, 12)
    assert (g1, g2) == (1, 2)
    for i in range(n):
        for f in ("T", "omg", "up", "ur", "psi"):
            assert np.array_equal(one[i][f], two[i][f]), (i, f)
    assert np.array_equal(d1, d2)
