"""The bench's full size: 256 instances, Nr=65, Nm=170 (Np=510), SBDF3,
dt=1e-6, run as two groups of 128 with the slice-plane contractions and the
tensor-core radix-17 stages.  Properties that hold at any size: identical
instances step to identical bits (every product is exact per column, so
neither the column, the group nor the launch shape matters), and an
instance agrees with the oracle to the suite's step tolerance."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def test_full_size_identical_instances_and_oracle(fg, orc):
    n, steps = 256, 6
    p = fg.make_params(65, 170, "SBDF3", ra=3e7, dt=1e-6)
    b = fg.Batch([p] * n)
    assert b.ngroups == 2
    b.init_noise([1234] * n, 1e-3)
    b.step(steps)
    s0 = b.get_state(0)
    for i in (1, 127, 128, 200, 255):
        si = b.get_state(i)
        for f in ("T", "omg", "up", "ur", "psi"):
            assert np.array_equal(s0[f], si[f]), (i, f)
    b.close()
    o = orc.Sim(orc.make_params(65, 170, "SBDF3", ra=3e7, dt=1e-6))
    o.init_noise(1234, 1e-3)
    o.step(steps)
    os_ = o.get_state()
    assert max(rel(s0[f], os_[f]) for f in ("T", "omg", "up", "ur")) < 1e-10
