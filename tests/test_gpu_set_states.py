"""falcon_batch_set_states (every instance's state in one call) against n
falcon_batch_set_state calls: the same device state, bit for bit, before and
after stepping, for batches whose groups interleave in instance order."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def smooth(rng, R, M):
    d = np.exp(-0.1 * np.arange(M))[None, :]
    return (rng.standard_normal((R, M)) + 1j * rng.standard_normal((R, M))) * d * 1e-3


def cases(fg):
    # groups interleave: (17, 8) SBDF3 at 0, 2, 3; (33, 20) BPR353 at 1, 4
    a = lambda ra: fg.make_params(17, 8, "SBDF3", ra=ra, dt=1e-4)
    b = lambda ra: fg.make_params(33, 20, "BPR353", ra=ra, dt=1e-5)
    return [a(1e4), b(1e5), a(2e4), a(3e4), b(2e5)]


@pytest.mark.parametrize("all_fields", [True, False])
def test_set_states_equals_set_state(fg, all_fields):
    ps = cases(fg)
    rng = np.random.default_rng(7)
    fields = [[smooth(rng, p.nr_max, p.nm_max + 1) for p in ps] for _ in range(4)]
    if not all_fields:
        fields[1:] = [None, None, None]
    one, bulk = fg.Batch(ps), fg.Batch(ps)
    assert one.ngroups == 2
    for i in range(len(ps)):
        one.set_state(i, *[None if f is None else f[i] for f in fields])
    flat = [None if f is None else np.concatenate([x.ravel() for x in f]) for f in fields]
    bulk.set_states(*flat)
    for step in (0, 12):
        if step:
            one.step(step)
            bulk.step(step)
        for i in range(len(ps)):
            s1, s2 = one.get_state(i), bulk.get_state(i)
            for k in ("T", "omg", "up", "ur", "psi"):
                assert np.array_equal(s1[k], s2[k]), (i, k, step)
            if step == 0:
                assert np.array_equal(s2["T"], fields[0][i])
                if all_fields:
                    assert np.array_equal(s2["ur"], fields[3][i])
    one.close()
    bulk.close()


def test_set_states_after_stepping_restarts_columns(fg):
    # a second load mid-run behaves like n set_state calls: histories cleared,
    # step count and run time kept
    ps = cases(fg)
    rng = np.random.default_rng(8)
    t0 = [smooth(rng, p.nr_max, p.nm_max + 1) for p in ps]
    t1 = [smooth(rng, p.nr_max, p.nm_max + 1) for p in ps]
    one, bulk = fg.Batch(ps), fg.Batch(ps)
    for b in (one, bulk):
        b.set_states(t0)
        b.step(5)
    for i in range(len(ps)):
        one.set_state(i, t1[i])
    bulk.set_states(t1)
    one.step(7)
    bulk.step(7)
    d1, d2 = one.diagnostics(), bulk.diagnostics()
    for i in range(len(ps)):
        s1, s2 = one.get_state(i), bulk.get_state(i)
        for k in ("T", "omg", "up", "ur"):
            assert np.array_equal(s1[k], s2[k]), (i, k)
        assert d1[i]["time"] == d2[i]["time"]
    one.close()
    bulk.close()


def test_set_states_rejects_wrong_size(fg):
    ps = cases(fg)
    b = fg.Batch(ps)
    with pytest.raises(ValueError):
        b.set_states(np.zeros(10, np.complex128))
    with pytest.raises(ValueError):
        b.set_states([np.zeros((p.nr_max, p.nm_max + 1), np.complex128) for p in ps[:-1]])
    b.close()
