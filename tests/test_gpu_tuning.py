"""The contraction autotuner (falcon_set_gemm_mode(4), the default): the first
time a contraction shape runs outside graph capture every available path
(FP64 FMA tiles of the cost model's shape and of the best 16-, 32- and
64-column shapes, mma.sync slices, tcgen05 slices where the contraction
fills the GPU) is timed on it and the fastest is kept.  Checked here:

- a run that measures gives the same bits as a later run that only reads
  the decisions (the chosen path runs last), in this process and in one
  that reads them back from the cache file;
- every decision is within 10 % of the fastest of its measured times (the
  fixed rule's path is kept unless another is 10 % faster), and narrow per-mode
  contractions (groups of a few instances, N < 16) were measured on the
  sliced paths too;
- the tuned run agrees with the oracle after 100 steps (1e-10).
"""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

FIELDS = ("T", "omg", "up", "ur", "psi")


def run(fg, params, seeds, nsteps):
    b = fg.Batch(params)
    b.init_noise(seeds)
    b.step(nsteps)
    out = [b.get_state(i) for i in range(len(params))]
    b.close()
    return out


def read_cache(path):
    lines = open(path).read().splitlines()
    assert lines[0] == "falcon-contraction-tuning 2"
    rows = []
    for ln in lines[1:]:
        f = ln.split()
        assert len(f) == 15, ln
        rows.append((f[0], [int(x) for x in f[1:9]], [float(x) for x in f[9:]]))
    return rows


@pytest.fixture
def tuned(fg, tmp_path):
    prev = fg.set_gemm_mode(4)
    fg.tune_clear()
    cache = tmp_path / "tune.txt"
    fg.set_tune_cache(cache)
    yield cache
    fg.set_tune_cache(None)
    fg.tune_clear()
    fg.set_gemm_mode(prev)


def test_tuned_runs_are_reproducible_and_pick_the_fastest(fg, tuned):
    # two operator keys (Pr 1 and 10) of 3 instances each, Nr = 33 and 65:
    # per-mode contractions of N = 6 columns, radial ones over all modes
    ps, seeds = [], []
    for R, Nm in ((33, 20), (65, 42)):
        for pr in (1.0, 10.0):
            for k in range(3):
                ps.append(fg.make_params(R, Nm, "SBDF3", ra=1e5 * (1 + k), dt=1e-5, pr=pr))
                seeds.append(900 + len(seeds))
    m0 = fg.tune_entries()[1]
    first = run(fg, ps, seeds, 10)
    n, measured = fg.tune_entries()
    assert n > 0 and measured - m0 == n
    rows = read_cache(tuned)
    assert len(rows) == n
    dev = fg.device_tag()
    narrow = 0
    for d, (r, K, N, batch, w, per_mode, reuse, path), us in rows:
        assert d == dev
        avail = [t for t in us if t >= 0]
        if per_mode >= 2:   # narrow row blocks: one tcgen05 launch (2) or the blocks (0)
            assert path in (0, 2) and us[0] > 0 and us[2] > 0
            assert us[path] <= 1.25 * min(avail), (r, K, N, batch, us, path)
            continue
        assert us[0] > 0 and us[1] > 0                       # FMA and mma.sync always measured
        # the fastest, or the fixed rule's path within 10 % of it
        assert us[path] <= 1.1 * min(avail), (r, K, N, batch, us, path)
        if per_mode and N < 16:
            narrow += 1
    assert narrow > 0
    # decisions read from memory: no new measurement, the same bits
    again = run(fg, ps, seeds, 10)
    assert fg.tune_entries()[1] == measured
    # decisions read from the file (as a new process would)
    fg.tune_clear()
    fg.set_tune_cache(tuned)
    assert fg.tune_entries()[0] == n
    reread = run(fg, ps, seeds, 10)
    assert fg.tune_entries()[1] == measured
    for i in range(len(ps)):
        for k in FIELDS:
            assert np.array_equal(first[i][k], again[i][k]), (i, k)
            assert np.array_equal(first[i][k], reread[i][k]), (i, k)


def test_tuned_batch_matches_oracle(fg, orc, tuned):
    R, Nm, B = 33, 20, 5
    ps = [fg.make_params(R, Nm, "ARS343", ra=1e5, dt=1e-5) for _ in range(B)]
    seeds = list(range(60, 60 + B))
    got = run(fg, ps, seeds, 100)
    for i in (0, B - 1):
        o = orc.Sim(orc.make_params(R, Nm, "ARS343", ra=1e5, dt=1e-5))
        o.init_noise(seeds[i])
        o.step(100)
        want = o.get_state()
        errs = {k: rel(got[i][k], want[k]) for k in ("T", "omg", "up", "ur")}
        assert max(errs.values()) < 1e-10, errs
