"""The operator contractions on the tensor cores by exact integer slicing of
the FP64 operands (the default) against the FP64 FMA tiles (set_gemm_mode(0))
and against the oracle, on batches large enough that both the radial and the
per-mode contractions take the sliced path.  The slices are exact below
2^(e-60) of each row / column maximum and every FP32 sum of slice products
is exact, so the two paths differ by FP64 rounding only; the oracle
tolerance is the suite's 1e-10 after the steps."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

FIELDS = ("T", "omg", "up", "ur", "psi")


def run(fg, params, seeds, nsteps, mode):
    prev = fg.set_gemm_mode(mode)
    try:
        b = fg.Batch(params)
        b.init_noise(seeds)
        b.step(nsteps)
        out = [b.get_state(i) for i in range(len(params))]
        b.close()
    finally:
        fg.set_gemm_mode(prev)
    return out


# Batches up to a few dozen instances take the kernel that slices its own X
# columns (N x batch <= 16384 columns); the 200-instance case (two groups of
# 100, N x batch = 200 x 86 per-mode columns) takes the slice planes of
# oz_slice_cols_kernel, as the bench's 256-instance batch does.
@pytest.mark.parametrize("scheme,R,Nm,B,dt", [("SBDF3", 65, 42, 12, 1e-5), ("ARS443", 33, 20, 10, 1e-5),
                                              ("CNAB2", 97, 42, 6, 1e-5), ("RK4", 33, 20, 8, 1e-6),
                                              ("BPR353", 33, 20, 9, 1e-5), ("SBDF3", 65, 85, 200, 1e-5)])
def test_sliced_contractions_match_fma_tiles(fg, scheme, R, Nm, B, dt):
    ras = np.geomspace(1e4, 1e6, B)
    ps = [fg.make_params(R, Nm, scheme, ra=float(ra), dt=dt) for ra in ras]
    seeds = list(range(100, 100 + B))
    a = run(fg, ps, seeds, 20, 1)
    f = run(fg, ps, seeds, 20, 0)
    for i in (range(B) if B <= 12 else (0, 1, B // 2, B - 1)):
        for k in FIELDS:
            assert rel(a[i][k], f[i][k]) < 1e-12, (i, k, rel(a[i][k], f[i][k]))


@pytest.mark.parametrize("scheme,R,Nm,B", [("SBDF3", 33, 20, 12), ("ARS343", 33, 20, 10)])
def test_sliced_batch_matches_oracle(orc, fg, scheme, R, Nm, B):
    ps = [fg.make_params(R, Nm, scheme, ra=1e5, dt=1e-5) for _ in range(B)]
    seeds = list(range(7, 7 + B))
    a = run(fg, ps, seeds, 100, 1)
    for i in (0, B - 1):
        o = orc.Sim(orc.make_params(R, Nm, scheme, ra=1e5, dt=1e-5))
        o.init_noise(seeds[i])
        o.step(100)
        os_ = o.get_state()
        errs = {k: rel(a[i][k], os_[k]) for k in FIELDS}
        assert max(errs.values()) < 1e-10, errs
